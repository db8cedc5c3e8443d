"""Shapes of the drop-in API: Circle, Polygon, Edge, Loop.

Construction arithmetic (edge normals, mass data, AABBs) repeats the
reference's float64 operation order -- pypybox2d/shapes.py Circle
(:128-236), Polygon (:238-616), Edge (:618-778), Loop (:780-882) and the
C-extension vector operations of pypybox2d/src/vec2module.c -- so a world
built here is bit-identical to the same world built with pypybox2d.  A loop
fixture becomes one edge record per child (``child_edge``), flagged
``FIX_LOOP_CHILD`` for the loop's fat-box rule.
"""
from __future__ import annotations

import math

from . import abi

EPSILON = 2.220446049250313e-16
EPSILON_SQR = EPSILON * EPSILON
FLT_EPSILON = 1.1920928955078125e-07
POLYGON_RADIUS = 2.0 * 0.005


def _normalized(x: float, y: float) -> tuple[float, float]:
    """vec2module.c Vec2_normalized."""
    length = math.sqrt(x * x + y * y)
    if length < FLT_EPSILON:
        return x, y
    inv = 1.0 / length
    return x * inv, y * inv


def _xmul(p, q, v):
    """transform.c Transform_mul: position + col1*x + col2*y, left to right."""
    c, s = q
    return (p[0] + c * v[0] + (-s) * v[1], p[1] + s * v[0] + c * v[1])


class MassData:
    def __init__(self, mass=0.0, center=(0.0, 0.0), I=0.0):
        self.mass, self.center, self.I = mass, tuple(center), I

    def __repr__(self):
        return f"MassData(mass={self.mass:g}, center={self.center}, I={self.I:g})"


class Shape:
    type = -1
    radius = 0.0

    def compute_mass(self, density):
        raise NotImplementedError

    def compute_aabb(self, p, q):
        raise NotImplementedError

    @property
    def child_count(self):
        return 1


class Circle(Shape):
    type = abi.SHAPE_CIRCLE

    def __init__(self, radius=0.2, position=(0, 0)):
        self.radius = float(radius)
        self.position = (float(position[0]), float(position[1]))

    def __copy__(self):
        return Circle(self.radius, self.position)

    def __repr__(self):
        return f"Circle(radius={self.radius:g}, position={self.position})"

    def compute_mass(self, density):
        """shapes.py:190-200"""
        r2 = self.radius ** 2
        mass = density * math.pi * r2
        px, py = self.position
        I = mass * (0.5 * self.radius ** 2 + (px * px + py * py))
        return MassData(mass, self.position, I)

    def compute_aabb(self, p, q):
        """shapes.py:178-189: p + R * position"""
        c, s = q
        x, y = self.position
        rx, ry = c * x + (-s) * y, s * x + c * y
        cx, cy = p[0] + rx, p[1] + ry
        r = self.radius
        return (cx - r, cy - r, cx + r, cy + r)


class Polygon(Shape):
    type = abi.SHAPE_POLYGON

    def __init__(self, vertices=None, box=None):
        self.radius = POLYGON_RADIUS
        self._vertices: list[tuple[float, float]] = []
        self._normals: list[tuple[float, float]] = []
        if box:
            self._set_box(*box)
        elif vertices is not None:
            self.vertices = vertices

    def __copy__(self):
        return Polygon(self._vertices)

    def __repr__(self):
        return f"Polygon({self._vertices})"

    def _set_box(self, hx, hy, center=(0, 0), angle=0.0):
        """shapes.py:484-501; the fixture's copy recomputes the normals."""
        hx, hy = float(hx), float(hy)
        verts = [(-hx, -hy), (hx, -hy), (hx, hy), (-hx, hy)]
        if center is not None:
            q = (math.cos(angle), math.sin(angle))
            verts = [_xmul((float(center[0]), float(center[1])), q, v) for v in verts]
        self.vertices = verts

    @property
    def vertices(self):
        return list(self._vertices)

    @vertices.setter
    def vertices(self, vertices):
        """shapes.py:442-482: edge normals and the convexity check."""
        vs = [(float(v[0]), float(v[1])) for v in vertices]
        n = len(vs)
        if n < 3:
            raise ValueError("Polygons are >= 3 vertices")
        if n > abi.MAX_POLY_VERTS:
            raise ValueError(f"Polygons are <= {abi.MAX_POLY_VERTS} vertices on the GPU")
        normals = []
        for i in range(n):
            ex, ey = vs[(i + 1) % n][0] - vs[i][0], vs[(i + 1) % n][1] - vs[i][1]
            if ex * ex + ey * ey <= EPSILON_SQR:
                raise ValueError("Edges are too short")
            normals.append(_normalized(1.0 * ey, -1.0 * ex))
        for i1 in range(n):
            i2 = (i1 + 1) % n
            ex, ey = vs[i2][0] - vs[i1][0], vs[i2][1] - vs[i1][1]
            for j in range(n):
                if j in (i1, i2):
                    continue
                rx, ry = vs[j][0] - vs[i1][0], vs[j][1] - vs[i1][1]
                if ex * ry - ey * rx <= 0.0:
                    raise ValueError("ERROR: Please ensure your polygon is convex and has a CCW winding order")
        self._normals = normals
        self._vertices = vs

    @property
    def normals(self):
        return list(self._normals)

    def compute_mass(self, density):
        """shapes.py:336-419"""
        vs = self._vertices
        n = len(vs)
        sx, sy = vs[0]
        for v in vs[1:]:
            sx, sy = sx + v[0], sy + v[1]
        sx, sy = sx / float(n), sy / float(n)
        cx = cy = 0.0
        area = 0.0
        I = 0.0
        inv3 = 1.0 / 3.0
        for i in range(n):
            e1x, e1y = vs[i][0] - sx, vs[i][1] - sy
            e2x, e2y = vs[(i + 1) % n][0] - sx, vs[(i + 1) % n][1] - sy
            D = e1x * e2y - e1y * e2x
            tri = 0.5 * D
            area += tri
            k = tri * inv3
            cx, cy = cx + k * (e1x + e2x), cy + k * (e1y + e2y)
            intx2 = e1x * e1x + e2x * e1x + e2x * e2x
            inty2 = e1y * e1y + e2y * e1y + e2y * e2y
            I += (0.25 * inv3 * D) * (intx2 + inty2)
        mass = density * area
        cx, cy = cx / area, cy / area
        mcx, mcy = cx + sx, cy + sy
        Im = density * I
        Im += mass * ((mcx * mcx + mcy * mcy) - (cx * cx + cy * cy))
        return MassData(mass, (mcx, mcy), Im)

    def compute_aabb(self, p, q):
        """shapes.py:316-334"""
        lx, ly = _xmul(p, q, self._vertices[0])
        ux, uy = lx, ly
        for v in self._vertices:
            x, y = _xmul(p, q, v)
            lx, ly = (lx if lx < x else x), (ly if ly < y else y)
            ux, uy = (ux if ux > x else x), (uy if uy > y else y)
        r = self.radius
        return (lx - r, ly - r, ux + r, uy + r)


class Edge(Shape):
    type = abi.SHAPE_EDGE

    def __init__(self, v1=None, v2=None, v0=None, v3=None):
        self.radius = POLYGON_RADIUS
        self.vertex1 = (float(v1[0]), float(v1[1]))
        self.vertex2 = (float(v2[0]), float(v2[1]))
        # shapes.py:633-641: a zero vector counts as absent (Vec2 truthiness)
        self.vertex0 = (float(v0[0]), float(v0[1])) if v0 is not None and (v0[0] != 0 or v0[1] != 0) else None
        self.vertex3 = (float(v3[0]), float(v3[1])) if v3 is not None and (v3[0] != 0 or v3[1] != 0) else None

    def __copy__(self):
        return Edge(self.vertex1, self.vertex2, self.vertex0, self.vertex3)

    def __repr__(self):
        return f"Edge(vertex1={self.vertex1}, vertex2={self.vertex2}, vertex0={self.vertex0}, vertex3={self.vertex3})"

    def compute_mass(self, density):
        return MassData(0.0, (0.5 * (self.vertex1[0] + self.vertex2[0]), 0.5 * (self.vertex1[1] + self.vertex2[1])), 0.0)

    def compute_aabb(self, p, q):
        """shapes.py:702-718"""
        x1, y1 = _xmul(p, q, self.vertex1)
        x2, y2 = _xmul(p, q, self.vertex2)
        r = self.radius
        return ((x1 if x1 < x2 else x2) - r, (y1 if y1 < y2 else y2) - r,
                (x1 if x1 > x2 else x2) + r, (y1 if y1 > y2 else y2) + r)


class Loop(Shape):
    """shapes.py:780-882: a closed chain of edges with double-sided
    collision; child i runs from vertex i to vertex i + 1 (mod n)."""

    type = abi.SHAPE_LOOP

    def __init__(self, vertices, *args):
        if len(vertices) == 2 and isinstance(vertices[0], (int, float)):
            vertices = [vertices, *args]
        if len(vertices) < 2:
            raise ValueError("Must be >= 2 vertices")
        self.radius = POLYGON_RADIUS
        self._vertices = [(float(v[0]), float(v[1])) for v in vertices]

    def __copy__(self):
        return Loop(self._vertices)

    def __repr__(self):
        return f"Loop(vertices={self._vertices})"

    @property
    def vertices(self):
        return list(self._vertices)

    @property
    def child_count(self):
        return len(self._vertices)

    def child_edge(self, index):
        """shapes.py:851-863: the edge of child `index` with its neighbours as
        vertex0 / vertex3"""
        n = len(self._vertices)
        i0, i1, i2 = (index - 1) % n, index, (index + 1) % n
        i3 = index + 2
        while i3 >= n:
            i3 -= n
        v = self._vertices
        return Edge(v[i1], v[i2], v[i0], v[i3])

    def compute_mass(self, density):
        """Loops have no mass (shapes.py:845-847)."""
        return MassData()

    def compute_aabb(self, p, q, child=0):
        """shapes.py:822-837: the child's two vertices, no radius margin"""
        n = len(self._vertices)
        x1, y1 = _xmul(p, q, self._vertices[child])
        x2, y2 = _xmul(p, q, self._vertices[(child + 1) % n])
        return min(x1, x2), min(y1, y2), max(x1, x2), max(y1, y2)
