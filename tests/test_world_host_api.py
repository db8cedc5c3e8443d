"""Host-side parts of the World API that need no step: the Body frame
helpers (body.py:662-708) and the World flags (world.py:139-181, 447-468),
pinned against the reference's own results for the same API calls
(tests/golden/api_frames.py, recorded by tests/golden/make_golden_queries.py).
Bit-exact: the helpers are single Transform / Mat22 products in the
reference's operation order."""
import os
import sys

import numpy as np
import pytest

import pypybox2d_gb300 as b2

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, GOLDEN)
import api_frames  # noqa: E402


def test_body_frame_helpers_match_reference():
    d = np.load(os.path.join(GOLDEN, "queries.npz"))
    rows, flags = api_frames.rows(b2)
    want = d["frames"]
    got = np.array(rows, dtype=np.float64)
    assert got.shape == want.shape
    bad = got != want
    assert not bad.any(), f"frame helper differs at {np.argwhere(bad)[0]}: {got[bad][0]!r} vs {want[bad][0]!r}"
    assert [int(f) for f in flags] == list(d["frame_world_flags"])


def test_world_flags_round_trip():
    w = api_frames.build(b2)
    for name in ("warm_starting", "continuous_physics", "allow_sleep", "auto_clear_forces"):
        assert getattr(w, name) is True
        setattr(w, name, False)
        assert getattr(w, name) is False
        setattr(w, name, True)
    assert w.sub_stepping is False
    with pytest.raises(NotImplementedError):
        w.sub_stepping = True
    body = w.bodies[1]
    assert body.allow_sleep == body.sleeping_allowed


def test_default_contact_filter():
    F = b2.Fixture
    cases = [
        (F(group_index=2), F(group_index=2), True),        # same positive group: always
        (F(group_index=-3), F(group_index=-3), False),     # same negative group: never
        (F(group_index=-3, category_bits=1, mask_bits=1), F(group_index=4, category_bits=1, mask_bits=1), True),
        (F(category_bits=0x2, mask_bits=0x1), F(category_bits=0x1, mask_bits=0x2), True),
        (F(category_bits=0x2, mask_bits=0x4), F(category_bits=0x1, mask_bits=0x2), False),
        (F(category_bits=0x2, mask_bits=0x1), F(category_bits=0x1, mask_bits=0x4), False),
    ]
    for a, b, want in cases:
        assert b2.World.default_contact_filter(a, b) is want
    w = b2.World()
    assert w.contact_filter is b2.World.default_contact_filter   # world.py:88-89
    w.contact_filter = None                                      # no filtering (contact_manager.py:145)
    assert w.contact_filter is None


def test_create_fixtures_and_destroy_fixture_match_reference():
    """create_fixtures, then destroy_fixture twice on a dynamic body: fixture
    count, mass data, centre of mass and the velocity shift of
    reset_mass_data (body.py:587-641) after each call, bit for bit."""
    d = np.load(os.path.join(GOLDEN, "queries.npz"))
    rows, world = api_frames.destroy_rows(b2)
    got = np.array(rows, dtype=np.float64)
    want = d["destroy_fixture"]
    assert got.shape == want.shape
    bad = got != want
    assert not bad.any(), f"differs at {np.argwhere(bad)[0]}: {got[bad][0]!r} vs {want[bad][0]!r}"
    w = api_frames.build(b2)
    other = w.bodies[1].fixtures[0]
    with pytest.raises(ValueError):
        w.bodies[2].destroy_fixture(other)


def test_records_after_destroy_fixture_step_like_the_reference():
    """The host records the API leaves after create_fixtures / destroy_fixture
    (bodies, fixtures, fat AABBs, the pending move buffer) stepped by the
    CPU restatement reproduce the reference's world after the same calls and
    the same steps, bit for bit: they are what the next GPU step uploads."""
    import oracle_lib
    d = np.load(os.path.join(GOLDEN, "queries.npz"))
    _, w = api_frames.destroy_rows(b2)
    B, F, C, M = w._B, w._F, w._C, w._M
    assert list(B["fixture_start"]) == list(np.concatenate([[0], np.cumsum(B["fixture_count"])[:-1]]))
    W = w._sb.world_record(len(B), len(F), len(M))
    W["contact_count"] = len(C)
    W["inv_dt0"] = w._inv_dt0
    orc = oracle_lib.OracleWorld(W, B, F, contacts=C if len(C) else None, libm=True, moves=M)
    for _ in range(api_frames.STEPS_AFTER_DESTROY):
        orc.step(1 / 60, 8, 3)
    want = d["destroy_fixture_bodies"]
    got = orc.bodies()
    for name in ("cx", "cy", "a", "vx", "vy", "w", "flags", "sleep_time"):
        assert np.array_equal(got[name], want[name]), f"bodies.{name}"
    assert len(orc.contacts()) == len(d["destroy_fixture_contacts"])


def test_mass_data_setter_and_reset_match_reference():
    """mass_data overrides and reset_mass_data (body.py:575-641), then 40
    steps of the restatement on the records left behind, against the
    reference after the same calls and steps, bit for bit."""
    import oracle_lib
    d = np.load(os.path.join(GOLDEN, "queries.npz"))
    rows, w = api_frames.mass_rows(b2)
    got = np.array(rows, dtype=np.float64)
    want = d["mass_data"]
    bad = got != want
    assert got.shape == want.shape and not bad.any(), f"differs at {np.argwhere(bad)[:3].tolist()}"
    B, F, C, M = w._B, w._F, w._C, w._M
    W = w._sb.world_record(len(B), len(F), len(M))
    orc = oracle_lib.OracleWorld(W, B, F, contacts=None, libm=True, moves=M)
    for _ in range(api_frames.STEPS_AFTER_DESTROY):
        orc.step(1 / 60, 8, 3)
    want_b, got_b = d["mass_data_bodies"], orc.bodies()
    for name in ("cx", "cy", "a", "vx", "vy", "w", "mass", "I", "lcx", "lcy"):
        assert np.array_equal(got_b[name], want_b[name]), f"bodies.{name}"


def test_type_fixed_rotation_and_sleeping_setters_match_reference():
    """Body.type (with mass reset, wake, refilter), fixed_rotation and
    sleeping setters, then 40 restated steps on the records they leave,
    against the reference after the same calls and steps, bit for bit."""
    import oracle_lib
    d = np.load(os.path.join(GOLDEN, "queries.npz"))
    rows, w = api_frames.type_rows(b2)
    got, want = np.array(rows, dtype=np.float64), d["body_setters"]
    bad = got != want
    assert got.shape == want.shape and not bad.any(), f"differs at {np.argwhere(bad)[:3].tolist()}"
    B, F, C, M = w._B, w._F, w._C, w._M
    W = w._sb.world_record(len(B), len(F), len(M))
    orc = oracle_lib.OracleWorld(W, B, F, contacts=None, libm=True, moves=M)
    for _ in range(api_frames.STEPS_AFTER_DESTROY):
        orc.step(1 / 60, 8, 3)
    want_b, got_b = d["body_setters_bodies"], orc.bodies()
    for name in ("type", "cx", "cy", "a", "vx", "vy", "w", "flags", "sleep_time", "mass", "I"):
        assert np.array_equal(got_b[name], want_b[name]), f"bodies.{name}"
    assert len(orc.contacts()) == len(d["body_setters_contacts"])


def test_fixture_setters_match_reference():
    """Fixture friction, restitution, density, sensor and filter setters
    (fixture.py:122-225, refiltering on filter changes), then 40 restated
    steps on the records they leave, against the reference: bodies and the
    contacts (pairs, mixed friction and restitution, flags) bit for bit."""
    import oracle_lib
    d = np.load(os.path.join(GOLDEN, "queries.npz"))
    rows, w = api_frames.fixture_rows(b2)
    got, want = np.array(rows, dtype=np.float64), d["fixture_setters"]
    bad = got != want
    assert got.shape == want.shape and not bad.any(), f"differs at {np.argwhere(bad)[:3].tolist()}"
    B, F, C, M = w._B, w._F, w._C, w._M
    W = w._sb.world_record(len(B), len(F), len(M))
    orc = oracle_lib.OracleWorld(W, B, F, contacts=None, libm=True, moves=M)
    for _ in range(api_frames.STEPS_AFTER_DESTROY):
        orc.step(1 / 60, 8, 3)
    want_b, got_b = d["fixture_setters_bodies"], orc.bodies()
    for name in ("cx", "cy", "a", "vx", "vy", "w", "flags", "mass", "I"):
        assert np.array_equal(got_b[name], want_b[name]), f"bodies.{name}"
    want_c, got_c = d["fixture_setters_contacts"], orc.contacts()
    assert len(got_c) == len(want_c) and len(want_c) > 0
    for name in ("fixture_a", "fixture_b", "friction", "restitution", "flags"):
        assert np.array_equal(got_c[name], want_c[name]), f"contacts.{name}"


@pytest.mark.parametrize("scene", ["mixed", "uneven"])
def test_world_manifold_matches_reference(scene):
    """Contact.world_manifold (contact_util.py:195-245: circles, face A and
    face B manifolds) of every contact of two stepped reference worlds, from
    the exported records, bit for bit."""
    from pypybox2d_gb300.world import world_manifold
    d = np.load(os.path.join(GOLDEN, "queries.npz"))
    B, F, C, want = d[f"{scene}_bodies"], d[f"{scene}_fixtures"], d[f"{scene}_contacts"], d[f"{scene}_world_manifolds"]
    types = set()
    for i, c in enumerate(C):
        normal, pts = world_manifold(c, B, F)
        got = np.full(6, np.nan)
        got[0], got[1] = normal[0], normal[1]
        for k, p in enumerate(pts):
            got[2 + 2 * k], got[3 + 2 * k] = p[0], p[1]
        same = (got == want[i]) | (np.isnan(got) & np.isnan(want[i]))
        assert same.all(), f"contact {i} (type {int(c['m_type'])}): {got} vs {want[i]}"
        if int(c["m_point_count"]):
            types.add(int(c["m_type"]))
    assert types == {0, 1, 2} or scene == "uneven"


def test_manifold_view_decodes_feature_ids():
    from pypybox2d_gb300 import abi
    from pypybox2d_gb300.world import Contact
    d = np.load(os.path.join(GOLDEN, "queries.npz"))
    C = d["mixed_contacts"]
    c = next(r for r in C if r["m_point_count"] == 2)

    class _W:            # the two fixture lookups a Contact makes
        def _fixture_child_at(self, f):
            return f, 0
    m = Contact(_W(), c).manifold
    assert m.type == int(c["m_type"]) and m.point_count == 2
    for k, p in enumerate(m.points):
        i = int(c["p_id"][k])
        assert p.id == (i & 255, (i >> 8) & 255, (i >> 16) & 255, i >> 24)
        assert (p.local_point[0], p.local_point[1], p.normal_impulse) == (c["p_lx"][k], c["p_ly"][k], c["p_ni"][k])
    assert m.type in (abi.M_CIRCLES, abi.M_FACE_A, abi.M_FACE_B)


def test_host_edits_between_steps_match_reference():
    """tests/golden/api_edits.py: fixture, filter, mass and body edits (and
    a fixture destroyed while touching) between steps of a world with live
    contacts, the World stepped by the libm build of the restatement:
    bodies, fat AABBs, contacts and the end_contact calls equal the
    reference's session bit for bit.  This checks the records every edit
    leaves for the next device upload."""
    import types
    import api_edits
    import oracle_lib

    class OracleBackedWorld(b2.World):
        def _make_batch(self, W, B, F, C, M, J=None, CT=None, CB=None):
            return oracle_lib.OracleBatch(W, B, F, C, M, libm=True, joints=J, controllers=CT, controller_bodies=CB)

    d = np.load(os.path.join(GOLDEN, "queries.npz"))
    snaps = {}

    def snap(label, world):
        world._materialise()
        snaps[label] = (world._B.copy(), world._F["aabb"].copy(), world._C.copy())

    ns = types.SimpleNamespace(World=OracleBackedWorld, Body=b2.Body, shapes=b2.shapes)
    _, log = api_edits.script(ns, snap)
    assert tuple(snaps) == api_edits.SNAPS
    for label, (B, aabb, C) in snaps.items():
        want_b = d[f"edits_{label}_bodies"]
        for name in want_b.dtype.names:
            if not name.startswith("_pad"):
                assert np.array_equal(B[name], want_b[name]), f"{label} bodies.{name}"
        assert np.array_equal(aabb, d[f"edits_{label}_aabb"]), f"{label} fat AABBs"
        want_c = d[f"edits_{label}_contacts"]
        assert len(C) == len(want_c), f"{label} contact count"
        for name in ("fixture_a", "fixture_b", "flags", "friction", "restitution", "m_point_count", "m_type"):
            assert np.array_equal(C[name], want_c[name]), f"{label} contacts.{name}"
    assert np.array_equal(np.array(log, dtype=np.int32).reshape(-1, 2), d["edits_end_log"])


def test_unsupported_joints_raise_clearly():
    w = b2.World()
    for name in ("create_gear_joint",):
        with pytest.raises(NotImplementedError):
            getattr(w, name)()
    with pytest.raises(NotImplementedError):
        w.add_body(object())
    with pytest.raises(NotImplementedError):
        w.add_joint(object())
