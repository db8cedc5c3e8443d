"""How far the portable sine/cosine moves the float64 step from the reference.

The float64 GPU path computes rotations with a portable sine/cosine (range
reduction and polynomials written in the library) that the oracle's
`liboracle.so` build shares formula for formula, so the GPU reproduces that
build bit for bit (tests/test_gpu_parity.py).  The reference uses libm, as
the oracle's `liboracle_libm.so` build does, and that build reproduces the
reference's golden vectors bit for bit (tests/test_oracle_golden.py).  This
test closes the chain: it steps the portable build in the reference's own
solver order against the golden vectors and bounds the difference the
sine/cosine alone makes.

Measured: the pyramid, bullet, sleep, kinematic, sensor/filter and 5-row pyramid scenes stay
within 1e-11 m of the reference over their whole runs (up to 300 steps) with
identical contact lists, touching flags, point counts, feature ids, sleep
flags and solver order.  The mixed and uneven scenes are chaotic piles: a
last-bit difference in a rotation grows until, after about 60 and 120 steps,
a discrete decision flips and the runs separate; up to step 30 they too are
identical in every discrete field and within 1e-11 m.
"""
import os

import numpy as np
import pytest

import oracle_lib

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL_M = 1e-11
# scene -> last snapshot step held to the bound (chaotic piles: the steps
# before the first discrete flip the sine/cosine causes)
HELD = {"pyramid": None, "pyramid5": None, "bullets": None, "sleep": None, "kinematic": None, "sensor_filter": None,
        "mixed": 30, "uneven": 60}


def _discrete_equal(o, d, s):
    c, rc = o.contacts(), d[f"s{s}_contacts"]
    b, rb = o.bodies(), d[f"s{s}_bodies"]
    return (len(c) == len(rc) and np.array_equal(c["fixture_a"], rc["fixture_a"]) and
            np.array_equal(c["fixture_b"], rc["fixture_b"]) and np.array_equal(c["flags"], rc["flags"]) and
            np.array_equal(c["m_point_count"], rc["m_point_count"]) and np.array_equal(c["m_type"], rc["m_type"]) and
            np.array_equal(c["p_id"], rc["p_id"]) and np.array_equal(b["flags"], rb["flags"]) and
            np.array_equal(o.solver_order(), d[f"s{s}_order"]))


@pytest.mark.parametrize("scene", sorted(HELD))
def test_portable_sincos_stays_with_the_reference(scene):
    d = np.load(os.path.join(GOLDEN, scene + ".npz"))
    dt = float(d["dt"][0])
    vi, pi = (int(x) for x in d["iters"])
    o = oracle_lib.OracleWorld(d["init_world"], d["init_bodies"], d["init_fixtures"], libm=False)
    snaps = [int(s) for s in d["snaps"]]
    last = HELD[scene] or max(snaps)
    worst = 0.0
    for s in range(1, last + 1):
        o.step(dt, vi, pi)
        if s in snaps:
            b, rb = o.bodies(), d[f"s{s}_bodies"]
            dp = float(np.hypot(b["cx"] - rb["cx"], b["cy"] - rb["cy"]).max())
            da = float(np.abs(b["a"] - rb["a"]).max())
            worst = max(worst, dp)
            assert dp <= TOL_M and da <= TOL_M, f"{scene} step {s}: position {dp:.2e} m, angle {da:.2e} rad"
            assert _discrete_equal(o, d, s), f"{scene} step {s}: discrete state differs"
    print(f"\n{scene}: largest position difference {worst:.1e} m over steps 1-{last}")
