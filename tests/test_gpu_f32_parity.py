"""The float32 batched form against the float64 oracle.

From identical float64 state (a sample batch settled by the float64 GPU
path, which the parity tests hold bit-exact to the oracle), one float32 step
on the GPU and one step of the oracle (the CPU restatement of World.step,
pypybox2d/world.py:307-354) solved in the float32 step's constraint order.

Tolerance, continuous: every world's largest position difference over the
dynamic bodies of islands in which both steps took the same decisions is at
most 1e-5 m (the batched form's stated per-step error).  The decisions a
step's final state does not show come from the step record
(gb_batch_get_step_record / or_get_step_record): the position iterations
each island ran before its early exit (island.py:141-153), the TOI
position-pass iterations and events of each body (contact.py:866-933) and
the restitution-bias and block-solver choices of its constraints
(contact.py:470-496).  Some of these sit on a threshold by construction: a
TOI event of a body moving in a straight line puts the separation after one
TOI position pass exactly on that pass's -1.5 slop early exit, so rounding
decides whether one more pass runs (3/32 of the slop, 4.7e-4 m).  The
decisions taken apart (step-record fields per body, plus the bodies of
contacts whose narrow-phase results differ) are counted and held to
MAX_DECISIONS_APART_RATE of the bodies compared; the islands they sit in (as
the solve's step record names them) are left out of the continuous bound.
Discrete state (pair set, contact order, touching flags, manifold types,
point counts, feature ids, awake flags, re-fattened proxies): the counts of
differences are printed and held to MAX_DISCRETE_RATE of the contacts (and
bodies, for the awake flags) compared, summed over the sample.

Samples: 64 uneven worlds spread over 10-2000 bodies at steps 60, 300 and
1000; 16 jittered pyramids at steps 60 and 300.
"""
import numpy as np
import pytest

from pypybox2d_gb300 import precision, scenes

pytestmark = pytest.mark.gpu

DT, VI, PI = 1.0 / 60.0, 8, 3
TOL_M = 1e-5
MAX_DISCRETE_RATE = 1e-3
MAX_DECISIONS_APART_RATE = 5e-3


def _oracle_step(W, B, F, C, orders):
    import oracle_lib
    Bo, Po, Cs, Rs = B.copy(), F["aabb"].copy(), [], []
    for w in range(len(W)):
        o = oracle_lib.OracleWorld(W, B, F, C, index=w)
        o.step(DT, VI, PI, order=orders[w])
        b0, nb = int(W["body_start"][w]), int(W["body_count"][w])
        f0, nf = int(W["fixture_start"][w]), int(W["fixture_count"][w])
        Bo[b0:b0 + nb] = o.bodies()
        Po[f0:f0 + nf] = o.fixtures()["aabb"]
        Cs.append(o.contacts())
        Rs.append(o.step_record())
    return Bo, Po, Cs, Rs


def _check(label, W, B, F, C):
    r = precision.one_step(W, B, F, C, DT, VI, PI, reference=_oracle_step)
    errs, alike, mm = r["errors"], r["errors_alike"], r["mismatch"]
    worst = int(np.argmax(alike[:, 0]))
    print(f"\n{label}: position error over islands decided alike {alike[:, 0].max():.3e} m (world {worst}), "
          f"over all bodies {errs[:, 0].max():.3e} m; angle {alike[:, 1].max():.3e} rad, velocity "
          f"{alike[:, 2].max():.3e} m/s; bodies decided apart {r['bodies_decided_apart']}; discrete mismatches {mm}")
    assert alike[:, 0].max() <= TOL_M, f"{label}: worlds over {TOL_M} m: {np.flatnonzero(alike[:, 0] > TOL_M).tolist()}"
    contact_diffs = mm["pairs"] + mm["touching"] + mm["manifold_type"] + mm["point_count"] + mm["feature_ids"]
    assert contact_diffs <= MAX_DISCRETE_RATE * max(mm["contacts"], 1), f"{label}: {mm}"
    assert mm["awake"] <= MAX_DISCRETE_RATE * max(mm["bodies"], 1), f"{label}: {mm}"
    assert r["decisions_apart"] <= MAX_DECISIONS_APART_RATE * max(mm["bodies"], 1), f"{label}: {mm}"
    return r


def _settled_samples(W, B, F, M, checkpoints):
    from pypybox2d_gb300.gpu import GpuBatch
    g = GpuBatch(W, B, F, precision="f64", moves=M)
    done = 0
    for s in checkpoints:
        g.step(DT, VI, PI, s - done, launch_mode=3, block_threads=64)
        done = s
        yield s, precision.batch_records(g, F, 1.0 / DT)


def test_f32_uneven_sample_against_the_oracle():
    counts = np.geomspace(10, 2000, 64).round().astype(int)
    W, B, F, M = scenes.uneven_batch(64, seed=100, counts=counts)
    for s, rec in _settled_samples(W, B, F, M, (60, 300, 1000)):
        _check(f"uneven x64 at step {s}", *rec)


def test_f32_pyramid_sample_against_the_oracle():
    W, B, F, M = scenes.pyramid_batch(16, rows=20, jitter=0.01, seed=7)
    for s, rec in _settled_samples(W, B, F, M, (60, 300)):
        _check(f"pyramid x16 at step {s}", *rec)
