"""Batches (mps_batch_*): many scenes per step with one shared persistent
solve launch, against the same scenes stepped one engine at a time.

The batch's pre- and post-solve kernels are the single engine's, so surface
flags, types and neighbour counts must be identical; the solve differs only in
how its dot products are split over blocks (each scene's group vs the whole
grid), so pressures agree to the solver tolerance (stated per assertion).
"""
import numpy as np
import pytest

from gpu_util import engine_or_skip, rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-8


def _small_scenes(n=6):
    from mps_gb300 import scenes

    return scenes.batch_scenes(seed=4, n_scenes=n, fluid_range=(200, 2500),
                               l0_range=(0.008, 0.02))


def _single(m, sc, steps):
    out = []
    for prm, pos, vel, t in sc:
        e = m.Engine(prm, pos, vel, t, precision=m.MIXED, tol=TOL)
        for _ in range(steps):
            st = e.step()
        out.append((e.state(), st))
        e.close()
    return out


@pytest.mark.parametrize("block", [256, 512, 1024])
def test_batch_matches_single_engines(block):
    m = engine_or_skip()
    sc = _small_scenes()
    steps = 3
    ref = _single(m, sc, steps)
    b = m.Batch(sc, tol=TOL)
    b.set_launch(block, 1.25)
    for _ in range(steps):
        stats, ms = b.step()
    info = b.launch_info()
    assert info["block"] == block and sum(info["group_blocks"]) == info["grid"]
    assert min(info["group_blocks"]) >= 1
    for s, (r, rst) in enumerate(ref):
        got = b.scene(s).state()
        for k in ("type", "bc", "dirichlet"):
            assert np.array_equal(got[k], r[k]), (s, k)
        assert rel_l2(got["pressure"], r["pressure"]) < 1e-5, s   # both solved to 1e-8
        assert np.max(np.abs(got["pos"] - r["pos"])) < 1e-8, s    # metres
        assert stats[s]["cg_relative_residual"] <= TOL, s          # per-scene convergence
        assert stats[s]["n_inner"] == rst["n_inner"], s
    assert all(st["graph_replayed"] == 1 for st in stats)
    b.close()


def test_batch_autotune_and_graph_replay():
    m = engine_or_skip()
    sc = _small_scenes(8)
    b = m.Batch(sc, tol=TOL)
    stats, _ = b.step()          # autotuning step (eager)
    info = b.launch_info()
    assert info["block"] in (256, 512, 1024) and len(info["tune_ms"]) == 9
    assert all(t > 0 for t in info["tune_ms"])
    assert all(st["graph_replayed"] == 0 for st in stats)
    stats, ms = b.step(2)        # captured once, then replayed
    assert ms > 0 and all(st["graph_replayed"] == 1 for st in stats)
    assert all(st["status"] == 0 for st in stats)
    b.close()
