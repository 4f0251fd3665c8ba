"""The batched driver loop (mps_run_report: many steps, one host wait per
up to 256 of them) against the same steps made one by one (mps_step): every
step's reported Courant number, iteration count, debug-event counts and
status, and the final state, identical bit for bit; the per-step device
times are positive and add up to about the batch's own duration."""
import numpy as np
import pytest

from golden_cases import load
from gpu_util import engine_or_skip

pytestmark = pytest.mark.gpu


# the dam break over 300 steps (two groups of the batched run: 256 + 44);
# the jittered scene (collisions and ghosts: debug events) over 12
@pytest.mark.parametrize("case,steps", [("ref_dambreak", 300), ("jitter_collide", 12)])
@pytest.mark.parametrize("precision", ["FP64", "MIXED"])
def test_run_report_matches_single_steps(precision, case, steps):
    m = engine_or_skip()
    g = load(case)
    prec = getattr(m, precision)
    a = m.Engine(g["params"], g["pos0"], g["vel0"], g["type0"], precision=prec)
    b = m.Engine(g["params"], g["pos0"], g["vel0"], g["type0"], precision=prec)
    one = [a.step() for _ in range(steps)]
    many = b.run_report(steps)
    assert len(many) == steps
    keys = ("courant", "cg_iterations", "cg_relative_residual", "refinements", "debug_log_count",
            "n_collision_candidates", "n_new_ghosts", "n_unconnected", "n_inner", "n_surface", "status")
    for s, (x, y) in enumerate(zip(one, many)):
        for k in keys:
            assert x[k] == y[k], (s, k, x[k], y[k])
        assert y["ms_step"] > 0.0
    if case == "jitter_collide":
        assert many[-1]["debug_log_count"] > 0
    sa, sb = a.state(), b.state()
    for k in sa:
        assert np.array_equal(sa[k], sb[k]), k
    a.close()
    b.close()


def test_run_report_zero_steps_and_bad_arguments():
    m = engine_or_skip()
    from mps_gb300 import engine

    g = load("ref_dambreak")
    e = m.Engine(g["params"], g["pos0"], g["vel0"], g["type0"])
    assert e.run_report(0) == []
    lib = engine.load()
    assert lib.mps_run_report(e._h, 3, None) == engine.MPS_ERR_ARG
    assert lib.mps_run_report(e._h, -1, None) == engine.MPS_ERR_ARG
    e.close()
