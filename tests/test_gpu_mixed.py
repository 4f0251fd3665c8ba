"""The mixed-precision solver against the FP64 one, from the same state, for
each preconditioner of the mixed solver (Jacobi, multigrid additive at the
particle level, multiplicative V(1,1), additive with the smoothed transfer):
the pressure agrees within relative L2 1e-6 (the solver stops at relative
residual 1e-10), surface flags exactly."""
import numpy as np
import pytest

from gpu_util import engine_or_skip, rel_l2

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", [0, 1, 2, 3])
def test_mixed_matches_fp64(mode):
    m = engine_or_skip()
    from mps_gb300 import scenes

    prm, pos, vel, t = scenes.dam_break(0.005, tank=(0.8, 0.5), column=(0.2, 0.4), dt=5e-4)
    warm = m.Engine(prm, pos, vel, t, precision=m.FP64)
    for _ in range(15):  # let the pressure field develop
        warm.step()
    w = warm.state()
    warm.close()
    ea = m.Engine(prm, w["pos"], w["vel"], w["type"], precision=m.FP64)
    eb = m.Engine(prm, w["pos"], w["vel"], w["type"], precision=m.MIXED)
    eb.set_multigrid(mode)
    sa, sb = ea.step(), eb.step()
    a, b = ea.state(), eb.state()
    assert np.linalg.norm(a["pressure"]) > 0
    assert rel_l2(b["pressure"], a["pressure"]) < 1e-6
    assert np.array_equal(a["bc"], b["bc"])
    assert sb["cg_relative_residual"] <= 1e-10
    if mode:
        assert sb["cg_iterations"] < sa["cg_iterations"] / 4  # the multigrid pays off
    ea.close()
    eb.close()


# Mixed trajectory against FP64 and the oracle (the 1M workload's solver on a crop)
P_TRAJ = 1e-6    # pressure relative L2 (the mixed solve's own error is ~1e-10 per step)
X_TRAJ = 1e-9    # metres, positions (particles move ~1e-6 m per step here)
V_TRAJ = 1e-6    # m/s


def test_mixed_trajectory_against_fp64_and_oracle():
    """60 steps of a 20,000-fluid-particle dam break (l0 2e-3 m, dt 2e-4 s:
    the 1M workload's dt / l0 ratio of 0.1 s/m) with the mixed solver and
    its default multigrid, side by side with the FP64 engine and the CPU
    oracle from the same initial state.  Every 10 steps: pressure within
    P_TRAJ relative L2, positions within X_TRAJ, velocities within V_TRAJ,
    surface flags, Dirichlet flags and types identical, collision pairs of
    every step identical."""
    m = engine_or_skip()
    from oracle import Oracle

    from mps_gb300 import scenes

    l0 = 2e-3
    prm, pos, vel, t = scenes.dam_break(l0, tank=(0.6, 0.5), column=(0.2, 0.4), dt=0.1 * l0)
    assert (t == scenes.FLUID).sum() == 20000 and len(t) <= 50000
    em = m.Engine(prm, pos, vel, t, precision=m.MIXED)
    ef = m.Engine(prm, pos, vel, t, precision=m.FP64)
    o = Oracle(prm, pos, vel, t)
    o.set_cg(solves=1)
    worst = {"p_fp64": 0.0, "p_oracle": 0.0, "x": 0.0, "v": 0.0}
    for s in range(1, 61):
        sm, sf, so = em.step(), ef.step(), o.step()
        assert sm["status"] == 0 and sm["cg_relative_residual"] <= 1e-10
        assert sm["debug_log_count"] == sf["debug_log_count"] == so["debug_log_count"], s
        mi, mj, _ = em.collisions()
        oi, oj, _ = o.collisions()
        assert np.array_equal(mi, oi) and np.array_equal(mj, oj), s
        if s % 10:
            continue
        a, b, c = em.state(), ef.state(), o.state()
        for k in ("type", "bc", "dirichlet"):
            assert np.array_equal(a[k], b[k]) and np.array_equal(a[k], c[k]), (s, k)
        assert np.linalg.norm(c["pressure"]) > 0
        worst["p_fp64"] = max(worst["p_fp64"], rel_l2(a["pressure"], b["pressure"]))
        worst["p_oracle"] = max(worst["p_oracle"], rel_l2(a["pressure"], c["pressure"]))
        worst["x"] = max(worst["x"], float(np.max(np.abs(a["pos"] - c["pos"]))))
        worst["v"] = max(worst["v"], float(np.max(np.abs(a["vel"] - c["vel"]))))
    assert worst["p_fp64"] < P_TRAJ and worst["p_oracle"] < P_TRAJ, worst
    assert worst["x"] < X_TRAJ and worst["v"] < V_TRAJ, worst
    em.close()
    ef.close()


def test_initial_guess_from_previous_step():
    """The mixed solver's default start from the previous step's solution
    against its zero start (the reference's): 40 steps of a dam break at the
    1M workload's dt / l0 from the same initial state; every step converges
    to the same tolerance, surface flags and types stay identical, pressures
    agree within 1e-7 relative L2, and the warm start needs fewer inner
    iterations in total.  The guess survives mps_upload: uploading the
    current state changes nothing in the next step (within the solver's
    tolerance); uploading an unrelated state (the initial one) makes the
    guess worse than zero, and the solve drops it and converges as a fresh
    engine's does."""
    m = engine_or_skip()
    from mps_gb300 import scenes

    l0 = 4e-3
    prm, pos, vel, t = scenes.dam_break(l0, tank=(0.6, 0.5), column=(0.2, 0.4), dt=0.1 * l0)
    ew = m.Engine(prm, pos, vel, t, precision=m.MIXED)
    ez = m.Engine(prm, pos, vel, t, precision=m.MIXED)
    ez.set_initial_guess(False)
    its = {"warm": 0, "zero": 0}
    worst = 0.0
    for s in range(1, 41):
        sw, sz = ew.step(), ez.step()
        for st in (sw, sz):
            assert st["status"] == 0 and st["cg_relative_residual"] <= 1e-10, s
        its["warm"] += sw["cg_iterations"]
        its["zero"] += sz["cg_iterations"]
        if s % 5 == 0:
            a, b = ew.state(), ez.state()
            assert np.array_equal(a["bc"], b["bc"]) and np.array_equal(a["type"], b["type"]), s
            worst = max(worst, rel_l2(a["pressure"], b["pressure"]))
    assert worst < 1e-7, worst
    assert its["warm"] < its["zero"], its
    # the current state uploaded again: the next step matches the one without upload
    st = ew.state()
    twin = m.Engine(prm, pos, vel, t, precision=m.MIXED)
    for _ in range(40):
        twin.step()
    ew.upload(pos=st["pos"], vel=st["vel"], types=st["type"])
    s1, s2 = ew.step(), twin.step()
    assert s1["status"] == 0 and s1["cg_relative_residual"] <= 1e-10
    assert rel_l2(ew.state()["pressure"], twin.state()["pressure"]) < 1e-7
    # an unrelated state: converges like a fresh engine's first step
    ew.upload(pos=pos, vel=vel, types=t)
    fresh = m.Engine(prm, pos, vel, t, precision=m.MIXED)
    s3, s4 = ew.step(), fresh.step()
    assert s3["status"] == 0 and s3["cg_relative_residual"] <= 1e-10
    assert rel_l2(ew.state()["pressure"], fresh.state()["pressure"]) < 1e-7
    for e in (ew, ez, twin, fresh):
        e.close()
