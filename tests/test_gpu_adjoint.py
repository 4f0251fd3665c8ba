"""The trajectory adjoint (mps_trajectory_backward) against central finite
differences of the same trajectory: on the GPU engine itself, and on the CPU
oracle (the reference's FP64 step), for the gradient w.r.t. gravity and for
directional derivatives w.r.t. the initial velocities.

Tolerance: relative 1e-4 between adjoint and finite differences (epsilon
1e-6 on gravity, a relative step on velocity directions), FP64 throughout.
"""
import numpy as np
import pytest

from gpu_util import engine_or_skip

pytestmark = pytest.mark.gpu

REL = 1e-4


def _scene(l0, size, steps, seed):
    from mps_gb300 import scenes

    prm, pos, vel, t = scenes.hydrostatic(l0, size=size, dt=1e-3)
    rng = np.random.default_rng(seed)
    fl = t == scenes.FLUID
    vel[fl, :2] = rng.normal(0.0, 0.01, (fl.sum(), 2))
    target = pos[fl] + np.c_[rng.normal(0.0, 0.1 * l0, (fl.sum(), 2)), np.zeros(fl.sum())]
    return prm, pos, vel, t, fl, target


def _loss_np(sp, pos, fl, target, w_p, w_x):
    return w_p * float(np.mean(sp ** 2)) + w_x * float(np.sum((pos[fl] - target) ** 2))


def _adjoint(m, prm, pos, vel, t, sensors, steps, every, fl, target, w_p, w_x):
    eng = m.Engine(prm, pos, vel, t, precision=m.FP64)
    tr = m.Trajectory(eng, steps, every, sensors)
    g = np.array(prm["gravity"], float)
    sp, pf, vf = tr.forward(vel, g)
    d_sp = w_p * 2.0 * sp / sp.size
    d_pos = np.zeros_like(pf)
    d_pos[fl] = w_x * 2.0 * (pf[fl] - target)
    gp, gv, gg = tr.backward(d_sp, d_pos, None)
    return eng, tr, sp, pf, gv, gg


def _fd_gpu(tr, vel, g, fl, target, w_p, w_x):
    sp, pf, _ = tr.forward(vel, g)
    return _loss_np(sp, pf, fl, target, w_p, w_x)


@pytest.mark.parametrize("terms", ["pressure", "position"])
def test_adjoint_vs_finite_differences_small(terms):
    """Small hydrostatic tank, several checkpoint segments: both loss terms."""
    m = engine_or_skip()
    from adjoint_harness import wall_sensors

    l0, steps, every = 0.02, 12, 5
    prm, pos, vel, t, fl, target = _scene(l0, (0.3, 0.3), steps, seed=7)
    sensors = wall_sensors(pos, t, l0, 8)
    w_p, w_x = (1.0, 0.0) if terms == "pressure" else (0.0, 1.0)
    eng, tr, sp, pf, gv, gg = _adjoint(m, prm, pos, vel, t, sensors, steps, every, fl, target,
                                       w_p, w_x)
    g = np.array(prm["gravity"], float)
    # gravity
    for d in (0, 1):
        eps = 1e-6
        gp_, gm_ = g.copy(), g.copy()
        gp_[d] += eps
        gm_[d] -= eps
        fd = (_fd_gpu(tr, vel, gp_, fl, target, w_p, w_x) - _fd_gpu(tr, vel, gm_, fl, target, w_p, w_x)) / (2 * eps)
        assert abs(gg[d] - fd) <= REL * max(abs(fd), 1e-3 * np.abs(gg).max()), (d, gg[d], fd)
    # initial-velocity directions (fluid only, in-plane)
    rng = np.random.default_rng(11)
    for _ in range(3):
        u = np.zeros_like(vel)
        u[fl, :2] = rng.normal(size=(fl.sum(), 2))
        u /= np.linalg.norm(u)
        eps = 1e-6
        fd = (_fd_gpu(tr, vel + eps * u, g, fl, target, w_p, w_x)
              - _fd_gpu(tr, vel - eps * u, g, fl, target, w_p, w_x)) / (2 * eps)
        ad = float(np.sum(gv * u))
        assert abs(ad - fd) <= REL * max(abs(fd), 1e-3 * np.linalg.norm(gv)), (ad, fd)
    tr.close()
    eng.close()


def test_adjoint_vs_oracle_finite_differences():
    """The adjoint against finite differences of the CPU oracle (the
    reference's FP64 step, pinned to its sources) on the same trajectory."""
    m = engine_or_skip()
    from adjoint_harness import wall_sensors
    from oracle import Oracle

    l0, steps, every = 0.02, 8, 3
    prm, pos, vel, t, fl, target = _scene(l0, (0.3, 0.3), steps, seed=3)
    sensors = wall_sensors(pos, t, l0, 8)
    eng, tr, sp, pf, gv, gg = _adjoint(m, prm, pos, vel, t, sensors, steps, every, fl, target,
                                       1.0, 1e6)

    def oracle_loss(v0, gvec):
        p = dict(prm)
        p["gravity"] = list(gvec)
        o = Oracle(p, pos, v0, t)
        o.set_cg(solves=1)
        sps = []
        for _ in range(steps):
            o.step()
            sps.append(o.state()["pressure"][sensors])
        st = o.state()
        return _loss_np(np.array(sps), st["pos"], fl, target, 1.0, 1e6)

    g = np.array(prm["gravity"], float)
    eps = 1e-6
    gp_, gm_ = g.copy(), g.copy()
    gp_[1] += eps
    gm_[1] -= eps
    fd = (oracle_loss(vel, gp_) - oracle_loss(vel, gm_)) / (2 * eps)
    assert abs(gg[1] - fd) <= REL * abs(fd), (gg[1], fd)
    rng = np.random.default_rng(5)
    u = np.zeros_like(vel)
    u[fl, :2] = rng.normal(size=(fl.sum(), 2))
    u /= np.linalg.norm(u)
    fd = (oracle_loss(vel + eps * u, g) - oracle_loss(vel - eps * u, g)) / (2 * eps)
    ad = float(np.sum(gv * u))
    assert abs(ad - fd) <= REL * abs(fd), (ad, fd)
    tr.close()
    eng.close()


def test_torch_autograd_function():
    """The torch.autograd.Function wrapper gives the same gradients as the
    direct C ABI calls, and its forward leaves the engine at the final state."""
    m = engine_or_skip()
    import torch

    from adjoint_harness import MpsTrajectoryFn, position_loss, sensor_loss, wall_sensors

    l0, steps, every = 0.02, 6, 4
    prm, pos, vel, t, fl, target = _scene(l0, (0.3, 0.3), steps, seed=9)
    sensors = wall_sensors(pos, t, l0, 16)
    eng = m.Engine(prm, pos, vel, t, precision=m.FP64)
    tr = m.Trajectory(eng, steps, every, sensors)
    v0 = torch.tensor(vel, dtype=torch.float64, requires_grad=True)
    g = torch.tensor(prm["gravity"], dtype=torch.float64, requires_grad=True)
    sp, pf, vf = MpsTrajectoryFn.apply(v0, g, tr)
    fm = torch.from_numpy(fl)
    loss = sensor_loss(sp) + position_loss(pf, torch.from_numpy(target), fm)
    loss.backward()
    st = eng.state()
    assert np.array_equal(st["pos"], pf.detach().numpy())
    # the same VJP through the raw binding
    d_sp = 2.0 * sp.detach().numpy() / sp.numel()
    d_pos = np.zeros_like(pf.detach().numpy())
    d_pos[fl] = 2.0 * (pf.detach().numpy()[fl] - target)
    _, gv, gg = tr.backward(d_sp, d_pos, None)
    assert np.allclose(v0.grad.numpy(), gv, rtol=1e-12, atol=0)
    assert np.allclose(g.grad.numpy(), gg, rtol=1e-12, atol=0)
    assert np.all(np.isfinite(gv)) and np.abs(gv[fl]).max() > 0
    tr.close()
    eng.close()


def test_adjoint_3d_against_finite_differences():
    """A non-planar scene (the 3-D box of the golden set, seeded 3-D initial
    velocities): the adjoint's z components (gravity and velocities) against
    central finite differences."""
    m = engine_or_skip()
    from golden_cases import load

    g = load("box3d")
    prm = dict(g["params"])
    pos, t = g["pos0"], g["type0"]
    rng = np.random.default_rng(21)
    fl = t == 0
    vel = np.zeros_like(pos)
    vel[fl] = rng.normal(0.0, 0.01, (fl.sum(), 3))
    steps, every = 6, 4
    target = pos[fl] + rng.normal(0.0, 1e-3, (fl.sum(), 3))
    eng = m.Engine(prm, pos, vel, t, precision=m.FP64)
    tr = m.Trajectory(eng, steps, every, np.flatnonzero(t == 1)[:8].astype(np.int32))
    gv0 = np.array(prm["gravity"], float)

    def loss(v0, gvec):
        sp, pf, _ = tr.forward(v0, gvec)
        return float(np.mean(sp ** 2)) + 1e6 * float(np.sum((pf[fl] - target) ** 2)), sp, pf

    L, sp, pf = loss(vel, gv0)
    d_pos = np.zeros_like(pf)
    d_pos[fl] = 2e6 * (pf[fl] - target)
    _, gvel, gg = tr.backward(2.0 * sp / sp.size, d_pos, None)
    eps = 1e-6
    for d in (1, 2):
        gp, gm = gv0.copy(), gv0.copy()
        gp[d] += eps
        gm[d] -= eps
        fd = (loss(vel, gp)[0] - loss(vel, gm)[0]) / (2 * eps)
        assert abs(gg[d] - fd) <= REL * max(abs(fd), 1e-3 * np.abs(gg).max()), (d, gg[d], fd)
    u = np.zeros_like(vel)
    u[fl] = rng.normal(size=(fl.sum(), 3))
    u /= np.linalg.norm(u)
    fd = (loss(vel + eps * u, gv0)[0] - loss(vel - eps * u, gv0)[0]) / (2 * eps)
    ad = float(np.sum(gvel * u))
    assert abs(ad - fd) <= REL * max(abs(fd), 1e-3 * np.linalg.norm(gvel)), (ad, fd)
    tr.close()
    eng.close()
