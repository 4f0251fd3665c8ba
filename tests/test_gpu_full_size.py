"""The 1M dam break at full size (999,698 fluid / 1,024,618 particles, the
benchmark's workload), through size-independent properties: the CPU oracle
takes over a minute per step there, so these checks stand in for it.

* the lattice known answer: every fluid particle whose 3.1 l0 disk lies
  inside the particle lattice has exactly 28 neighbours in the initial list;
* after steps of the mixed engine, the neighbour relation is symmetric with
  bit-identical distances in both directions, every distance lies in
  (0, re_max), no particle is its own neighbour, and the PPE matrix is
  bitwise symmetric with rows only for Inner particles (src/mps.cpp:322-360);
* from one developed state, one mixed step and one FP64 step give the same
  surface flags, pressures within the mixed solver's tolerance and positions
  within 1e-9 m;
* five steps as CUDA graph replays and as eager launches end in bit-identical
  states (the solver's reductions have a fixed order).
"""
import numpy as np
import pytest

from gpu_util import engine_or_skip, rel_l2

pytestmark = pytest.mark.gpu

BC_INNER = 2


def _dambreak_1m():
    from mps_gb300 import scenes

    return scenes.dam_break(0.5 / 707, tank=(2.0, 1.2), column=(0.5, 1.0), dt=5e-5)


def _csr(vals, cols, offsets, n):
    from scipy.sparse import csr_matrix

    return csr_matrix((vals, cols, offsets), shape=(n, n))


def test_full_size_lists_matrix_and_mixed_step():
    m = engine_or_skip()
    pytest.importorskip("scipy.sparse")
    prm, pos, vel, t = _dambreak_1m()
    n, l0 = len(t), prm["particle_distance"]
    assert int((t == 0).sum()) == 999_698
    re_max = max(prm["re_pressure"], prm["re_viscosity"], prm["re_surface"])

    e = m.Engine(prm, pos, vel, t, precision=m.MIXED)
    off, ids, dist = e.neighbors()
    cnt = np.diff(off)
    inside = (t == 0) & (pos[:, 0] < 0.5 - 3.5 * l0) & (pos[:, 1] < 1.0 - 3.5 * l0)
    assert inside.sum() > 0.98 * (t == 0).sum()
    assert np.all(cnt[inside] == 28)
    assert cnt.max() <= 28

    for _ in range(3):
        assert e.step()["status"] == 0
    off, ids, dist = e.neighbors()
    rows = np.repeat(np.arange(n, dtype=np.int32), np.diff(off))
    assert np.all(ids != rows)
    assert np.all(dist > 0.0) and np.all(dist < re_max)
    nb = _csr(dist, ids, off, n)
    assert (nb != nb.T).nnz == 0  # same pairs, same distance bits both ways

    s = e.state()
    src, rp, col, val = e.system()
    a = _csr(val, col, rp, n)
    assert (a != a.T).nnz == 0
    has_row = np.diff(rp) > 0
    assert np.array_equal(has_row, s["bc"] == BC_INNER)
    assert np.all(src[s["bc"] != BC_INNER] == 0.0)
    e.close()

    # one mixed and one FP64 step from the developed state
    out = {}
    for name, prec in (("mixed", m.MIXED), ("fp64", m.FP64)):
        g = m.Engine(prm, s["pos"], s["vel"], s["type"], precision=prec)
        assert g.step()["status"] == 0
        out[name] = g.state()
        g.close()
    mx, fp = out["mixed"], out["fp64"]
    assert np.array_equal(mx["bc"], fp["bc"])
    assert np.array_equal(mx["type"], fp["type"])
    assert rel_l2(mx["pressure"], fp["pressure"]) < 1e-6
    assert np.max(np.abs(mx["pos"] - fp["pos"])) < 1e-9


def test_full_size_graph_replays_equal_eager_steps():
    """Determinism at full size: the same five steps as CUDA graph replays and
    as eager launches end in bit-identical states."""
    m = engine_or_skip()
    prm, pos, vel, t = _dambreak_1m()
    out = []
    for graphs in (True, False):
        e = m.Engine(prm, pos, vel, t, precision=m.MIXED)
        e.set_graphs(graphs)
        st = [e.step() for _ in range(5)]
        assert all(x["status"] == 0 for x in st)
        if graphs:
            assert st[-1]["graph_replayed"]
        out.append((e.state(), [x["cg_iterations"] for x in st]))
        e.close()
    (a, ia), (b, ib) = out
    assert ia == ib
    for k in a:
        assert np.array_equal(a[k], b[k]), k
