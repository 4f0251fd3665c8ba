"""Failure statuses of the C ABI, made on the host (no GPU fault, trap or hang):

* a pressure solve stopped at a tiny iteration cap reports
  MPS_ERR_NOT_CONVERGED, and the step still advanced the state, as the
  reference's step does after its solver.info() check (src/mps.cpp:462-464);
* a NaN position uploaded by the caller is caught by the next neighbour
  search: MPS_ERR_NONFINITE, the particle becomes a Ghost, later steps run;
* the matrix symmetry test of solvePoissonEquation (src/mps.cpp:418-442),
  through mps_check_symmetry on host-built CSR matrices: the reference's own
  golden matrix passes, and a perturbed copy reports the reference's first
  asymmetric pair.
"""
import numpy as np
import pytest

from golden_cases import load
from gpu_util import engine_or_skip

pytestmark = pytest.mark.gpu


def _small_dam_break():
    from mps_gb300 import scenes

    return scenes.dam_break(0.02, tank=(0.6, 0.4), column=(0.2, 0.3))


@pytest.mark.parametrize("precision", ["FP64", "MIXED"])
def test_iteration_cap_reports_not_converged(precision):
    m = engine_or_skip()
    from mps_gb300 import engine

    prm, pos, vel, t = _small_dam_break()
    prec = getattr(m, precision)
    e = m.Engine(prm, pos, vel, t, precision=prec)
    for _ in range(12):  # until the pressure field is nonzero
        e.step()
    before = e.state()
    e.set_solver(prec, 0.0, 3)  # three (inner) iterations cannot reach the tolerance
    with pytest.raises(engine.MpsError) as ex:
        e.step()
    assert ex.value.code == engine.MPS_ERR_NOT_CONVERGED
    assert "iteration cap" in str(ex.value)
    after = e.state()
    assert not np.array_equal(after["pos"], before["pos"])  # the step completed
    assert np.all(np.isfinite(after["pressure"]))
    e.set_solver(prec)  # default cap again: the next step converges
    st = e.step()
    assert st["status"] == 0 and st["cg_relative_residual"] <= (1e-10 if prec == m.MIXED else 1e-13)
    e.close()


def test_nan_position_reports_nonfinite():
    m = engine_or_skip()
    from mps_gb300 import engine, scenes

    prm, pos, vel, t = _small_dam_break()
    e = m.Engine(prm, pos, vel, t, precision=m.FP64)
    e.step()
    s = e.state()
    k = int(np.flatnonzero(s["type"] == scenes.FLUID)[7])
    p = s["pos"].copy()
    p[k, 0] = np.nan
    e.upload(pos=p)
    with pytest.raises(engine.MpsError) as ex:
        e.step()
    assert ex.value.code == engine.MPS_ERR_NONFINITE
    r = e.state()
    assert r["type"][k] == scenes.GHOST
    assert np.all(np.isfinite(r["pressure"]))
    st = e.step()  # the particle left the neighbour search; the scene goes on
    assert st["status"] == 0
    assert np.all(np.isfinite(np.delete(e.state()["pos"], k, axis=0)))
    e.close()


def _golden_system(name="jitter_collide"):
    g = load(name)
    return g["s1_row_ptr"].astype(np.int64), g["s1_col"].astype(np.int32), g["s1_val"].astype(np.float64)


def _entry(rp, col, i, j):
    """Index of entry (i, j) in the CSR, or None."""
    hit = np.flatnonzero(col[rp[i]:rp[i + 1]] == j)
    return int(rp[i] + hit[0]) if len(hit) else None


def _offdiag_pairs(rp, col, count):
    """Some stored pairs i < j, spread over the matrix."""
    rows = np.repeat(np.arange(len(rp) - 1), np.diff(rp))
    up = np.flatnonzero(rows < col)
    pick = up[np.linspace(0, len(up) - 1, count).astype(int)]
    return [(int(rows[q]), int(col[q])) for q in pick]


def test_symmetry_check_on_the_reference_matrix():
    engine_or_skip()
    from mps_gb300 import engine

    rp, col, val = _golden_system()
    rc, i, j, msg = engine.check_symmetry(rp, col, val)
    assert rc == engine.MPS_OK and (i, j) == (-1, -1)


@pytest.mark.parametrize("how", ["upper_1e-6", "lower_1e-6", "dropped", "one_ulp", "two_pairs"])
def test_symmetry_check_reports_the_first_pair(how):
    engine_or_skip()
    from mps_gb300 import engine

    rp, col, val = _golden_system()
    (a, b), (c, d) = _offdiag_pairs(rp, col, 2)
    assert a < b and c < d and (a, b) < (c, d)
    v = val.copy()
    cl = col.copy()
    if how == "upper_1e-6":
        v[_entry(rp, col, a, b)] += 1e-6
    elif how == "lower_1e-6":
        v[_entry(rp, col, b, a)] -= 1e-6
    elif how == "dropped":  # A(b, a) set to an explicit zero: a missing entry
        v[_entry(rp, col, b, a)] = 0.0
    elif how == "one_ulp":
        q = _entry(rp, col, a, b)
        v[q] = np.nextafter(v[q], np.inf)
    else:  # the later pair differs beyond 1e-10, the earlier only by one ulp
        q = _entry(rp, col, a, b)
        v[q] = np.nextafter(v[q], np.inf)
        v[_entry(rp, col, c, d)] *= 1.01
    rc, i, j, msg = engine.check_symmetry(rp, cl, v)
    assert rc == engine.MPS_ERR_ASYMMETRIC
    want = (c, d) if how == "two_pairs" else (a, b)
    assert (i, j) == want, (i, j, want)
    assert msg.startswith(f"Matrix is not symmetric at ({want[0]}, {want[1]}): A({want[0]}, {want[1]}) = ")
    assert ("all differences <= 1e-10" in msg) == (how == "one_ulp")


def test_engine_steps_pass_their_symmetry_check():
    """Every step runs the check on its own matrix: a golden scene's steps
    return MPS_OK, and its assembled matrix passes mps_check_symmetry too."""
    m = engine_or_skip()
    from mps_gb300 import engine

    g = load("jitter_collide")
    e = m.Engine(g["params"], g["pos0"], g["vel0"], g["type0"], precision=m.MIXED)
    for _ in range(3):
        assert e.step()["status"] == 0
    _, rp, col, val = e.system()
    assert engine.check_symmetry(rp, col, val)[0] == engine.MPS_OK
    e.close()
