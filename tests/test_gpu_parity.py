"""GPU engine (through the C ABI) against the reference's golden vectors and the oracle.

Bit-exact: neighbour lists (ids, order, FP64 distances), surface flags,
collision candidate pairs, source term and PPE matrix entries, Dirichlet
flags and number densities.  Within tolerance (stated per assertion):
pressures, which come from a CG whose parallel dot products sum in a
different order than the reference's serial ones, and everything downstream
of them.
"""
import numpy as np
import pytest

from golden_cases import CASES, load
from gpu_util import engine_or_skip, rel_l2

pytestmark = pytest.mark.gpu

# FP64 CG to machine epsilon on both sides: solutions agree to ~kappa * eps.
P_TOL = 1e-9     # relative L2 of pressure
X_TOL = 1e-12    # absolute, metres (positions move ~1e-5 m per step)
V_TOL = 1e-9     # absolute, m/s


@pytest.mark.parametrize("name", CASES)
def test_first_step_bit_exact(name):
    m = engine_or_skip()
    g = load(name)
    e = m.Engine(g["params"], g["pos0"], g["vel0"], g["type0"], precision=m.FP64)
    # state after loadInitialState: number density ratios (src/mps.cpp:106)
    s0 = e.state()
    if "s0_ndr" in g:
        assert np.array_equal(s0["ndr"], g["s0_ndr"])
    st = e.step(export=bool(g["meta"]["export_every"] == 1))
    ci, cj, cd = e.collisions()
    assert np.array_equal(ci, g["s1_coll_i"]) and np.array_equal(cj, g["s1_coll_j"])
    assert np.array_equal(cd, g["s1_coll_d"])
    s = e.state()
    if "s1_bc" in g:
        for k in ("bc", "type", "dirichlet"):
            assert np.array_equal(s[k], g[f"s1_{k}"]), k
        assert rel_l2(s["pressure"], g["s1_pressure"]) < P_TOL
        assert np.max(np.abs(s["pos"] - g["s1_pos"])) < X_TOL
        assert np.max(np.abs(s["vel"] - g["s1_vel"])) < V_TOL
    if "s1_nb_off" in g:
        off, ids, dist = e.neighbors()
        assert np.array_equal(off, g["s1_nb_off"])
        assert np.array_equal(ids, g["s1_nb_id"])
        assert np.array_equal(dist, g["s1_nb_dist"])
        src, rp, col, val = e.system()
        assert np.array_equal(src, g["s1_source"])
        assert np.array_equal(rp, g["s1_row_ptr"])
        assert np.array_equal(col, g["s1_col"])
        assert np.array_equal(val, g["s1_val"])
    assert st["status"] == 0


# MIXED step 1 against the FP64 goldens (see the test's docstring)
PM_TOL = 1e-6    # relative L2 of pressure: the mixed solve stops at relative residual 1e-10
XM_TOL = 1e-9    # metres: the FP32 pressure-gradient sum (relative error ~1e-7 of accelerations
                 # up to ~1e3 m/s^2 in the jittered scenes) moves particles by up to ~1e-10 m per step
VM_TOL = 1e-6    # m/s


@pytest.mark.parametrize("name", CASES)
def test_first_step_mixed_against_reference(name):
    """The MIXED step (FP32 viscosity and pressure-gradient sums, FP32
    Krylov iterations with FP64 refinement) on the reference's golden scenes.
    From rest the viscosity sum is exactly 0 in any precision (every
    v_j - v_i is 0), so the positions before the pressure part are the FP64
    step's and the pressure phase's neighbour lists (ids, order, FP64
    distances), collision pairs, surface and Dirichlet flags, source term and
    matrix equal the goldens bit for bit.  Scenes that start moving (the
    jittered ones, the 3-D box) carry the FP32 viscosity's rounding into their
    positions (at 12 m/s, ~1e-13 m after one step): there ids, order, flags
    and collision pairs are still exact, distances agree within 1e-10
    relative and matrix entries within 1e-9 of the largest.  Pressure,
    positions and velocities within PM_TOL, XM_TOL, VM_TOL."""
    m = engine_or_skip()
    g = load(name)
    at_rest = not np.any(g["vel0"])
    e = m.Engine(g["params"], g["pos0"], g["vel0"], g["type0"], precision=m.MIXED)
    st = e.step(export=bool(g["meta"]["export_every"] == 1))
    assert st["status"] == 0
    ci, cj, cd = e.collisions()
    assert np.array_equal(ci, g["s1_coll_i"]) and np.array_equal(cj, g["s1_coll_j"])
    if at_rest:
        assert np.array_equal(cd, g["s1_coll_d"])
    else:
        assert np.allclose(cd, g["s1_coll_d"], rtol=1e-10, atol=0)
    s = e.state()
    if "s1_bc" in g:
        for k in ("bc", "type", "dirichlet"):
            assert np.array_equal(s[k], g[f"s1_{k}"]), k
        assert rel_l2(s["pressure"], g["s1_pressure"]) < PM_TOL
        assert np.max(np.abs(s["pos"] - g["s1_pos"])) < XM_TOL
        assert np.max(np.abs(s["vel"] - g["s1_vel"])) < VM_TOL
    if "s1_nb_off" in g:
        off, ids, dist = e.neighbors()
        assert np.array_equal(off, g["s1_nb_off"])
        assert np.array_equal(ids, g["s1_nb_id"])
        src, rp, col, val = e.system()
        assert np.array_equal(rp, g["s1_row_ptr"]) and np.array_equal(col, g["s1_col"])
        if at_rest:
            assert np.array_equal(dist, g["s1_nb_dist"])
            assert np.array_equal(src, g["s1_source"])
            assert np.array_equal(val, g["s1_val"])
        else:
            assert np.allclose(dist, g["s1_nb_dist"], rtol=1e-10, atol=0)
            assert np.max(np.abs(val - g["s1_val"])) <= 1e-9 * np.max(np.abs(g["s1_val"]))
    e.close()


@pytest.mark.parametrize("name", CASES)
def test_trajectory_against_reference(name):
    m = engine_or_skip()
    g = load(name)
    meta = g["meta"]
    e = m.Engine(g["params"], g["pos0"], g["vel0"], g["type0"], precision=m.FP64)
    ex = meta["export_every"]
    for s in range(1, meta["steps"] + 1):
        st = e.step(export=bool(ex) and s % ex == 0)
        assert abs(st["courant"] - g["courant"][s]) <= 1e-9 * max(1.0, g["courant"][s])
        assert st["debug_log_count"] == g["debug_log_count"][s], s
        if s in meta["full_steps"]:
            r = e.state()
            for k in ("type", "bc", "dirichlet"):
                assert np.array_equal(r[k], g[f"s{s}_{k}"]), (s, k)
            assert rel_l2(r["pressure"], g[f"s{s}_pressure"]) < 1e-7, s
            # setMinimumPressure (src/mps.cpp:481-503) of those pressures
            assert rel_l2(r["min_pressure"], g[f"s{s}_min_pressure"]) < 1e-7, s
            assert np.max(np.abs(r["pos"] - g[f"s{s}_pos"])) < 1e-10, s
            assert np.max(np.abs(r["vel"] - g[f"s{s}_vel"])) < 1e-7, s
            assert rel_l2(r["ndr"], g[f"s{s}_ndr"]) < 1e-12, s
        ci, cj, _ = e.collisions()
        assert np.array_equal(ci, g[f"s{s}_coll_i"]) and np.array_equal(cj, g[f"s{s}_coll_j"]), s


@pytest.mark.parametrize("precision", ["FP64", "MIXED"])
def test_graph_replay_matches_eager(precision):
    """Non-export steps replayed as CUDA graphs give bit-identical states to
    the same steps launched kernel by kernel (collisions and ghosts included)."""
    m = engine_or_skip()
    g = load("jitter_collide")
    prec = getattr(m, precision)
    runs = []
    for graphs in (True, False):
        e = m.Engine(g["params"], g["pos0"], g["vel0"], g["type0"], precision=prec)
        e.set_graphs(graphs)
        flags = []
        for s in range(6):
            st = e.step(export=(s == 3))
            flags.append(st["graph_replayed"])
        runs.append((e.state(), flags))
        e.close()
    (a, fa), (b, fb) = runs
    assert fa == [1, 1, 1, 0, 1, 1] and fb == [0] * 6
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def test_fp64_step_at_config1_resolution_against_oracle():
    """The plain FP64 step at the 2M workload's particle distance and time
    step (l0 = 5e-4 m, dt = 5e-5 s, same tank walls and physics), on a small
    seeded crop of that scene (a 60 x 120 column), against the CPU oracle:
    bit-exact flags and collision pairs, pressure within the CG tolerance."""
    m = engine_or_skip()
    from oracle import Oracle

    from mps_gb300 import scenes

    l0 = 5e-4
    prm, pos, vel, t = scenes.dam_break(l0, tank=(0.06, 0.075), column=(0.03, 0.06), dt=5e-5,
                                        margin=0.005)
    rng = np.random.default_rng(12)
    fl = t == scenes.FLUID
    vel[fl, :2] = rng.normal(0.0, 0.02, (fl.sum(), 2))
    e = m.Engine(prm, pos, vel, t, precision=m.FP64)
    o = Oracle(prm, pos, vel, t)
    o.set_cg(solves=1)
    for s in range(5):
        st = e.step()
        so = o.step()
        assert st["debug_log_count"] == so["debug_log_count"], s
        ci, cj, _ = e.collisions()
        oi, oj, _ = o.collisions()
        assert np.array_equal(ci, oi) and np.array_equal(cj, oj), s
    a, b = e.state(), o.state()
    for k in ("type", "bc", "dirichlet"):
        assert np.array_equal(a[k], b[k]), k
    assert rel_l2(a["pressure"], b["pressure"]) < 1e-7
    assert np.max(np.abs(a["pos"] - b["pos"])) < 1e-12
    e.close()


def _sealed_box(l0, nf, origin, wall_layers=2, dummy_layers=2):
    """A fully packed nf x nf fluid block closed by walls and dummies on all
    four sides: none of its particles is Surface, so its component has no
    Dirichlet connection (src/mps.cpp:362-415 doubles its Inner diagonals)."""
    from mps_gb300 import scenes

    L = wall_layers + dummy_layers
    ix, iy = np.meshgrid(np.arange(-L, nf + L), np.arange(-L, nf + L), indexing="ij")
    ix, iy = ix.ravel(), iy.ravel()
    ring = np.maximum(np.maximum(-ix, ix - (nf - 1)), np.maximum(-iy, iy - (nf - 1)))
    t = np.where(ring <= 0, scenes.FLUID,
                 np.where(ring <= wall_layers, scenes.WALL, scenes.DUMMY)).astype(np.int32)
    pos = np.zeros((len(t), 3))
    pos[:, 0] = origin[0] + (ix + 0.5) * l0
    pos[:, 1] = origin[1] + (iy + 0.5) * l0
    return pos, np.zeros_like(pos), t


@pytest.mark.parametrize("box_n", [10, 60])
def test_unconnected_component_against_oracle(box_n):
    """A dam break beside a sealed, fully packed box (no Surface particle):
    the box's particles are unconnected.  At box_n = 10 the dam break is the
    largest component, at 60 the box is, so both sides of the sampled
    component search are covered.  Dirichlet flags, boundary flags and the
    unconnected count bit-exact, pressure within the CG tolerance."""
    m = engine_or_skip()
    from oracle import Oracle

    from mps_gb300 import scenes

    l0 = 0.01
    prm, pos, vel, t = scenes.dam_break(l0, tank=(0.3, 0.25), column=(0.1, 0.2), dt=1e-3,
                                        margin=0.05)
    bp, bv, bt = _sealed_box(l0, box_n, (0.5, 0.05))
    prm["domain_max"] = [0.5 + (box_n + 10) * l0, max(prm["domain_max"][1], 0.05 + (box_n + 10) * l0),
                         0.0]
    pos, vel, t = np.vstack([pos, bp]), np.vstack([vel, bv]), np.concatenate([t, bt])
    e = m.Engine(prm, pos, vel, t, precision=m.FP64)
    o = Oracle(prm, pos, vel, t)
    o.set_cg(solves=1)
    in_box = pos[:, 0] > 0.45
    for s in range(3):
        st = e.step()
        so = o.step()
        assert st["debug_log_count"] == so["debug_log_count"], s
        a, b = e.state(), o.state()
        for k in ("type", "bc", "dirichlet"):
            assert np.array_equal(a[k], b[k]), (s, k)
        assert not a["dirichlet"][in_box].any() and a["dirichlet"][~in_box & (t == scenes.FLUID)].all()
        assert rel_l2(a["pressure"], b["pressure"]) < 1e-7, s
    e.close()
