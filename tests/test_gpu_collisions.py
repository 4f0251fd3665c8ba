"""The collision pass's parallel application (each candidate pair applied
after exactly the earlier pairs that touch its particles) against the
serial application in the reference's order (src/mps.cpp:217-250): the same
state bit for bit, on the golden jittered scene and on a hydrostatic tank
run at a time step where it has thousands of candidate pairs per step."""
import numpy as np
import pytest

from golden_cases import load
from gpu_util import engine_or_skip

pytestmark = pytest.mark.gpu


def _pairs_per_partner(e, types):
    ci, cj, _ = e.collisions()
    fl = types[cj] == 0
    return 0 if not fl.any() else int(np.bincount(cj[fl]).max())


def _compare(m, prm, pos, vel, t, steps, prec):
    a = m.Engine(prm, pos, vel, t, precision=prec)
    b = m.Engine(prm, pos, vel, t, precision=prec)
    b.set_collisions(serial=True)
    most, most_per_partner = 0, 0
    for s in range(steps):
        sa, sb = a.step(), b.step()
        assert sa["n_collision_candidates"] == sb["n_collision_candidates"], s
        ra, rb = a.state(), b.state()
        for k in ra:
            assert np.array_equal(ra[k], rb[k]), (s, k)
        if sa["n_collision_candidates"] > most:
            most = sa["n_collision_candidates"]
            most_per_partner = _pairs_per_partner(a, ra["type"])
    a.close()
    b.close()
    return most, most_per_partner


@pytest.mark.parametrize("precision", ["FP64", "MIXED"])
def test_parallel_collisions_match_serial_on_golden_scene(precision):
    m = engine_or_skip()
    g = load("jitter_collide")
    most, _ = _compare(m, g["params"], g["pos0"], g["vel0"], g["type0"], 6, getattr(m, precision))
    assert most > 0


def test_parallel_collisions_match_serial_with_thousands_of_pairs():
    """The 25,600-particle hydrostatic tank at dt = 1e-3 s (4x the stable
    dt / l0): within a few steps thousands of pairs collide every step."""
    m = engine_or_skip()
    from mps_gb300 import scenes

    l0 = 2.5e-3
    prm, pos, vel, t = scenes.hydrostatic(l0, size=(0.4, 0.4), dt=1e-3)
    rng = np.random.default_rng(0)
    fl = t == scenes.FLUID
    vel[fl, :2] = rng.normal(0.0, 0.01, (fl.sum(), 2))
    most, per_partner = _compare(m, prm, pos, vel, t, 12, m.FP64)
    assert most > 2000, most
    print(f"candidates {most}, most pairs with one partner {per_partner}")
