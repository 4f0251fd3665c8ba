"""The collision pass's parallel application (each candidate pair applied
after exactly the earlier pairs that touch its particles) against the
serial application in the reference's order (src/mps.cpp:217-250): the same
state bit for bit, on the golden jittered scene and on a shaken dam-break
column with thousands of candidate pairs per step."""
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
    """A 200 x 200 dam-break column shaken (positions +-0.4 l0, velocities
    N(0, 0.1) m/s): thousands of candidate pairs in the first steps, at most a
    few per particle, so the parallel pass (not its serial fallback) runs."""
    m = engine_or_skip()
    from mps_gb300 import scenes

    l0 = 2.5e-3
    scene = scenes.shaken(scenes.dam_break(l0, tank=(1.0, 0.8), column=(0.5, 0.5), dt=2.5e-4))
    most, per_partner = _compare(m, *scene, 4, m.FP64)
    assert most > 2000, most
    assert 0 < per_partner <= 8, per_partner
