"""Asynchronous export (mps_export_begin / view / write): the snapshot taken at
an export step equals the state downloaded synchronously at that step, while
the following steps run before the snapshot is read, and the files written
from it equal the writers' output for that state."""
import threading

import numpy as np
import pytest

from golden_cases import load
from gpu_util import engine_or_skip

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["FP64", "MIXED"])
def test_snapshot_survives_the_following_steps(precision, tmp_path):
    m = engine_or_skip()
    from mps_gb300 import write_snapshot

    g = load("jitter_collide")
    e = m.Engine(g["params"], g["pos0"], g["vel0"], g["type0"], precision=getattr(m, precision))
    for _ in range(2):
        e.step()
    e.step(export=True)
    ref = e.state()
    e.export_begin()
    writer = threading.Thread(target=e.export_write,
                              args=(tmp_path / "a.csv", tmp_path / "a.vtu", 0.003))
    writer.start()
    for _ in range(3):  # these steps change every array the snapshot holds
        e.step()
    writer.join()
    snap = e.export_snapshot()
    for k in ("pos", "vel", "pressure", "ndr", "type", "bc"):
        assert np.array_equal(snap[k], ref[k]), k
    assert not np.array_equal(e.state()["pos"], ref["pos"])
    write_snapshot(ref, tmp_path / "b.csv", tmp_path / "b.vtu", 0.003)
    assert (tmp_path / "a.csv").read_bytes() == (tmp_path / "b.csv").read_bytes()
    assert (tmp_path / "a.vtu").read_bytes() == (tmp_path / "b.vtu").read_bytes()
    # a second snapshot replaces the first
    e.export_begin()
    assert np.array_equal(e.export_snapshot()["pos"], e.state()["pos"])
    e.close()
