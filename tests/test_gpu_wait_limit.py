"""The device-side wait limits: a grid barrier that can never complete (one
block of its group never arrives) gives up in every block with the timeout
status instead of hanging, and the context stays usable afterwards.  The
failure is made on the host side of the wait (an arrival count nothing
completes); nothing faults."""
import pytest

from golden_cases import load
from gpu_util import engine_or_skip

pytestmark = pytest.mark.gpu


def test_barrier_wait_gives_up_and_context_survives():
    m = engine_or_skip()
    from mps_gb300.engine import selftest_wait_limit

    rc, gave_up, seconds = selftest_wait_limit()
    assert rc == 0 and gave_up == 8, (rc, gave_up)
    assert seconds < 10.0
    g = load("dambreak_l0_01")
    e = m.Engine(g["params"], g["pos0"], g["vel0"], g["type0"], precision=m.FP64)
    st = e.step()
    assert st["status"] == 0
    e.close()
