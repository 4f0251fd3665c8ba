"""mps_number_density_static: the number-density pass for callers that cannot
allocate device memory (an application that owns all device memory itself, or
a timing-critical loop that cannot take an allocation's synchronisation).

The entry point works in a fixed static scratch array inside the library; the
caller passes device buffers for the inputs and the output.  Its result must
equal what the allocating entry point (mps_create, which computes the same
ratios for loadInitialState) produces, bit for bit, on two calls in a row (the
second call reuses the scratch the first one left behind).  This file is
named to run after every other test file.
"""
import ctypes as C

import numpy as np
import pytest

from gpu_util import engine_or_skip

pytestmark = pytest.mark.gpu


def _entry():
    from mps_gb300 import engine

    lib = engine.load(build_if_missing=True)
    fn = lib.mps_number_density_static
    fn.argtypes = [C.POINTER(engine.MpsParams), C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p,
                   C.c_void_p]
    fn.restype = C.c_int
    return engine, fn


@pytest.mark.parametrize("scene", ["dambreak", "jittered_with_ghosts", "box3d", "outside_domain"])
def test_static_scratch_number_density_matches_create(scene):
    """Planar scenes (which mps_create sweeps with its planar cell keys while
    this entry point always uses the 3-D key), a 3-D box, and particles placed
    outside the domain (their cell coordinates clamped to the grid)."""
    m = engine_or_skip()
    import torch

    from mps_gb300 import scenes

    engine, fn = _entry()
    prm, pos, vel, t = scenes.dam_break(0.01, tank=(0.6, 0.4), column=(0.2, 0.3))
    if scene == "jittered_with_ghosts":
        rng = np.random.default_rng(3)
        fl = t == scenes.FLUID
        pos[fl, :2] += rng.uniform(-0.3, 0.3, (fl.sum(), 2)) * 0.01
        t[np.flatnonzero(fl)[::17]] = scenes.GHOST
    elif scene == "box3d":
        from golden_cases import load

        g = load("box3d")
        prm, pos, vel, t = g["params"], g["pos0"].copy(), g["vel0"].copy(), g["type0"].copy()
        assert prm["dim"] == 3 and len(t) < 65536
    elif scene == "outside_domain":
        fl = np.flatnonzero(t == scenes.FLUID)
        lo, hi = prm["domain_min"], prm["domain_max"]
        pos[fl[0], 0] = lo[0] - 0.05        # left of the grid
        pos[fl[1], 1] = hi[1] + 0.2         # above it
        pos[fl[2], :2] = [hi[0] + 1.0, lo[1] - 1.0]
        pos[fl[3], 0] = pos[fl[2], 0] + 0.005  # a neighbour out there too
        pos[fl[3], 1] = pos[fl[2], 1]
    # the allocating path: mps_create computes the initial number density ratios
    eng = m.Engine(prm, pos, vel, t)
    want = eng.state()["ndr"]
    eng.close()

    dev = torch.device("cuda:0")
    d_pos = torch.tensor(np.ascontiguousarray(pos), dtype=torch.float64, device=dev)
    d_type = torch.tensor(np.ascontiguousarray(t, np.int32), dtype=torch.int32, device=dev)
    d_ndr = torch.full((len(t),), float("nan"), dtype=torch.float64, device=dev)
    prm_c = engine.make_params(prm)
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        d_ndr.fill_(-1.0)
        rc = fn(C.byref(prm_c), len(t), d_pos.data_ptr(), d_type.data_ptr(), d_ndr.data_ptr(),
                stream)
        assert rc == 0, engine.load().mps_last_error().decode()
        torch.cuda.synchronize()
        got = d_ndr.cpu().numpy()
        assert np.array_equal(got, want), f"call {call}: max diff {np.nanmax(np.abs(got - want))}"


def test_static_scratch_rejects_oversize_requests():
    engine_or_skip()
    import torch

    from mps_gb300 import scenes

    engine, fn = _entry()
    prm, *_ = scenes.dam_break(0.01)
    prm_c = engine.make_params(prm)
    dev = torch.device("cuda:0")
    buf = torch.zeros(3, dtype=torch.float64, device=dev)
    rc = fn(C.byref(prm_c), 1 << 17, buf.data_ptr(), buf.data_ptr(), buf.data_ptr(), None)
    assert rc == engine.MPS_ERR_ARG
    assert "exceed" in engine.load().mps_last_error().decode()
    big = dict(prm, domain_min=[-10.0, -10.0, 0.0], domain_max=[10.0, 10.0, 0.0])
    rc = fn(C.byref(engine.make_params(big)), 10, buf.data_ptr(), buf.data_ptr(), buf.data_ptr(),
            None)
    assert rc == engine.MPS_ERR_ARG
    assert "cells" in engine.load().mps_last_error().decode()


def test_static_scratch_rejects_a_bad_domain():
    """An inverted or non-finite domain is refused before any launch (it
    would give an axis fewer than the 3 cells the clamped sweep needs)."""
    engine_or_skip()
    import torch

    from mps_gb300 import scenes

    engine, fn = _entry()
    prm, *_ = scenes.dam_break(0.01)
    buf = torch.zeros(30, dtype=torch.float64, device=torch.device("cuda:0"))
    for lo, hi in (([0.5, -0.1, 0.0], [-0.1, 0.7, 0.0]), ([float("nan"), -0.1, 0.0], [1.1, 0.7, 0.0])):
        bad = dict(prm, domain_min=lo, domain_max=hi)
        rc = fn(C.byref(engine.make_params(bad)), 10, buf.data_ptr(), buf.data_ptr(), buf.data_ptr(), None)
        assert rc == engine.MPS_ERR_ARG
        assert "domain" in engine.load().mps_last_error().decode()
