"""CPU-only checks: the C ABI library builds, loads and exports every entry
point its header declares; the C++ front end reads the reference's settings
format like the Python reader; scene generation and the CSV format."""
import ctypes
import json
import os
import re
import subprocess

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared(header):
    text = open(os.path.join(REPO, "include", header)).read()
    return sorted(set(re.findall(r"\b(mps_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def built():
    from mps_gb300 import build

    so = build.build_engine()
    exe = build.build_host()
    return so, exe


def test_library_exports_every_declared_symbol(built):
    so, _ = built
    lib = ctypes.CDLL(so)
    names = _declared("mps_gb300.h")
    assert "mps_create" in names and "mps_step" in names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", so], capture_output=True, text=True).stdout
    for n in names:
        assert re.search(rf"\bT {n}\b", out), n


def test_create_without_gpu_fails_loudly(built):
    """No silent CPU path: without a device the engine refuses to start."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from mps_gb300 import Engine, MpsError, scenes

    prm, pos, vel, t = scenes.dam_break(0.05, tank=(0.5, 0.4), column=(0.2, 0.2))
    with pytest.raises(MpsError):
        Engine(prm, pos, vel, t)


def _yaml(tmp_path, prm):
    import sys

    sys.path.insert(0, os.path.join(REPO, "tests", "golden"))
    from make_golden import yaml_text

    p = tmp_path / "settings.yml"
    p.write_text(yaml_text(prm, "input.csv"))
    return p


@pytest.mark.parametrize("variant", ["dambreak", "higher_order", "three_d"])
def test_cpp_settings_reader_matches_python(built, tmp_path, variant):
    from mps_gb300 import scenes
    from mps_gb300.settings import load_settings

    prm, *_ = scenes.dam_break(0.01)
    if variant == "higher_order":
        prm.update(higher_order_on=1, higher_order_gamma=1e-3, quasi_compressibility_on=0)
    if variant == "three_d":
        prm.update(dim=3, domain_min=[-0.1, -0.1, -0.2], domain_max=[1.1, 0.7, 0.2])
    path = _yaml(tmp_path, prm)
    _, exe = built
    out = subprocess.run([exe, "-s", str(path), "--check-settings"], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    c = json.loads(out.stdout)
    py = load_settings(str(path))
    for k in ("particle_distance", "dt", "re_pressure", "re_viscosity", "re_surface", "density",
              "kinematic_viscosity", "surface_threshold", "relaxation", "collision_distance",
              "restitution", "cfl", "compressibility", "higher_order_gamma"):
        assert c[k] == py[k], k
    assert c["dim"] == py["dim"]
    assert c["domain_min"] == py["domain_min"] and c["domain_max"] == py["domain_max"]
    assert c["gravity"] == py["gravity"]
    assert c["quasi_compressibility_on"] == py["quasi_compressibility_on"]
    assert c["higher_order_on"] == py["higher_order_on"]
    assert c["re_max"] == max(py["re_pressure"], py["re_viscosity"], py["re_surface"])


def test_cli_rejects_missing_settings(built, tmp_path):
    _, exe = built
    out = subprocess.run([exe, "-s", str(tmp_path / "nope.yml")], capture_output=True, text=True)
    assert out.returncode != 0 and "cannot be found" in out.stdout


def test_scene_counts_match_configurations():
    from mps_gb300 import scenes

    _, _, _, t = scenes.dam_break(0.01)
    assert (t == 0).sum() == 1250                       # 25 x 50 column
    _, _, _, t = scenes.dam_break(0.5 / 707, tank=(2.0, 1.2), column=(0.5, 1.0), dt=5e-5)
    assert (t == 0).sum() == 707 * 1414                 # 999,698
    _, _, _, t = scenes.hydrostatic(2.5e-3)
    assert (t == 0).sum() == 160 * 160                  # 25,600


def test_csv_round_trip(tmp_path):
    from mps_gb300 import scenes

    _, pos, vel, t = scenes.dam_break(0.02, tank=(0.4, 0.3), column=(0.1, 0.2))
    p = tmp_path / "in.csv"
    scenes.write_csv(p, pos, vel, t, time=0.25)
    t0, pos2, vel2, t2 = scenes.read_csv(p)
    assert t0 == 0.25 and np.array_equal(t2, t)
    assert np.allclose(pos2, pos, atol=5e-7) and np.allclose(vel2, vel, atol=5e-7)


def test_batch_scenes_are_seeded_and_in_range():
    from mps_gb300 import scenes

    a = scenes.batch_scenes(seed=0)
    b = scenes.batch_scenes(seed=0)
    assert len(a) == 64
    for (pa, xa, va, ta), (pb, xb, vb, tb) in zip(a, b):
        assert pa == pb and np.array_equal(xa, xb) and np.array_equal(ta, tb)
        nf = int((ta == scenes.FLUID).sum())
        assert 1900 <= nf <= 61000
        l0 = pa["particle_distance"]
        assert 1e-3 <= l0 <= 5e-3 and abs(pa["dt"] - 0.1 * l0) < 1e-15
        assert pa["re_pressure"] == 3.1 * l0 and pa["collision_distance"] == 0.5 * l0
    total = sum(int((t == scenes.FLUID).sum()) for _, _, _, t in a)
    assert 1.5e6 < total < 2.5e6


def test_wall_taps_sit_under_the_fluid():
    from mps_gb300 import scenes

    l0 = 2.5e-3
    prm, pos, vel, t = scenes.hydrostatic(l0, size=(0.4, 0.4))
    taps = scenes.wall_taps(pos, t, l0, 16)
    assert len(taps) == 16 and len(set(taps.tolist())) == 16
    assert np.all(t[taps] == scenes.WALL)
    assert np.allclose(pos[taps, 1], pos[t == scenes.FLUID, 1].min() - l0)
    assert np.all(np.diff(pos[taps, 0]) > 0)


def _reference_csv(s, time):
    """src/exporter.cpp:10-55 in Python: printf("%.6f") fields, Ghosts skipped."""
    out = [f"Time (s),{time:.6f}\n", f"Number of Particles,{len(s['type'])}\n",
           "ID,Type,Position.x (m),Position.y (m),Position.z (m),Velocity.x (m/s),Velocity.y (m/s),"
           "Velocity.z (m/s),Pressure (Pa),Number Density Ratio\n"]
    for i, t in enumerate(s["type"]):
        if t == -1:
            continue
        vals = list(s["pos"][i]) + list(s["vel"][i]) + [s["pressure"][i], s["ndr"][i]]
        out.append(f"{i},{t}," + ",".join("%.6f" % v for v in vals) + "\n")
    return "".join(out)


def _reference_vtu(s, time):
    """src/exporter.cpp:57-167 in Python: ostream default (printf "%g") fields."""
    g = lambda v: "%g" % v
    n = len(s["type"])
    arr = lambda c, ty, name: f"<DataArray NumberOfComponents='{c}' type='{ty}' Name='{name}' format='ascii'>\n"
    out = ["<?xml version='1.0' encoding='UTF-8'?>\n",
           "<VTKFile byte_order='LittleEndian' version='0.1' type = 'UnstructuredGrid'>\n",
           "<UnstructuredGrid>\n", "<FieldData>\n",
           "<DataArray type='Float64' Name='Time' NumberOfComponents='1' NumberOfTuples='1' format='ascii'>\n",
           g(time) + "\n", "</DataArray>\n", "</FieldData>\n",
           f"<Piece NumberOfCells='{n}' NumberOfPoints='{n}'>\n", "<Points>\n",
           "<DataArray NumberOfComponents='3' type='Float64' Name='position' format='ascii'>\n"]
    out += [" ".join(g(v) for v in p) + "\n" for p in s["pos"]]
    out += ["</DataArray>\n", "</Points>\n", "<PointData>\n", arr(1, "Int32", "Type")]
    out += [f"{t}\n" for t in s["type"]] + ["</DataArray>\n", arr(3, "Float64", "Velocity")]
    out += [f"{g(v[0])} {g(v[1])} 0\n" for v in s["vel"]] + ["</DataArray>\n", arr(1, "Float64", "Pressure")]
    out += [g(v) + "\n" for v in s["pressure"]] + ["</DataArray>\n", arr(1, "Float64", "Number Density Ratio")]
    out += [g(v) + "\n" for v in s["ndr"]] + ["</DataArray>\n", arr(1, "Int32", "Boundary Condition")]
    out += [f"{b}\n" for b in s["bc"]] + ["</DataArray>\n", "</PointData>\n", "<Cells>\n",
                                          "<DataArray type='Int32' Name='connectivity' format='ascii'>\n"]
    out += [f"{i}\n" for i in range(n)] + ["</DataArray>\n", "<DataArray type='Int32' Name='offsets' format='ascii'>\n"]
    out += [f"{i + 1}\n" for i in range(n)] + ["</DataArray>\n", "<DataArray type='UInt8' Name='types' format='ascii'>\n"]
    out += ["1\n"] * n + ["</DataArray>\n", "</Cells>\n", "</Piece>\n", "</UnstructuredGrid>\n", "</VTKFile>\n"]
    return "".join(out)


@pytest.mark.parametrize("n", [7, 70000])
def test_export_writers_match_reference_formats(built, tmp_path, n):
    """The engine's multithreaded CSV / VTU writers (to_chars) against the
    reference's printf / ostream formats, byte for byte, including negative
    zero, values that round to -0.000000, large and tiny magnitudes; 70,000
    particles take the multithreaded path."""
    from mps_gb300 import write_snapshot

    rng = np.random.default_rng(3)
    pos = rng.normal(0.0, 0.7, (n, 3))
    vel = rng.normal(0.0, 1e-3, (n, 3))
    pressure = rng.random(n) * 2e4
    ndr = rng.random(n) * 1.2
    edge = np.array([0.0, -0.0, -1e-9, 5e-7, -4.9999999e-7, 123456.789012345, 1e-5, 2.5, -0.125, 1e15])
    m = min(n, len(edge))
    pos[:m, 0] = edge[:m]
    vel[:m, 1] = edge[::-1][:m]
    pressure[:m] = edge[:m]
    types = rng.integers(-1, 3, n).astype(np.int32)
    bc = rng.integers(0, 3, n).astype(np.int32)
    s = dict(pos=pos, vel=vel, pressure=pressure, ndr=ndr, type=types, bc=bc)
    write_snapshot(s, tmp_path / "o.csv", tmp_path / "o.vtu", 0.0125)
    assert (tmp_path / "o.csv").read_text() == _reference_csv(s, 0.0125)
    assert (tmp_path / "o.vtu").read_text() == _reference_vtu(s, 0.0125)


def test_csv_reader_matches_python_parser(built, tmp_path):
    """mps_read_csv (parallel, from_chars) against the Python reader on a
    scene written in the reference's CSV format, with CRLF line ends and an
    empty line; a bad ID is reported."""
    from mps_gb300 import read_particles_csv, scenes

    prm, pos, vel, t = scenes.dam_break(1 / 640, tank=(1.0, 0.6), column=(0.5, 0.5))
    rng = np.random.default_rng(5)
    vel[:, :2] = rng.normal(0.0, 0.3, (len(t), 2))
    path = tmp_path / "in.csv"
    scenes.write_csv(path, pos, vel, t, time=0.25)
    assert len(t) > 65536  # the multithreaded path
    tm, p2, v2, t2 = read_particles_csv(path)
    tm0, p0, v0, t0 = scenes.read_csv(path)
    assert tm == tm0 == 0.25
    assert np.array_equal(p2, p0) and np.array_equal(v2, v0) and np.array_equal(t2, t0)
    lines = path.read_text().splitlines()
    crlf = tmp_path / "crlf.csv"
    crlf.write_bytes(("\r\n".join(lines[:10] + [""] + lines[10:]) + "\r\n").encode())
    tm, p3, v3, t3 = read_particles_csv(crlf)
    assert np.array_equal(p3, p0) and np.array_equal(t3, t0)
    bad = tmp_path / "bad.csv"
    bad.write_text("\n".join(lines[:5] + [lines[6]] + lines[6:]) + "\n")
    with pytest.raises(Exception, match="bad row"):
        read_particles_csv(bad)


def _no_gpu_or_skip():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present: these calls pass unchecked host pointers")


@pytest.mark.parametrize("domain", ["inverted_x", "inverted_y_by_one_cell", "nan", "inf"])
def test_bad_domain_rejected_before_the_gpu(built, domain):
    """A domain that is not finite or whose max lies below its min on an axis
    would give the bucket grid fewer than 3 cells on that axis (or undefined
    integer casts); mps_create and mps_number_density_static refuse it with
    MPS_ERR_ARG before any device call, so here (no GPU) the code is ARG, not
    NO_DEVICE."""
    _no_gpu_or_skip()
    import ctypes as C

    from mps_gb300 import engine, scenes

    prm, pos, vel, t = scenes.dam_break(0.05, tank=(0.5, 0.4), column=(0.2, 0.2))
    lo, hi = list(prm["domain_min"]), list(prm["domain_max"])
    re = max(prm["re_pressure"], prm["re_viscosity"], prm["re_surface"])
    if domain == "inverted_x":
        lo[0], hi[0] = hi[0], lo[0]
    elif domain == "inverted_y_by_one_cell":
        hi[1] = lo[1] - 1.5 * re
    elif domain == "nan":
        lo[0] = float("nan")
    else:
        hi[1] = float("inf")
    bad = dict(prm, domain_min=lo, domain_max=hi)
    with pytest.raises(engine.MpsError) as ex:
        engine.Engine(bad, pos, vel, t)
    assert ex.value.code == engine.MPS_ERR_ARG and "domain" in str(ex.value)
    lib = engine.load()
    fn = lib.mps_number_density_static
    fn.argtypes = [C.POINTER(engine.MpsParams), C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p,
                   C.c_void_p]
    fn.restype = C.c_int
    # non-null placeholders: the call must return before it would use them
    rc = fn(C.byref(engine.make_params(bad)), 10, 16, 16, 16, None)
    assert rc == engine.MPS_ERR_ARG and b"domain" in lib.mps_last_error()


def test_check_symmetry_rejects_bad_csr_on_the_host(built):
    """mps_check_symmetry validates a host CSR before it copies anything to
    the device: a decreasing row_ptr or an out-of-range column is MPS_ERR_ARG
    (so on this GPU-less machine no CUDA error can occur first)."""
    _no_gpu_or_skip()
    from mps_gb300 import engine

    rc, *_ = engine.check_symmetry([0, 2, 1], [0, 1], [1.0, 2.0])
    assert rc == engine.MPS_ERR_ARG
    rc, *_ = engine.check_symmetry([0, 1, 2], [0, 2], [1.0, 2.0])
    assert rc == engine.MPS_ERR_ARG
    rc, *_ = engine.check_symmetry([0, 1, 2], [0, -1], [1.0, 2.0])
    assert rc == engine.MPS_ERR_ARG
