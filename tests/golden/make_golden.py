"""Generate the golden fixtures in tests/golden/*.npz from the reference itself.

Runs ONLY in a container that has the reference sources at REF_ROOT: it builds
oracle/_ref/ref_driver (the reference's src/mps.cpp, bucket.cpp, particle.cpp
and settings.cpp compiled in place with the stand-in headers of
oracle/ref_shim/), drives the reference's MPS class over a set of scenes and
stores what it computed.  The scenes are produced by mps_gb300.scenes, whose
lattice generator reproduces the reference's own inputs/*/input.csv byte for
byte (checked below before anything is written).

    python tests/golden/make_golden.py REF_ROOT

Each fixture holds the initial condition, the settings, and per step either
the full per-particle arrays or SHA-256 digests of them (for the larger
scenes), the neighbour lists / source term / PPE matrix at selected steps,
and the collision candidate pairs (i, j, distance) that the reference's
collision pass (src/mps.cpp:217-250) sees, taken from its neighbour lists.
"""
from __future__ import annotations

import hashlib
import json
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, HERE)

from mps_gb300 import scenes  # noqa: E402
from mps_gb300.settings import load_settings  # noqa: E402
from refdump import read_dump  # noqa: E402

STATE_KEYS = ("pos", "vel", "pressure", "min_pressure", "ndr", "type", "bc", "dirichlet")
NB_KEYS = ("nb_off", "nb_id", "nb_dist")
SYS_KEYS = ("source", "row_ptr", "col", "val")


def digest(arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def yaml_text(p: dict, csv_name: str) -> str:
    """settings.yml in the reference's layout (tutorials/dambreak/settings.yml)."""
    l0 = p["particle_distance"]
    f = lambda v: repr(float(v))  # noqa: E731  (always carries a decimal point)
    lines = [
        f"dim: {int(p['dim'])}", f"particle distance: {f(l0)}", f"dt: {f(p['dt'])}",
        "finish time: 1.0", "output interval: 1.0", f"CFL condition: {f(p['cfl'])}",
        f"domain range X: [{f(p['domain_min'][0])}, {f(p['domain_max'][0])}]",
        f"domain range Y: [{f(p['domain_min'][1])}, {f(p['domain_max'][1])}]",
        f"domain range Z: [{f(p['domain_min'][2])}, {f(p['domain_max'][2])}]",
        f"density: {f(p['density'])}", f"kinematic viscosity: {f(p['kinematic_viscosity'])}",
        f"gravity: [{', '.join(f(g) for g in p['gravity'])}]",
        "effective radius ratio:",
        f"  pressure: {f(p['re_pressure'] / l0)}",
        f"  viscosity: {f(p['re_viscosity'] / l0)}",
        f"  surface detection: {f(p['re_surface'] / l0)}",
        f"threshold for surface detection: {f(p['surface_threshold'])}",
        "pressure stabilization:", "  quasi compressibility:",
        f"    on: {'True' if p['quasi_compressibility_on'] else 'False'}",
        f"    compressibility: {f(p['compressibility'])}", "  higher order source term:",
        f"    on: {'True' if p['higher_order_on'] else 'False'}",
        f"    gamma: {f(p['higher_order_gamma'])}",
        f"relaxation coefficient for pressure: {f(p['relaxation'])}",
        f"collision distance ratio: {f(p['collision_distance'] / l0)}",
        f"coefficient of restitution: {f(p['restitution'])}",
        f"inputCsvPath: {csv_name}",
    ]
    return "\n".join(lines) + "\n"


def collision_candidates(d: dict, cd: float):
    """Pairs the reference's collision loop tests (src/mps.cpp:217-229), in its order."""
    out_i, out_j, out_d = [], [], []
    t = d["type"]
    for i in range(len(t)):
        if t[i] != scenes.FLUID:
            continue
        for k in range(d["nb_off"][i], d["nb_off"][i + 1]):
            j = int(d["nb_id"][k])
            if t[j] == scenes.FLUID and j >= i:
                continue
            if d["nb_dist"][k] < cd:
                out_i.append(i)
                out_j.append(j)
                out_d.append(d["nb_dist"][k])
    return np.array(out_i, np.int32), np.array(out_j, np.int32), np.array(out_d)


def run_case(driver, name, params, pos, vel, types, steps, export_every=0, full_steps=(),
             nb_steps=(), yaml_override=None):
    tmp = tempfile.mkdtemp(prefix=f"golden_{name}_")
    try:
        scenes.write_csv(os.path.join(tmp, "input.csv"), pos, vel, types)
        text = yaml_override if yaml_override is not None else yaml_text(params, "input.csv")
        with open(os.path.join(tmp, "settings.yml"), "w") as fh:
            fh.write(text)
        prm = load_settings(os.path.join(tmp, "settings.yml"))
        _, pos_in, vel_in, types_in = scenes.read_csv(os.path.join(tmp, "input.csv"))
        out = os.path.join(tmp, "dump")
        subprocess.run([driver, "settings.yml", str(steps), out, str(export_every), "phases"],
                       cwd=tmp, check=True)
        fx = {"pos0": pos_in, "vel0": vel_in, "type0": types_in}
        prm_json = {k: v for k, v in prm.items() if k != "input_csv"}
        fx["params_json"] = np.array(json.dumps(prm_json))
        fx["meta"] = np.array(json.dumps({"steps": steps, "export_every": export_every,
                                          "full_steps": list(full_steps),
                                          "nb_steps": list(nb_steps)}))
        courant, dlc, hs, hn, hsys = [], [], [], [], []
        for s in range(steps + 1):
            d = read_dump(os.path.join(out, f"step_{s:04d}.bin"))
            courant.append(d["courant"])
            dlc.append(d["debug_log_count"])
            hs.append(digest([d[k] for k in STATE_KEYS]))
            hn.append(digest([d[k] for k in NB_KEYS]))
            hsys.append(digest([d[k] for k in SYS_KEYS]))
            if s in full_steps:
                for k in STATE_KEYS:
                    fx[f"s{s}_{k}"] = d[k]
            if s in nb_steps:
                for k in NB_KEYS + SYS_KEYS:
                    fx[f"s{s}_{k}"] = d[k]
            if s >= 1:
                c = read_dump(os.path.join(out, f"collide_{s:04d}.bin"))
                ci, cj, cdist = collision_candidates(c, prm["collision_distance"])
                fx[f"s{s}_coll_i"], fx[f"s{s}_coll_j"], fx[f"s{s}_coll_d"] = ci, cj, cdist
        fx["courant"] = np.array(courant)
        fx["debug_log_count"] = np.array(dlc, np.int64)
        fx["hash_state"] = np.array(hs)
        fx["hash_nb"] = np.array(hn)
        fx["hash_sys"] = np.array(hsys)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **fx)
        ncoll = sum(len(fx[f"s{s}_coll_i"]) for s in range(1, steps + 1))
        print(f"{name}: n={len(types_in)} steps={steps} collisions={ncoll} "
              f"ghosts={int((read_dump(os.path.join(out, f'step_{steps:04d}.bin'))['type'] < 0).sum())}")
    finally:
        shutil.rmtree(tmp, ignore_errors=True)


def jittered(seed, l0=0.01, vel_scale=0.6, jitter=0.3):
    """Dam-break lattice shaken to force collisions, surface flags and ghosts."""
    rng = np.random.default_rng(seed)
    prm, pos, vel, t = scenes.dam_break(l0, tank=(0.3, 0.25), column=(0.12, 0.2), dt=2e-3,
                                        wall_layers=1, dummy_layers=2, margin=0.05)
    fl = t == scenes.FLUID
    pos[fl, :2] += rng.uniform(-jitter, jitter, (fl.sum(), 2)) * l0
    vel[fl, :2] = rng.normal(0.0, vel_scale, (fl.sum(), 2))
    # a few fluid particles shot towards the domain edges to become ghosts
    idx = np.flatnonzero(fl)[:: max(1, fl.sum() // 6)]
    vel[idx, 0] = -12.0
    prm["gravity"] = [0.0, -9.81, 0.0]
    return prm, pos, vel, t


def box3d(l0=0.02, nf=5):
    """Small 3-D cube of fluid on a wall/dummy floor, jittered (exercises the z path)."""
    rng = np.random.default_rng(7)
    pts, ty = [], []
    for ix in range(-3, nf + 3):
        for iy in range(-3, nf + 3):
            for iz in range(-3, nf + 3):
                inside = 0 <= ix < nf and 0 <= iy < nf and 0 <= iz < nf
                if inside:
                    ty.append(scenes.FLUID)
                elif iy < 0 and -3 <= ix < nf + 3 and -3 <= iz < nf + 3:
                    ty.append(scenes.WALL if iy == -1 else scenes.DUMMY)
                else:
                    continue
                pts.append(((ix + 0.5) * l0, (iy + 0.5) * l0, (iz + 0.5) * l0))
    pos = np.array(pts)
    t = np.array(ty, np.int32)
    fl = t == scenes.FLUID
    pos[fl] += rng.uniform(-0.2, 0.2, (fl.sum(), 3)) * l0
    vel = np.zeros_like(pos)
    vel[fl] = rng.normal(0, 0.3, (fl.sum(), 3))
    prm = scenes.baseline_physics(l0, 2e-3, (-0.1, -0.1, -0.1), (0.2, 0.25, 0.2))
    prm["dim"] = 3
    prm["re_surface"] = 2.1 * l0
    return prm, pos, vel, t


def main():
    if len(sys.argv) < 2:
        raise SystemExit("usage: python tests/golden/make_golden.py REF_ROOT (the reference checkout)")
    ref_root = sys.argv[1]
    src = os.path.join(ref_root, "src")
    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "ref", f"REF_SRC={src}"],
                   check=True)
    driver = os.path.join(REPO, "oracle", "_ref", "ref_driver")

    # The generator must reproduce the reference's own inputs before anything else.
    gen = {"dambreak": (0.01, (0, 0.3), (0, 0.25), (0, 0.1), (0, 0.2)),
           "dambreak_fine": (0.004, (0, 1.0), (0, 0.25), (0, 0.4), (0, 0.2)),
           "hydrostatic": (0.005, (0, 0.2), (0, 0.35), (0, 0.2), (0, 0.3))}
    made = {}
    for k, (l0, tx, ty, fx_, fy) in gen.items():
        pos, vel, t = scenes.tank_scene(l0, tx, ty, fx_, fy, 1, 2)
        path = os.path.join(tempfile.gettempdir(), f"gen_{k}.csv")
        scenes.write_csv(path, pos, vel, t)
        with open(path) as a, open(os.path.join(ref_root, "inputs", k, "input.csv")) as b:
            if a.read() != b.read():
                raise SystemExit(f"scene generator does not reproduce inputs/{k}/input.csv")
        made[k] = (pos, vel, t)

    def tutorial_yaml(rel):
        with open(os.path.join(ref_root, rel)) as fh:
            lines = fh.read().splitlines()
        return "\n".join("inputCsvPath: input.csv" if ln.startswith("inputCsvPath") else ln
                         for ln in lines) + "\n"

    run_case(driver, "ref_dambreak", None, *made["dambreak"], steps=20, export_every=10,
             full_steps=range(0, 21), nb_steps=(1, 20),
             yaml_override=tutorial_yaml("tutorials/dambreak/settings.yml"))
    run_case(driver, "ref_hydrostatic_original", None, *made["hydrostatic"], steps=5,
             full_steps=(5,), nb_steps=(5,),
             yaml_override=tutorial_yaml(
                 "tutorials/pressure_stabilization/01_original/hydrostatic/settings.yml"))
    run_case(driver, "ref_dambreak_fine", None, *made["dambreak_fine"], steps=3,
             full_steps=(3,), yaml_override=tutorial_yaml("tutorials/dambreak_fine/settings.yml"))

    prm, pos, vel, t = scenes.dam_break(0.01)
    run_case(driver, "dambreak_l0_01", prm, pos, vel, t, steps=10, export_every=5,
             full_steps=(5, 10), nb_steps=(10,))
    prm, pos, vel, t = jittered(1)
    run_case(driver, "jitter_collide", prm, pos, vel, t, steps=6, export_every=3,
             full_steps=range(0, 7), nb_steps=(1, 6))
    prm, pos, vel, t = jittered(2)
    prm.update(higher_order_on=1, higher_order_gamma=1e-3, quasi_compressibility_on=0,
               relaxation=1.0)
    run_case(driver, "jitter_higher_order", prm, pos, vel, t, steps=4,
             full_steps=range(0, 5), nb_steps=(4,))
    prm, pos, vel, t = box3d()
    run_case(driver, "box3d", prm, pos, vel, t, steps=3, full_steps=range(0, 4), nb_steps=(3,))


if __name__ == "__main__":
    main()
