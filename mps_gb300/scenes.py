"""Lattice scene generation and the reference's CSV particle format.

`tank_scene` restates the reference's scene generators
(iori3150/MPS inputs/dambreak/main.cpp:26-80, with the parameters of
inputs/dambreak_fine and inputs/hydrostatic as special cases): particles on
the square lattice ((ix + 0.5) l0, (iy + 0.5) l0), classified as dummy wall,
wall or fluid with the same eps = 0.01 l0 inclusion test, emitted ix-major
so that a particle's id is its array index.

`write_csv` / `read_csv` follow Exporter::toCsv (src/exporter.cpp:10-55,
six-decimal fixed notation, Ghost particles skipped) and
MPS::importInitialCondition (src/mps.cpp:38-94).
"""
from __future__ import annotations

import math

import numpy as np

GHOST, FLUID, WALL, DUMMY = -1, 0, 1, 2


def _c_round(v: float) -> int:
    """C's round(): half away from zero."""
    return int(math.floor(v + 0.5)) if v >= 0 else -int(math.floor(-v + 0.5))


def _inside(x, y, xr, yr, eps):
    xr = sorted(xr)
    yr = sorted(yr)
    return (xr[0] - eps < x) & (x < xr[1] + eps) & (yr[0] - eps < y) & (y < yr[1] + eps)


def tank_scene(l0, tank_x, tank_y, fluid_x, fluid_y, wall_layers=1, dummy_layers=2,
               density=1000.0):
    """Open-top tank with walls and a rectangular water column.

    tank_x/tank_y and fluid_x/fluid_y are (min, max) ranges in metres.  Returns
    (pos[n,3], vel[n,3], type[n]) in the generator's id order.
    """
    eps = 0.01 * l0
    for r in (fluid_x, fluid_y):
        nrm = (max(r) - min(r)) / l0
        if abs(nrm - round(nrm)) > eps:
            raise ValueError("fluid range is not divisible by the particle distance")
    all_layers = dummy_layers + wall_layers
    ix0 = _c_round(tank_x[0] / l0) - all_layers
    ix1 = _c_round(tank_x[1] / l0) + all_layers
    iy0 = _c_round(tank_y[0] / l0) - all_layers
    iy1 = _c_round(tank_y[1] / l0) + all_layers
    ix, iy = np.meshgrid(np.arange(ix0, ix1 + 1), np.arange(iy0, iy1 + 1), indexing="ij")
    x = (ix.ravel() + 0.5) * l0
    y = (iy.ravel() + 0.5) * l0
    xmax, ymax = tank_x[1], tank_y[1]
    t = np.full(x.shape, GHOST, np.int32)
    t[_inside(x, y, (-all_layers * l0, xmax + all_layers * l0), (-all_layers * l0, ymax), eps)] = DUMMY
    t[_inside(x, y, (-wall_layers * l0, xmax + wall_layers * l0), (-wall_layers * l0, ymax), eps)] = WALL
    t[_inside(x, y, (0.0, xmax), (0.0, ymax), eps)] = GHOST
    t[_inside(x, y, fluid_x, fluid_y, eps)] = FLUID
    keep = t != GHOST
    n = int(keep.sum())
    pos = np.zeros((n, 3))
    pos[:, 0] = x[keep]
    pos[:, 1] = y[keep]
    return pos, np.zeros((n, 3)), t[keep].copy()


def write_csv(path, pos, vel, types, pressure=None, ndr=None, time=0.0):
    """Exporter::toCsv format (src/exporter.cpp:10-55)."""
    n = len(types)
    pressure = np.zeros(n) if pressure is None else pressure
    ndr = np.zeros(n) if ndr is None else ndr
    lines = [f"Time (s),{time:.6f}", f"Number of Particles,{n}",
             "ID,Type,Position.x (m),Position.y (m),Position.z (m),Velocity.x (m/s),"
             "Velocity.y (m/s),Velocity.z (m/s),Pressure (Pa),Number Density Ratio"]
    for i in range(n):
        if types[i] == GHOST:
            continue
        lines.append(f"{i},{int(types[i])},{pos[i,0]:.6f},{pos[i,1]:.6f},{pos[i,2]:.6f},"
                     f"{vel[i,0]:.6f},{vel[i,1]:.6f},{vel[i,2]:.6f},{pressure[i]:.6f},{ndr[i]:.6f}")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def read_csv(path):
    """MPS::importInitialCondition (src/mps.cpp:38-94): returns time, pos, vel, type."""
    with open(path) as f:
        rows = [ln.rstrip("\r\n") for ln in f if ln.strip()]
    time = float(rows[0].split(",")[1])
    head = rows[2].split(",")
    col = {h: k for k, h in enumerate(head)}
    data = [r.split(",") for r in rows[3:]]
    n = len(data)
    pos = np.zeros((n, 3))
    vel = np.zeros((n, 3))
    types = np.zeros(n, np.int32)
    for k, r in enumerate(data):
        if int(r[col["ID"]]) != k:
            raise ValueError("particle ids must equal their row index")
        types[k] = int(r[col["Type"]])
        pos[k] = [float(r[col[c]]) for c in ("Position.x (m)", "Position.y (m)", "Position.z (m)")]
        vel[k] = [float(r[col[c]]) for c in ("Velocity.x (m/s)", "Velocity.y (m/s)", "Velocity.z (m/s)")]
    return time, pos, vel, types


def baseline_physics(l0, dt, domain_min, domain_max, re_surface_ratio=2.1):
    """Physics shared by the dam-break/hydrostatic workloads: rho 1000, nu 1e-6,
    g (0, -9.81), radii 3.1/3.1/2.1 l0, beta 0.97, alpha 0.45e-9, gamma 0.2,
    collision 0.5 l0, restitution 0.2."""
    return dict(dim=2, particle_distance=l0, dt=dt, domain_min=list(domain_min),
                domain_max=list(domain_max), density=1000.0, kinematic_viscosity=1e-6,
                gravity=[0.0, -9.81, 0.0], re_pressure=3.1 * l0, re_viscosity=3.1 * l0,
                re_surface=re_surface_ratio * l0, surface_threshold=0.97,
                quasi_compressibility_on=1, compressibility=0.45e-9, higher_order_on=0,
                higher_order_gamma=1e-3, relaxation=0.2, collision_distance=0.5 * l0,
                restitution=0.2, cfl=0.3)


def dam_break(l0, tank=(1.0, 0.6), column=(0.25, 0.5), dt=1e-3, wall_layers=2, dummy_layers=2,
              margin=0.1):
    """Dam-break workload: water column in the left corner of an open tank."""
    pos, vel, t = tank_scene(l0, (0.0, tank[0]), (0.0, tank[1]), (0.0, column[0]),
                             (0.0, column[1]), wall_layers, dummy_layers)
    prm = baseline_physics(l0, dt, (-margin, -margin, 0.0),
                           (tank[0] + margin, tank[1] + margin, 0.0))
    return prm, pos, vel, t


def shaken(scene, jitter=0.4, vel_sigma=0.1, seed=0):
    """A lattice scene's fluid particles displaced uniformly by up to
    +-jitter l0 in x and y and given N(0, vel_sigma) m/s velocities: a
    collision-heavy workload (at jitter 0.4 about 8 % of neighbouring fluid
    pairs start closer than the collision distance 0.5 l0, at most two per
    particle)."""
    prm, pos, vel, t = scene
    pos, vel = pos.copy(), vel.copy()
    rng = np.random.default_rng(seed)
    fl = t == FLUID
    l0 = prm["particle_distance"]
    pos[fl, :2] += rng.uniform(-jitter, jitter, (fl.sum(), 2)) * l0
    vel[fl, :2] = rng.normal(0.0, vel_sigma, (fl.sum(), 2))
    return prm, pos, vel, t


def hydrostatic(l0, size=(0.4, 0.4), tank_height=None, dt=1e-3, wall_layers=2, dummy_layers=2,
                margin=0.1):
    """Hydrostatic tank: the whole tank width filled to `size[1]`."""
    th = size[1] * 1.1 if tank_height is None else tank_height
    pos, vel, t = tank_scene(l0, (0.0, size[0]), (0.0, th), (0.0, size[0]), (0.0, size[1]),
                             wall_layers, dummy_layers)
    prm = baseline_physics(l0, dt, (-margin, -margin, 0.0), (size[0] + margin, th + margin, 0.0))
    return prm, pos, vel, t


def batch_scenes(seed=0, n_scenes=64, fluid_range=(2000, 60000), aspect_range=(0.5, 2.0),
                 l0_range=(1e-3, 5e-3)):
    """Independent uneven scenes for one batch: per scene a seeded fluid
    particle count, column aspect (height / width) and particle distance,
    alternately a dam break (column in the left corner of a tank 4x its
    width and 1.2x its height) and a hydrostatic tank (column filling the
    tank's width), with the dam-break physics at dt = 0.1 s/m x l0 (the
    1,250-particle case's dt / l0).  Returns a list of (params, pos, vel, types)."""
    rng = np.random.default_rng(seed)
    out = []
    for s in range(n_scenes):
        nf = int(rng.integers(fluid_range[0], fluid_range[1] + 1))
        aspect = float(rng.uniform(*aspect_range))
        l0 = float(rng.uniform(*l0_range))
        cols = max(2, int(round(math.sqrt(nf / aspect))))
        rows = max(2, int(round(nf / cols)))
        w, h = cols * l0, rows * l0
        dt = 0.1 * l0
        if s % 2 == 0:
            out.append(dam_break(l0, tank=(4 * w, 1.2 * h), column=(w, h), dt=dt,
                                 margin=2 * l0 * 10))
        else:
            out.append(hydrostatic(l0, size=(w, h), dt=dt, margin=2 * l0 * 10))
    return out


def wall_taps(pos, types, l0, count=16):
    """`count` wall particles of the innermost bottom wall row (the row just
    below the fluid), evenly spread over its length: pressure taps."""
    wall = np.flatnonzero(types == WALL)
    fluid_y = pos[types == FLUID, 1].min()
    below = wall[pos[wall, 1] < fluid_y]
    row = below[np.isclose(pos[below, 1], pos[below, 1].max(), rtol=0, atol=0.25 * l0)]
    row = row[np.argsort(pos[row, 0])]
    idx = np.linspace(0, len(row) - 1, count).round().astype(int)
    return row[idx].astype(np.int32)
