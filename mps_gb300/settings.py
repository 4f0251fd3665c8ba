"""Reader for the reference's settings.yml (Settings::load, src/settings.cpp:12-89).

Accepts the reference's files unchanged: block mappings by indentation,
flow sequences, scalars and comments.  Radii are ratios times the particle
distance and re_max is the largest, as src/settings.cpp:43-56 derives them.
"""
from __future__ import annotations


def _scalar(s: str):
    s = s.strip()
    if len(s) >= 2 and s[0] in "'\"" and s[-1] == s[0]:
        return s[1:-1]
    if s in ("True", "true", "TRUE"):
        return True
    if s in ("False", "false", "FALSE"):
        return False
    try:
        return int(s)
    except ValueError:
        pass
    try:
        return float(s)
    except ValueError:
        return s


def parse_yaml(text: str) -> dict:
    root: dict = {}
    stack = [(-1, root)]
    for raw in text.splitlines():
        line = raw.split("#", 1)[0].rstrip()
        if not line.strip():
            continue
        indent = len(line) - len(line.lstrip(" "))
        body = line.strip()
        if ":" not in body:
            raise ValueError(f"unsupported YAML line: {raw!r}")
        key, val = body.split(":", 1)
        key, val = key.strip(), val.strip()
        while stack[-1][0] >= indent:
            stack.pop()
        parent = stack[-1][1]
        if not val:
            child: dict = {}
            parent[key] = child
            stack.append((indent, child))
        elif val.startswith("["):
            parent[key] = [_scalar(v) for v in val.strip("[]").split(",")]
        else:
            parent[key] = _scalar(val)
    return root


def load_settings(path: str) -> dict:
    """Returns the engine parameter dict plus 'finish_time', 'output_interval'
    and 'input_csv' (relative to the working directory, as the reference)."""
    with open(path) as f:
        y = parse_yaml(f.read())
    l0 = float(y["particle distance"])
    er = y["effective radius ratio"]
    ps = y["pressure stabilization"]
    qc, ho = ps["quasi compressibility"], ps["higher order source term"]
    return dict(
        dim=int(y["dim"]), particle_distance=l0, dt=float(y["dt"]),
        finish_time=float(y["finish time"]), output_interval=float(y["output interval"]),
        cfl=float(y["CFL condition"]),
        domain_min=[float(y["domain range X"][0]), float(y["domain range Y"][0]),
                    float(y["domain range Z"][0])],
        domain_max=[float(y["domain range X"][1]), float(y["domain range Y"][1]),
                    float(y["domain range Z"][1])],
        density=float(y["density"]), kinematic_viscosity=float(y["kinematic viscosity"]),
        gravity=[float(v) for v in y["gravity"]],
        re_pressure=float(er["pressure"]) * l0, re_viscosity=float(er["viscosity"]) * l0,
        re_surface=float(er["surface detection"]) * l0,
        surface_threshold=float(y["threshold for surface detection"]),
        quasi_compressibility_on=int(bool(qc["on"])),
        compressibility=float(qc["compressibility"]) if qc["on"] else 0.0,
        higher_order_on=int(bool(ho["on"])),
        higher_order_gamma=float(ho["gamma"]) if ho["on"] else 0.0,
        relaxation=float(y["relaxation coefficient for pressure"]),
        collision_distance=float(y["collision distance ratio"]) * l0,
        restitution=float(y["coefficient of restitution"]),
        input_csv=str(y["inputCsvPath"]),
    )
