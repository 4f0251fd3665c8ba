"""The C++ front end (mps -s settings.yml: Simulation/MPS/Exporter) end to end
on the GPU, checked against the CPU oracle driven over the same steps."""
import os
import subprocess
import sys

import numpy as np
import pytest

from gpu_util import engine_or_skip

pytestmark = pytest.mark.gpu
REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cli_simulation_matches_oracle(tmp_path):
    engine_or_skip()
    from mps_gb300 import build, scenes
    from oracle import Oracle

    sys.path.insert(0, os.path.join(REPO, "tests", "golden"))
    from make_golden import yaml_text

    exe = build.build_host()
    prm, pos, vel, t = scenes.dam_break(0.02, tank=(0.6, 0.4), column=(0.2, 0.3), dt=2e-3)
    scenes.write_csv(tmp_path / "input.csv", pos, vel, t)
    text = yaml_text(prm, "input.csv").replace("finish time: 1.0", "finish time: 0.0201") \
                                      .replace("output interval: 1.0", "output interval: 0.01")
    (tmp_path / "settings.yml").write_text(text)
    out = subprocess.run([exe, "-s", "settings.yml"], cwd=tmp_path, capture_output=True, text=True,
                         timeout=300)
    assert out.returncode == 0, out.stdout[-2000:] + out.stderr[-2000:]
    res = tmp_path / "result"
    csvs = sorted(os.listdir(res / "csv"))
    assert csvs == ["output_0000.csv", "output_0001.csv", "output_0002.csv"]
    assert len(os.listdir(res / "vtu")) == 3
    assert (res / "time_step_report.csv").exists() and (res / "execution.log").exists()

    _, pos0, vel0, t0 = scenes.read_csv(tmp_path / "input.csv")
    o = Oracle(prm, pos0, vel0, t0)
    o.set_cg(solves=1)
    for s in range(1, 11):
        o.step(export=(s % 5 == 0))
    ref = o.state()
    tm, p_cli, v_cli, t_cli = scenes.read_csv(res / "csv" / "output_0002.csv")
    assert abs(tm - 0.02) < 1e-9
    keep = ref["type"] != -1
    assert np.array_equal(t_cli, ref["type"][keep])
    assert np.max(np.abs(p_cli - ref["pos"][keep])) <= 1e-6   # six-decimal CSV
    assert np.max(np.abs(v_cli - ref["vel"][keep])) <= 1e-6
