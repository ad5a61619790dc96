"""The bounds-checked build (-DAPIC_BOUNDS_CHECK: particle slots, cells,
faces and sort destinations tested before every data-dependent access, an
index outside its buffer failing the update) runs the dam-break scene in
both solver families, without the Morton sort, and the dense and degenerate
P2G scenes without a finding, and gives the same bits as the default
build."""
import os
import subprocess
import sys

import numpy as np
import pytest

import apic_gb300 as A
from apic_gb300 import build as gpu_build
from parity_helpers import eq

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def test_checked_build_matches_default(gpu_lib, tmp_path):
    checked = gpu_build.build(checked=True)
    out = tmp_path / "checked.npz"
    env = dict(os.environ)
    env["PYTHONPATH"] = os.pathsep.join([HERE, os.path.dirname(A.__file__) + "/.."] +
                                        ([env["PYTHONPATH"]] if env.get("PYTHONPATH") else []))
    r = subprocess.run([sys.executable, os.path.join(HERE, "bounds_scenarios.py"), checked, str(out)],
                       capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    import bounds_scenarios
    ref = bounds_scenarios.run_all()
    got = np.load(out)
    assert sorted(got.files) == sorted(ref.keys())
    for k, v in ref.items():
        eq(got[k], v, f"checked build: {k}")
