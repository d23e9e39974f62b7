"""The host planner (idash2019_2_gb300/csrc/plan.cpp) without a GPU: split
plans executed on the CPU as the kernels execute them equal a direct
evaluation of the model (tests/native/plan_emulation.cpp); tensor-core plans
decode to the model's coefficients and their digit arithmetic, restated in
integers, equals direct evaluation within the exactness bound
(tests/native/tc_plan_check.cpp)."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_split_plans_match_direct_evaluation(tmp_path):
    exe = tmp_path / "plan_emulation"
    csrc = os.path.join(ROOT, "idash2019_2_gb300", "csrc")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", csrc, "-o", str(exe),
                    os.path.join(ROOT, "tests", "native", "plan_emulation.cpp"), os.path.join(csrc, "plan.cpp")],
                   check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("trial")]
    assert len(lines) == 40 and all(" ok:" in ln for ln in lines)
    assert any("phases=1 " not in ln for ln in lines)  # some plans did split


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_tensor_core_plans_decode_and_stay_exact(tmp_path):
    exe = tmp_path / "tc_plan_check"
    csrc = os.path.join(ROOT, "idash2019_2_gb300", "csrc")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", csrc, "-o", str(exe),
                    os.path.join(ROOT, "tests", "native", "tc_plan_check.cpp"), os.path.join(csrc, "plan.cpp")],
                   check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-3000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("trial")]
    assert len(lines) == 24 and all(" ok:" in ln for ln in lines)
    assert "refused ok" in r.stdout
