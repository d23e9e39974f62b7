"""The no-allocation entry point's planning (idash2019_2_gb300/csrc/
noalloc_plan.cpp) without a GPU: which kernel it runs and how much of its
fixed 64 MiB scratch array the plan's tables take.

The full-scale model (16,184 tags, 80,882 targets x 3 outputs, 5 neighbours:
3.9 M terms) must fit in the reference's own record layout, whose variance
program (row and coefficient per term) is the largest table, as well as in
dense rows and at NUM_REGIONS = 10.  A 30-neighbour model (90 slots per
output, more than any window holds) plans the direct kernel, and a model
beyond the array is refused with the sizes in the message."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    exe = tmp_path_factory.mktemp("noalloc") / "noalloc_plan_check"
    csrc = os.path.join(ROOT, "idash2019_2_gb300", "csrc")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", csrc, "-o", str(exe),
                    os.path.join(ROOT, "tests", "native", "noalloc_plan_check.cpp"),
                    os.path.join(csrc, "noalloc_plan.cpp"), os.path.join(csrc, "plan.cpp")], check=True)
    return exe


def _write_csr(path, ptr, feat, coef):
    with open(path, "wb") as f:
        np.array([len(ptr) - 1, len(feat)], np.uint64).tofile(f)
        np.ascontiguousarray(ptr, np.uint64).tofile(f)
        np.ascontiguousarray(feat, np.uint32).tofile(f)
        np.ascontiguousarray(coef, np.int32).tofile(f)


def _plan(checker, path, regions, rs, n_rows, var, index):
    r = subprocess.run([str(checker), str(path), str(regions), str(rs), str(n_rows), str(int(var)), str(int(index))],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    fields = dict(kv.split("=", 1) for kv in r.stdout.strip().split(" ", 5))
    return {"bytes": int(fields["bytes"]), "limit": int(fields["limit"]), "window": fields["window"] == "1",
            "err": fields["err"]}


@pytest.fixture(scope="module")
def full_scale(tmp_path_factory):
    gpu = pytest.importorskip("idash2019_2_gb300.gpu")
    try:
        w = gpu.synth_model(seed=0x1DA52019, n_tags=16184, n_targets=80882, neighbours=5)
    except ImportError as e:
        pytest.skip(str(e))
    path = tmp_path_factory.mktemp("csr") / "full.bin"
    _write_csr(path, w.model.term_ptr, w.model.term_feat, w.model.term_coef)
    return path


@pytest.mark.parametrize("regions,rs,var,index", [
    (1, 1024, True, True),    # the reference's record layout: variance program + output indices
    (1, 1024, False, False),  # dense rows
    (10, 102, True, True),    # records, 10 regions (rotated slots)
])
def test_full_scale_model_fits_the_scratch(checker, full_scale, regions, rs, var, index):
    n_rows = (3 * 16184 + regions - 1) // regions
    p = _plan(checker, full_scale, regions, rs, n_rows, var, index)
    assert p["err"] == "-", p
    assert p["window"]
    assert 0 < p["bytes"] <= p["limit"] == 64 << 20


def test_large_neighbourhoods_plan_the_direct_kernel(checker, tmp_path):
    gpu = pytest.importorskip("idash2019_2_gb300.gpu")
    try:
        w = gpu.synth_model(seed=44, n_tags=100, n_targets=60, neighbours=30)
    except ImportError as e:
        pytest.skip(str(e))
    path = tmp_path / "wide.bin"
    _write_csr(path, w.model.term_ptr, w.model.term_feat, w.model.term_coef)
    p = _plan(checker, path, 1, 1024, 300, False, False)
    assert p["err"] == "-" and not p["window"]


def test_models_beyond_the_scratch_are_refused(checker, tmp_path):
    n_out, per = 1_200_000, 16
    path = tmp_path / "big.bin"
    _write_csr(path, np.arange(n_out + 1, dtype=np.uint64) * per, np.tile(np.arange(per, dtype=np.uint32), n_out),
               np.ones(n_out * per, np.int32))
    p = _plan(checker, path, 1, 1024, 64, False, False)
    assert p["bytes"] > p["limit"]
    assert "64 MiB" in p["err"]
