"""The reference-side binding links: the reference's unmodified eval/cloud.cpp,
eval/idash.cpp (its cloud_compute_score renamed) and eval/parse_vw.cpp,
against oracle/tfhe_compat, with the GPU adapter and libidash_gpu.so.
Only where the reference sources are present (skipped elsewhere)."""
import os
import subprocess

import pytest

from conftest import ROOT

REF = os.environ.get("REF_DIR", "/root/reference")
LIB = os.path.join(ROOT, "idash2019_2_gb300", "libidash_gpu.so")


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "eval")), reason="reference sources not present")
@pytest.mark.skipif(not os.path.exists(LIB), reason="libidash_gpu.so not built")
def test_reference_cloud_links_against_gpu_cloud_compute_score():
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "_ref/cloud_gpu", f"REF_DIR={REF}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    exe = os.path.join(ROOT, "oracle", "_ref", "cloud_gpu")
    syms = subprocess.run(["nm", "-C", exe], capture_output=True, text=True).stdout
    assert "T cloud_compute_score(EncryptedPredictions&" in syms
    assert "T cloud_compute_score_cpu(EncryptedPredictions&" in syms
