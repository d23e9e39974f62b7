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


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "eval")), reason="reference sources not present")
@pytest.mark.skipif(not os.path.exists(LIB), reason="libidash_gpu.so not built")
@pytest.mark.parametrize("exe,fn,sig", [
    ("decrypt_gpu", "decrypt_predictions", "(DecryptedPredictions&, EncryptedPredictions const&, IdashKey const&)"),
    ("encrypt_gpu", "encrypt_data_ph1", "(EncryptedData&, PlaintextData const&, IdashKey const&)"),
])
def test_reference_party_a_links_against_gpu_functions(exe, fn, sig):
    """The reference's decrypt and encrypt mains, with decrypt_predictions /
    encrypt_data_ph1 taken from integration/party_a_gpu.cpp."""
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), f"_ref/{exe}", f"REF_DIR={REF}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    syms = subprocess.run(["nm", "-C", os.path.join(ROOT, "oracle", "_ref", exe)], capture_output=True,
                          text=True).stdout
    assert f"T {fn}{sig}" in syms
    assert f"T {fn}_cpu{sig}" in syms
    dyn = subprocess.run(["nm", "-D", "-C", os.path.join(ROOT, "oracle", "_ref", exe)], capture_output=True,
                         text=True).stdout
    assert "U idash_decrypt_trlwe_device" in dyn and "U idash_encrypt_trlwe_device" in dyn
