"""The reference-side adapters (idash2019_2_gb300/integration/), linked into
the reference's own unmodified mains.

* Link checks: eval/cloud.cpp, eval/decrypt.cpp and eval/encrypt.cpp with
  cloud_compute_score / decrypt_predictions / encrypt_data_ph1 taken from the
  adapters and libidash_gpu.so.
* Byte checks on CPU: the same mains and adapters linked with an oracle-backed
  stand-in of the C ABI (tests/native/capi_oracle_standin.cpp) must write the
  reference's own encrypted_prediction.bin, result.csv and result_bypos.csv
  (tests/golden/<case>, produced by the reference) byte for byte.  This pins
  what the adapters themselves decide: the record order of the prediction
  file (outputs created in the model map's iteration order,
  eval/idash.cpp:772-777 then :605-608), the FeatIndex -> row map, the record
  layouts and the variance bookkeeping.

Only where the reference sources are present (skipped elsewhere)."""
import os
import shutil
import subprocess

import pytest

from conftest import GOLDEN, HAVE_REF, REF_DIR, ROOT, SMALL_CASES

LIB = os.path.join(ROOT, "idash2019_2_gb300", "libidash_gpu.so")
REF_BIN = os.path.join(ROOT, "oracle", "_ref")
needs_ref = pytest.mark.skipif(not HAVE_REF, reason="reference sources not present")


def _make(target):
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), target, f"REF_DIR={REF_DIR}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


@needs_ref
@pytest.mark.skipif(not os.path.exists(LIB), reason="libidash_gpu.so not built")
def test_reference_cloud_links_against_gpu_cloud_compute_score():
    _make("_ref/cloud_gpu")
    syms = subprocess.run(["nm", "-C", os.path.join(REF_BIN, "cloud_gpu")], capture_output=True, text=True).stdout
    assert "T cloud_compute_score(EncryptedPredictions&" in syms
    assert "T cloud_compute_score_cpu(EncryptedPredictions&" in syms


@needs_ref
@pytest.mark.skipif(not os.path.exists(LIB), reason="libidash_gpu.so not built")
@pytest.mark.parametrize("exe,fn,sig", [
    ("decrypt_gpu", "decrypt_predictions", "(DecryptedPredictions&, EncryptedPredictions const&, IdashKey const&)"),
    ("encrypt_gpu", "encrypt_data_ph1", "(EncryptedData&, PlaintextData const&, IdashKey const&)"),
])
def test_reference_party_a_links_against_gpu_functions(exe, fn, sig):
    """The reference's decrypt and encrypt mains, with decrypt_predictions /
    encrypt_data_ph1 taken from integration/party_a_gpu.cpp."""
    _make(f"_ref/{exe}")
    syms = subprocess.run(["nm", "-C", os.path.join(REF_BIN, exe)], capture_output=True, text=True).stdout
    assert f"T {fn}{sig}" in syms
    assert f"T {fn}_cpu{sig}" in syms
    dyn = subprocess.run(["nm", "-D", "-C", os.path.join(REF_BIN, exe)], capture_output=True, text=True).stdout
    assert "U idash_decrypt_trlwe_device" in dyn and "U idash_encrypt_trlwe_device" in dyn


def _case_dir(tmp_path, case):
    d = tmp_path / case
    d.mkdir()
    for f in ("params.bin", "encrypted_data.bin", "keys.bin"):
        shutil.copy(os.path.join(GOLDEN, case, f), d / f)
    shutil.copytree(os.path.join(GOLDEN, case, "model"), d / "model")
    return d


def _bytes(path):
    with open(path, "rb") as f:
        return f.read()


@needs_ref
@pytest.mark.parametrize("case", SMALL_CASES)
def test_adapter_cloud_writes_the_reference_prediction_file(tmp_path, case):
    """eval/cloud.cpp + the cloud_compute_score adapter (C ABI from the
    oracle stand-in): encrypted_prediction.bin equals the reference's, records
    in the same order."""
    _make("_ref/cloud_standin")
    d = _case_dir(tmp_path, case)
    r = subprocess.run([os.path.join(REF_BIN, "cloud_standin"), "model"], cwd=d, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert _bytes(d / "encrypted_prediction.bin") == _bytes(os.path.join(GOLDEN, case, "encrypted_prediction.bin"))


@needs_ref
@pytest.mark.parametrize("case", SMALL_CASES)
def test_adapter_decrypt_writes_the_reference_csv(tmp_path, case):
    """eval/decrypt.cpp + the decrypt_predictions adapter (C ABI from the
    oracle stand-in) on the reference's predictions: result.csv and
    result_bypos.csv equal the reference's."""
    _make("_ref/decrypt_standin")
    d = _case_dir(tmp_path, case)
    shutil.copy(os.path.join(GOLDEN, case, "encrypted_prediction.bin"), d / "encrypted_prediction.bin")
    for args, name in (([], "result.csv"), (["bypos"], "result_bypos.csv")):
        r = subprocess.run([os.path.join(REF_BIN, "decrypt_standin"), *args], cwd=d, capture_output=True, text=True)
        assert r.returncode == 0, r.stdout + r.stderr
        assert _bytes(d / name) == _bytes(os.path.join(GOLDEN, case, name)), name
