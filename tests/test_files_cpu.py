"""Failure handling of the cloud step's file inputs, without a GPU: every
malformed input is an error status with a message (the reference aborts via
REQUIRE_DRAMATICALLY, eval/idash.h:12), reported before the device is used."""
import os
import shutil

import pytest

from conftest import GOLDEN

gpu = pytest.importorskip("idash2019_2_gb300.gpu")


@pytest.fixture()
def case(tmp_path):
    try:
        gpu._lib.load()
    except ImportError as e:
        pytest.skip(str(e))
    src = os.path.join(GOLDEN, "ref_r10")
    for f in ["params.bin", "encrypted_data.bin"]:
        shutil.copy(os.path.join(src, f), tmp_path / f)
    shutil.copytree(os.path.join(src, "model"), tmp_path / "model")
    return tmp_path


def run(d, params="params.bin", data="encrypted_data.bin"):
    return gpu.cloud_files(str(d / params), str(d / "model"), str(d / data), str(d / "out.bin"), device=0)


def expect(d, name, **kw):
    with pytest.raises(gpu.IdashError) as e:
        run(d, **kw)
    assert e.value.name == name, str(e.value)
    return str(e.value)


def test_missing_params(case):
    expect(case, "IDASH_ERR_IO", params="nope.bin")


def test_truncated_params(case):
    raw = (case / "params.bin").read_bytes()
    (case / "params.bin").write_bytes(raw[:len(raw) // 2])
    assert "truncated" in expect(case, "IDASH_ERR_FORMAT")


def test_inconsistent_regions(case):
    raw = bytearray((case / "params.bin").read_bytes())
    raw[20:24] = (2048).to_bytes(4, "little")  # NUM_REGIONS * REGION_SIZE > N
    (case / "params.bin").write_bytes(bytes(raw))
    expect(case, "IDASH_ERR_FORMAT")


def test_missing_model_file(case):
    victim = sorted(os.listdir(case / "model"))[4]
    os.remove(case / "model" / victim)
    assert victim in expect(case, "IDASH_ERR_IO")


def test_model_names_an_unknown_tag(case):
    victim = sorted(os.listdir(case / "model"))[0]
    with open(case / "model" / victim, "a") as f:
        f.write("999999999_1 17\n")
    expect(case, "IDASH_ERR_INDEX")


def test_bad_feature_name(case):
    victim = sorted(os.listdir(case / "model"))[1]
    with open(case / "model" / victim, "a") as f:
        f.write("notafeature 3\n")
    expect(case, "IDASH_ERR_FORMAT")


def test_truncated_ciphertexts(case):
    raw = (case / "encrypted_data.bin").read_bytes()
    (case / "encrypted_data.bin").write_bytes(raw[:-100])
    assert "8208" in expect(case, "IDASH_ERR_FORMAT")


def test_missing_ciphertexts(case):
    expect(case, "IDASH_ERR_IO", data="absent.bin")


# ------------------------------------------------ decryption inputs (party A)
@pytest.fixture()
def dcase(tmp_path):
    try:
        gpu._lib.load()
    except ImportError as e:
        pytest.skip(str(e))
    src = os.path.join(GOLDEN, "ref_r10")
    for f in ["keys.bin", "encrypted_prediction.bin"]:
        shutil.copy(os.path.join(src, f), tmp_path / f)
    return tmp_path


def dexpect(d, name, keys="keys.bin", preds="encrypted_prediction.bin"):
    with pytest.raises(gpu.IdashError) as e:
        gpu.decrypt_files(str(d / keys), str(d / preds), str(d / "out.csv"), True, device=0)
    assert e.value.name == name, str(e.value)
    assert not (d / "out.csv").exists()
    return str(e.value)


def test_decrypt_missing_key(dcase):
    assert "nope.bin" in dexpect(dcase, "IDASH_ERR_IO", keys="nope.bin")


def test_decrypt_truncated_key(dcase):
    raw = (dcase / "keys.bin").read_bytes()
    (dcase / "keys.bin").write_bytes(raw[:-100])
    assert "truncated" in dexpect(dcase, "IDASH_ERR_FORMAT")


def test_decrypt_key_record_tag(dcase):
    raw = bytearray((dcase / "keys.bin").read_bytes())
    raw[len(raw) - (12 + 16 + 4096)] ^= 0xFF  # the key record's tag
    (dcase / "keys.bin").write_bytes(bytes(raw))
    assert "key record" in dexpect(dcase, "IDASH_ERR_FORMAT")


def test_decrypt_missing_prediction_record(dcase):
    raw = (dcase / "encrypted_prediction.bin").read_bytes()
    rec = 8208
    count = int.from_bytes(raw[:8], "little")
    (dcase / "encrypted_prediction.bin").write_bytes((count - 1).to_bytes(8, "little") + raw[8:8 + (count - 1) * rec])
    assert "no record" in dexpect(dcase, "IDASH_ERR_INDEX")


def test_decrypt_truncated_predictions(dcase):
    raw = (dcase / "encrypted_prediction.bin").read_bytes()
    (dcase / "encrypted_prediction.bin").write_bytes(raw[:-10])
    dexpect(dcase, "IDASH_ERR_FORMAT")


# ------------------------------------------------ encryption inputs (party A)
@pytest.fixture()
def ecase(tmp_path):
    try:
        gpu._lib.load()
    except ImportError as e:
        pytest.skip(str(e))
    src = os.path.join(GOLDEN, "ref_r10")
    for f in ["keys.bin", "tags.txt"]:
        shutil.copy(os.path.join(src, f), tmp_path / f)
    return tmp_path


def eexpect(d, name, keys="keys.bin", tags="tags.txt"):
    with pytest.raises(gpu.IdashError) as e:
        gpu.encrypt_files(str(d / keys), str(d / tags), str(d / "enc.bin"), seed=1, device=0)
    assert e.value.name == name, str(e.value)
    assert not (d / "enc.bin").exists()
    return str(e.value)


def test_encrypt_missing_challenge(ecase):
    assert "nope.txt" in eexpect(ecase, "IDASH_ERR_IO", tags="nope.txt")


def test_encrypt_missing_key(ecase):
    eexpect(ecase, "IDASH_ERR_IO", keys="nope.bin")


def test_encrypt_bad_chromosome_field(ecase):
    lines = (ecase / "tags.txt").read_text().splitlines()
    lines[3] = "21" + lines[3][2:]
    (ecase / "tags.txt").write_text("\n".join(lines) + "\n")
    assert "22" in eexpect(ecase, "IDASH_ERR_FORMAT")


def test_encrypt_missing_positions(ecase):
    lines = (ecase / "tags.txt").read_text().splitlines()
    (ecase / "tags.txt").write_text("\n".join(lines[:-2]) + "\n")
    assert "missing positions" in eexpect(ecase, "IDASH_ERR_FORMAT")


def test_encrypt_unknown_position(ecase):
    lines = (ecase / "tags.txt").read_text().splitlines()
    f = lines[0].split()
    f[1] = f[2] = "999999999"
    lines[0] = " ".join(f)
    (ecase / "tags.txt").write_text("\n".join(lines) + "\n")
    assert "not an input position" in eexpect(ecase, "IDASH_ERR_FORMAT")
