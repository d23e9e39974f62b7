"""Party A's decryption on the GPU (decrypt_predictions + the CSV writer,
eval/idash.cpp:682-761 and :436-469, eval/decrypt.cpp) against the
reference's own decrypt output and the oracle, bit for bit."""
import filecmp
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, SMALL_CASES

pytestmark = pytest.mark.gpu

gpu = pytest.importorskip("idash2019_2_gb300.gpu")


@pytest.fixture(scope="module")
def ctx():
    c = gpu.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("by_position", [True, False])
@pytest.mark.parametrize("name", SMALL_CASES)
def test_decrypt_files_byte_identical_to_reference(tmp_path, name, by_position):
    """keys.bin + the reference's encrypted_prediction.bin -> the CSV the
    reference's decrypt wrote, byte for byte (result_bypos.csv / result.csv)."""
    d = os.path.join(GOLDEN, name)
    out = tmp_path / "out.csv"
    rep = gpu.decrypt_files(os.path.join(d, "keys.bin"), os.path.join(d, "encrypted_prediction.bin"), str(out),
                            by_position)
    assert rep["n_lines"] > 0 and rep["n_records"] > 0
    want = os.path.join(d, "result_bypos.csv" if by_position else "result.csv")
    assert filecmp.cmp(out, want, shallow=False)


@pytest.mark.parametrize("name", SMALL_CASES)
def test_decrypt_cli_matches_reference(tmp_path, name):
    """idash_decrypt: eval/decrypt.cpp's file names and argv."""
    d = os.path.join(GOLDEN, name)
    for f in ["keys.bin", "encrypted_prediction.bin"]:
        shutil.copy(os.path.join(d, f), tmp_path / f)
    exe = os.path.join(ROOT, "idash2019_2_gb300", "idash_decrypt")
    r = subprocess.run([exe, "bypos"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "decrypt wall time" in r.stdout
    assert filecmp.cmp(tmp_path / "result_bypos.csv", os.path.join(d, "result_bypos.csv"), shallow=False)
    r = subprocess.run([exe], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert filecmp.cmp(tmp_path / "result.csv", os.path.join(d, "result.csv"), shallow=False)


@pytest.mark.parametrize("key_kind", ["binary", "integer", "zero"])
@pytest.mark.parametrize("num_samples", [1, 5, 1000, 1024])
def test_decrypt_device_vs_oracle(ctx, oracle, key_kind, num_samples):
    """Random rows, record layout: every float bit-exact to the oracle's
    restatement of tLwePhase + t32tod."""
    rng = np.random.default_rng(num_samples)
    n_rows = 333
    rows = rng.integers(0, 2 ** 32, size=(n_rows, 2048), dtype=np.uint64).astype(np.uint32).view(np.int32)
    if key_kind == "binary":
        key = rng.integers(0, 2, size=1024).astype(np.int32)
    elif key_kind == "integer":
        key = rng.integers(-3, 4, size=1024).astype(np.int32)
    else:
        key = np.zeros(1024, np.int32)
    rec = np.zeros((n_rows, gpu.RECORD_BYTES), np.uint8)
    rec[:, 8:8 + 8192] = rows.view(np.uint8).reshape(n_rows, 8192)
    d_in = ctx.device_alloc(rec.nbytes)
    d_in.upload(rec)
    d_out = ctx.device_alloc(n_rows * num_samples * 4)
    gpu.decrypt_device(ctx, key, d_in.ptr, gpu.RECORD_IN, n_rows, num_samples, d_out.ptr)
    ctx.sync()
    got = d_out.download(dtype=np.float32).reshape(n_rows, num_samples)
    want = oracle.trlwe_decrypt(rows, key, num_samples)
    np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))
    d_in.free()
    d_out.free()


def test_encrypt_score_decrypt_round_trip(ctx, oracle):
    """Synthetic encryptions (device) -> batched scoring -> decryption: the
    decrypted scores are the plaintext model scores (bias + sum of the
    coefficients of the set one-hot bits, in units of 2^-14) within the noise,
    and the decryption is bit-exact to the oracle on the scored rows."""
    seed, n_tags, n_targets, ns = 11, 60, 150, 1000
    w = gpu.synth_model(seed, n_tags, n_targets, neighbours=5)
    params = gpu.TrlweParams(1024, 1, ns, 1, 1024, 1 << 18, 42)
    n_rows = 3 * n_tags
    d_in = ctx.device_alloc(n_rows * 8192)
    gpu.synth_trlwe_device(ctx, seed, params, n_tags, d_in.ptr, gpu.DENSE_TRLWE)
    m = gpu.TrlweModel(ctx, w.model, n_rows, ns, 1, 1024)
    d_out = ctx.device_alloc(m.n_out * 8192)
    m.score_device(d_in.ptr, gpu.DENSE_TRLWE, d_out.ptr, gpu.DENSE_TRLWE)
    d_dec = ctx.device_alloc(m.n_out * ns * 4)
    key = gpu.synth_key(seed)
    gpu.decrypt_device(ctx, key, d_out.ptr, gpu.DENSE_TRLWE, m.n_out, ns, d_dec.ptr)
    ctx.sync()
    dec = d_dec.download(dtype=np.float32).reshape(m.n_out, ns)
    outs = d_out.download(dtype=np.int32).reshape(m.n_out, 2048)
    np.testing.assert_array_equal(dec.view(np.uint32), oracle.trlwe_decrypt(outs, key, ns).view(np.uint32))
    # plaintext: genotype g(p, s) = hash(seed, 2, p*ns + s) % 3 sets feature 3p + g
    geno = np.array([[oracle.lib().oracle_hash32(seed, 2, p * ns + s) % 3 for s in range(ns)]
                     for p in range(n_tags)])
    csr = w.model
    for o in range(0, m.n_out, 7):
        lo, hi = int(csr.term_ptr[o]), int(csr.term_ptr[o + 1])
        want = np.zeros(ns)
        coefs = []
        for t in range(lo, hi):
            f, c = int(csr.term_feat[t]), int(csr.term_coef[t])
            if f == 0xFFFFFFFF:
                want += c
            else:
                want += c * (geno[f // 3] == f % 3)
                coefs.append(c)
        want *= 2.0 ** -14
        diff = (dec[o].astype(np.float64) - want + 0.5) % 1.0 - 0.5
        bound = 8 * 128 * 2.0 ** -32 * np.sqrt(1 + sum(c * c for c in coefs)) + 2.0 ** -24
        assert np.max(np.abs(diff)) <= bound, f"output {o}: {np.max(np.abs(diff))} > {bound}"
    for b in (d_in, d_out, d_dec):
        b.free()
    m.free()


def test_decrypt_errors(ctx):
    key = np.zeros(1024, np.int32)
    d = ctx.device_alloc(8192)
    with pytest.raises(gpu.IdashError):
        gpu.decrypt_device(ctx, key, d.ptr, gpu.DENSE_TRLWE, 1, 1025, d.ptr)  # num_samples > N
    with pytest.raises(gpu.IdashError):
        gpu.decrypt_device(ctx, key[:1000], d.ptr, gpu.DENSE_TRLWE, 1, 10, d.ptr)  # N not a power of two
    d.free()


@pytest.mark.parametrize("N", [4, 16, 32, 64, 256, 2048])
def test_decrypt_polynomial_sizes(ctx, oracle, N):
    """Every polynomial size the entry point takes, binary keys: N a multiple
    of 32 runs the register-windowed kernel (1, 2, 4 or 8 rows per CTA by
    the number of samples), N = 4 and 16 the general one; bit-exact."""
    rng = np.random.default_rng(N)
    n_rows = 37
    rows = rng.integers(0, 2 ** 32, size=(n_rows, 2 * N), dtype=np.uint64).astype(np.uint32).view(np.int32)
    key = rng.integers(0, 2, size=N).astype(np.int32)
    d_in = ctx.device_alloc(rows.nbytes)
    d_in.upload(rows)
    lay = gpu.RowLayout(2 * N * 4, 0, -1, -1)
    for ns in sorted({1, min(N, 17), N // 2 + 1, N}):
        d_out = ctx.device_alloc(n_rows * ns * 4)
        gpu.decrypt_device(ctx, key, d_in.ptr, lay, n_rows, ns, d_out.ptr)
        ctx.sync()
        got = d_out.download(dtype=np.float32).reshape(n_rows, ns)
        want = oracle.trlwe_decrypt(rows, key, ns)
        np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32), err_msg=f"N={N} ns={ns}")
        d_out.free()
    d_in.free()
