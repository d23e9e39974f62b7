"""Party A's encryption on the GPU (encrypt_data_ph1/ph2 and the record
writer, eval/idash.cpp:615-679, :536-556, eval/encrypt.cpp).  The random
masks and noise cannot match the reference's generator, so parity is:
the algebra exactly (b - a*s - m equals the noise the kernel reports, the
mask is the documented counter-based stream), the file's record order,
indices, tags and variances exactly as the reference writes them, and the
decryptions equal to the reference's within the encryption noise."""
import filecmp
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, SMALL_CASES

pytestmark = pytest.mark.gpu

gpu = pytest.importorskip("idash2019_2_gb300.gpu")

N = 1024


@pytest.fixture(scope="module")
def ctx():
    c = gpu.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("regions", [1, 3])
def test_encrypt_device_exact(ctx, oracle, regions):
    rng = np.random.default_rng(regions)
    rs = N // regions
    ns = min(rs, 300)
    n_rows, n_pos, seed = 40, 37, 12345
    key = rng.integers(0, 2, size=N).astype(np.int32)
    geno = rng.integers(-1, 3, size=(n_pos, ns)).astype(np.int8)
    slot_src = np.full(n_rows * regions, 0xFFFFFFFF, np.uint32)
    used = rng.choice(n_rows * regions, size=min(3 * n_pos, n_rows * regions), replace=False)
    slot_src[used] = np.arange(len(used), dtype=np.uint32) % (3 * n_pos)
    row_out = rng.permutation(n_rows).astype(np.uint32)
    row_index = rng.integers(0, 10 ** 6, size=n_rows).astype(np.uint32)
    bufs = {k: ctx.device_alloc(v.nbytes) for k, v in
            (("src", slot_src), ("geno", geno), ("out_row", row_out), ("index", row_index))}
    bufs["src"].upload(slot_src)
    bufs["geno"].upload(geno)
    bufs["out_row"].upload(row_out)
    bufs["index"].upload(row_index)
    d_out = ctx.device_alloc(n_rows * gpu.RECORD_BYTES)
    d_noise = ctx.device_alloc(n_rows * N * 4)
    params = gpu.encrypt_params(ns, regions, rs)
    gpu.encrypt_device(ctx, params, key, seed, n_rows, bufs["src"].ptr, bufs["geno"].ptr, ns, d_out.ptr,
                       gpu.RECORD_OUT, bufs["index"].ptr, bufs["out_row"].ptr, d_noise.ptr)
    ctx.sync()
    rec = d_out.download().reshape(n_rows, gpu.RECORD_BYTES)
    noise = d_noise.download(dtype=np.int32).reshape(n_rows, N)
    for r in range(n_rows):
        o = rec[row_out[r]]
        assert int(o[:4].view(np.uint32)[0]) == row_index[r] and int(o[4:8].view(np.int32)[0]) == 42
        assert o[8200:8208].view(np.float64)[0] == 2.0 ** -50
        words = o[8:8200].view(np.int32)
        mask = np.array([oracle.lib().oracle_hash32(seed, 21, r * N + j) for j in range(N)], np.uint32)
        np.testing.assert_array_equal(words[:N].view(np.uint32), mask)
        msg = np.zeros(N, np.uint32)
        for g in range(regions):
            src = slot_src[r * regions + g]
            if src == 0xFFFFFFFF:
                continue
            p, v = divmod(int(src), 3)
            gv = geno[p]
            val = np.where(gv == v, params.one_t32, np.where((gv < 0) | (gv > 2), params.nan_t32[v], 0))
            msg[g * rs:g * rs + ns] = val.astype(np.int64).astype(np.uint32)
        e = (oracle.phase(words, key) - msg).astype(np.uint32).view(np.int32)
        np.testing.assert_array_equal(e, noise[r])
    sd = noise.std()
    assert abs(noise.mean()) < 3 and abs(sd / 128.0 - 1) < 0.03, (noise.mean(), sd)
    assert np.abs(noise).max() < 6.5 * 128
    for b in list(bufs.values()) + [d_out, d_noise]:
        b.free()


@pytest.mark.parametrize("name", SMALL_CASES)
def test_encrypt_files_layout_and_decryption(tmp_path, oracle, name):
    """keys.bin + the challenge genotypes -> encrypted_data.bin with the
    reference's size, record order, indices, tags and variances; each record
    decrypts to the reference record's plaintext within two noises."""
    d = os.path.join(GOLDEN, name)
    out = tmp_path / "encrypted_data.bin"
    rep = gpu.encrypt_files(os.path.join(d, "keys.bin"), os.path.join(d, "tags.txt"), str(out), seed=99)
    ours, ref = oracle.read_records(str(out)), oracle.read_records(os.path.join(d, "encrypted_data.bin"))
    assert rep["n_records"] == len(ref) == len(ours)
    np.testing.assert_array_equal(ours["idx"], ref["idx"])
    assert np.all(ours["tag"] == ref["tag"])
    np.testing.assert_array_equal(ours["var"], ref["var"])
    key = oracle.read_key(os.path.join(d, "keys.bin"))
    for a, b in zip(ours, ref):
        diff = (oracle.phase(a["coef"], key) - oracle.phase(b["coef"], key)).astype(np.uint32).view(np.int32)
        assert np.abs(diff.astype(np.int64)).max() < 2 * 6.5 * 128


@pytest.mark.parametrize("name", ["ref_r10", "ref_r1"])
def test_encrypt_cloud_decrypt_pipeline(tmp_path, name):
    """GPU encrypt -> GPU cloud -> GPU decrypt on the reference's inputs gives
    the reference's decrypted CSV within the encryption noise."""
    d = os.path.join(GOLDEN, name)
    shutil.copytree(os.path.join(d, "model"), tmp_path / "model")
    gpu.encrypt_files(os.path.join(d, "keys.bin"), os.path.join(d, "tags.txt"), str(tmp_path / "enc.bin"), seed=7)
    gpu.cloud_files(os.path.join(d, "params.bin"), str(tmp_path / "model"), str(tmp_path / "enc.bin"),
                    str(tmp_path / "pred.bin"))
    gpu.decrypt_files(os.path.join(d, "keys.bin"), str(tmp_path / "pred.bin"), str(tmp_path / "out.csv"), True)
    got = open(tmp_path / "out.csv").read().splitlines()
    want = open(os.path.join(d, "result_bypos.csv")).read().splitlines()
    assert got[0] == want[0] and len(got) == len(want)
    diffs = []
    for g, w in zip(got[1:], want[1:]):
        gs, ws = g.split(","), w.split(",")
        assert gs[:2] == ws[:2]
        for x, y in zip(gs[2:], ws[2:]):
            d = abs((float(x) - float(y) + 0.5) % 1.0 - 0.5)
            # two independent noises of sd 2^-25 * sqrt(sum w^2) each, with
            # |w| <= 8192 and 15 terms: at most 1.4e-3 together; 7 sd below 1e-2
            assert d < 1e-2, (g, w)
            diffs.append(d)
    assert np.sqrt(np.mean(np.square(diffs))) < 1.5e-3  # no systematic offset


def test_encrypt_cli_is_reproducible_with_a_seed(tmp_path):
    d = os.path.join(GOLDEN, "ref_r10")
    shutil.copy(os.path.join(d, "keys.bin"), tmp_path / "keys.bin")
    exe = os.path.join(ROOT, "idash2019_2_gb300", "idash_encrypt")
    env = dict(os.environ, IDASH_SEED="31337")
    r = subprocess.run([exe, os.path.join(d, "tags.txt")], cwd=tmp_path, env=env, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "encrypt wall time" in r.stdout
    gpu.encrypt_files(str(tmp_path / "keys.bin"), os.path.join(d, "tags.txt"), str(tmp_path / "api.bin"), seed=31337)
    assert filecmp.cmp(tmp_path / "encrypted_data.bin", tmp_path / "api.bin", shallow=False)


@pytest.mark.parametrize("n", [16, 32, 256, 2048])
def test_encrypt_polynomial_sizes(ctx, oracle, n):
    """Fresh encryptions at other polynomial sizes (binary keys: N a multiple
    of 32 runs the register-windowed kernel, N = 16 the general one): the
    mask is the documented stream and b - a*s - m equals the reported noise."""
    rng = np.random.default_rng(n)
    ns, n_rows, seed = min(n, 20), 9, 777
    key = rng.integers(0, 2, size=n).astype(np.int32)
    geno = rng.integers(-1, 3, size=(3, ns)).astype(np.int8)
    slot_src = np.array([0, 4, 8, 0xFFFFFFFF, 2, 5, 7, 1, 3], np.uint32)
    d_src, d_geno = ctx.device_alloc(slot_src.nbytes), ctx.device_alloc(geno.nbytes)
    d_src.upload(slot_src)
    d_geno.upload(geno)
    d_out = ctx.device_alloc(n_rows * 2 * n * 4)
    d_noise = ctx.device_alloc(n_rows * n * 4)
    params = gpu.encrypt_params(ns, 1, n, N=n)
    gpu.encrypt_device(ctx, params, key, seed, n_rows, d_src.ptr, d_geno.ptr, ns, d_out.ptr,
                       gpu.RowLayout(2 * n * 4, 0, -1, -1), d_noise=d_noise.ptr)
    ctx.sync()
    rows = d_out.download(dtype=np.int32).reshape(n_rows, 2 * n)
    noise = d_noise.download(dtype=np.int32).reshape(n_rows, n)
    for r in range(n_rows):
        a = rows[r, :n].view(np.uint32)
        mask = np.array([oracle.lib().oracle_hash32(seed, 21, r * n + j) for j in range(n)], np.uint32)
        np.testing.assert_array_equal(a, mask)
        msg = np.zeros(n, np.uint32)
        if slot_src[r] != 0xFFFFFFFF:
            p, v = divmod(int(slot_src[r]), 3)
            gv = geno[p]
            val = np.where(gv == v, params.one_t32, np.where((gv < 0) | (gv > 2), params.nan_t32[v], 0))
            msg[:ns] = val.astype(np.int64).astype(np.uint32)
        ph = (rows[r, n:].view(np.uint32) - oracle.negacyclic_mul(key, a)).astype(np.uint32)
        np.testing.assert_array_equal((ph - msg).astype(np.uint32).view(np.int32), noise[r])
    for b in (d_src, d_geno, d_out, d_noise):
        b.free()
