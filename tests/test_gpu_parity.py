"""GPU parity: the CUDA path (through the C ABI) against the reference's own
outputs and the oracle, bit for bit.  Run on a GB300 after build()."""
import filecmp
import hashlib
import json
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


def copy_case(name, dst):
    src = os.path.join(GOLDEN, name)
    for f in ["params.bin", "encrypted_data.bin"]:
        shutil.copy(os.path.join(src, f), dst / f)
    shutil.copytree(os.path.join(src, "model"), dst / "model")
    return src


@pytest.mark.parametrize("name", SMALL_CASES)
def test_cloud_files_byte_identical_to_reference(tmp_path, name):
    """The whole cloud step on the reference's own fixture files writes an
    encrypted_prediction.bin identical byte for byte to the reference's."""
    src = copy_case(name, tmp_path)
    rep = gpu.cloud_files(str(tmp_path / "params.bin"), str(tmp_path / "model"), str(tmp_path / "encrypted_data.bin"),
                          str(tmp_path / "encrypted_prediction.bin"))
    assert rep["n_out_records"] > 0
    assert filecmp.cmp(tmp_path / "encrypted_prediction.bin", os.path.join(src, "encrypted_prediction.bin"),
                       shallow=False)


@pytest.mark.parametrize("name", ["rand_r1_i1000", "rand_r4_i250", "rand_r10_i100"])
def test_cloud_files_hash_pinned_medium(tmp_path, name):
    import gen_inputs
    meta = json.load(open(os.path.join(GOLDEN, "hashes.json")))[name]
    gen_inputs.write_random_case(str(tmp_path), **{k: meta[k] for k in
                                                  ("seed", "n_indiv", "n_tags", "n_targets", "neighbours")})
    gpu.cloud_files(str(tmp_path / "params.bin"), str(tmp_path / "model"), str(tmp_path / "encrypted_data.bin"),
                    str(tmp_path / "encrypted_prediction.bin"))
    raw = open(tmp_path / "encrypted_prediction.bin", "rb").read()
    assert len(raw) == meta["bytes"]
    assert hashlib.sha256(raw).hexdigest() == meta["sha256"]


def test_model_cache_is_written_then_used(tmp_path, monkeypatch):
    """IDASH_MODEL_CACHE: the first run parses the .hr files and writes the
    flattened model; the second reads it; both outputs equal the reference's."""
    src = copy_case("ref_r3_edge", tmp_path)
    monkeypatch.setenv("IDASH_MODEL_CACHE", str(tmp_path / "model.cache"))
    plan = tmp_path / "model.cache.plan"
    for expect_cached in (0, 1):
        out = tmp_path / f"pred{expect_cached}.bin"
        rep = gpu.cloud_files(str(tmp_path / "params.bin"), str(tmp_path / "model"),
                              str(tmp_path / "encrypted_data.bin"), str(out))
        assert rep["model_from_cache"] == expect_cached
        assert filecmp.cmp(out, os.path.join(src, "encrypted_prediction.bin"), shallow=False)
        # the first run records the tuned plan (magic, fingerprint, kernel kind, slice width)
        raw = plan.read_bytes()
        assert len(raw) == 32 and raw[:8] == b"IDGPLAN1"
        kind, slice_words = np.frombuffer(raw[16:], np.uint64)
        assert (kind <= 3 and slice_words in (128, 256, 512, 1024, 2048)) or (kind == 4 and slice_words == 64)
    # a damaged plan file is ignored and replaced
    plan.write_bytes(b"IDGPLAN1" + b"\xff" * 24)
    rep = gpu.cloud_files(str(tmp_path / "params.bin"), str(tmp_path / "model"),
                          str(tmp_path / "encrypted_data.bin"), str(tmp_path / "pred_p.bin"))
    assert filecmp.cmp(tmp_path / "pred_p.bin", os.path.join(src, "encrypted_prediction.bin"), shallow=False)
    assert plan.read_bytes()[8:16] != b"\xff" * 8
    # a cache for other params is ignored (and replaced)
    (tmp_path / "params2.bin").write_bytes((tmp_path / "params.bin").read_bytes())
    rep = gpu.cloud_files(str(tmp_path / "params2.bin"), str(tmp_path / "model"),
                          str(tmp_path / "encrypted_data.bin"), str(tmp_path / "pred2.bin"))
    assert rep["model_from_cache"] == 1  # same bytes, same directory: same fingerprint
    (tmp_path / "model.cache").write_bytes(b"IDASHFM1" + b"\0" * 40)
    rep = gpu.cloud_files(str(tmp_path / "params.bin"), str(tmp_path / "model"),
                          str(tmp_path / "encrypted_data.bin"), str(tmp_path / "pred3.bin"))
    assert rep["model_from_cache"] == 0
    assert filecmp.cmp(tmp_path / "pred3.bin", os.path.join(src, "encrypted_prediction.bin"), shallow=False)


def test_cloud_cli_matches_reference(tmp_path):
    src = copy_case("ref_r10", tmp_path)
    cli = os.path.join(ROOT, "idash2019_2_gb300", "idash_cloud")
    r = subprocess.run([cli, "model"], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "fhe wall time (seconds)" in r.stdout and "BENCHMARK" in r.stdout
    assert filecmp.cmp(tmp_path / "encrypted_prediction.bin", os.path.join(src, "encrypted_prediction.bin"),
                       shallow=False)


def random_rows(seed, n_rows, n=1024):
    rng = np.random.default_rng(seed)
    return rng.integers(0, 2 ** 32, size=(n_rows, 2 * n), dtype=np.uint64).astype(np.uint32).view(np.int32)


@pytest.mark.parametrize("regions", [1, 3, 10])
@pytest.mark.parametrize("kernel", [0, 1])
def test_trlwe_synth_vs_oracle(ctx, oracle, regions, kernel):
    num_samples = 1024 // regions - 1 if regions > 1 else 1000
    region_size = 1024 // regions
    w = gpu.synth_model(seed=7 + regions, n_tags=150, n_targets=400, neighbours=5)
    n_rows = (3 * 150 + regions - 1) // regions
    rows = random_rows(regions, n_rows)
    ctx.set_option("kernel", kernel)
    try:
        m = gpu.TrlweModel(ctx, w.model, n_rows, num_samples, regions, region_size)
        got = m.score(rows)
        m.free()
    finally:
        ctx.set_option("kernel", 0)
    want, _ = oracle.trlwe_score(w.model.term_ptr, w.model.term_feat, w.model.term_coef, rows, num_samples,
                                 regions, region_size)
    np.testing.assert_array_equal(got, want)


KIND_OF_OPTION = {2: 0, 3: 2, 4: 3}  # "kernel" option -> idash_model_info.kernel


@pytest.mark.parametrize("slice_words", [128, 256, 512, 1024, 2048])
@pytest.mark.parametrize("kernel,graph", [(2, 0), (2, 1), (3, 1), (4, 0), (4, 1)])
def test_trlwe_device_path_tiles(ctx, oracle, slice_words, kernel, graph):
    """Every slice width of the single-buffer (2) and double-buffer (3)
    persistent kernels, with and without graph replay, on the
    device-resident path (dense rows).  At most 3 neighbours (9 slots) so that
    even a double-buffered 2048-word window (10 slots) holds every output."""
    w = gpu.synth_model(seed=3, n_tags=200, n_targets=700, choices=[3, 2, 1])
    n_rows = 600
    rows = random_rows(5, n_rows)
    ctx.set_option("slice_words", slice_words)
    ctx.set_option("graph", graph)
    ctx.set_option("kernel", kernel)
    try:
        m = gpu.TrlweModel(ctx, w.model, n_rows, 1000, 1, 1024)
        d_in = ctx.device_alloc(rows.nbytes)
        d_out = ctx.device_alloc(m.n_out * 8192)
        d_in.upload(rows)
        for _ in range(2):  # second call replays the graph
            d_out.zero()
            m.score_device(d_in.ptr, gpu.DENSE_TRLWE, d_out.ptr, gpu.DENSE_TRLWE)
            ctx.sync()
            got = d_out.download(dtype=np.int32).reshape(m.n_out, 2048)
            want, _ = oracle.trlwe_score(w.model.term_ptr, w.model.term_feat, w.model.term_coef, rows, 1000, 1,
                                         1024)
            np.testing.assert_array_equal(got, want)
        assert m.info()["slice_words"] == slice_words
        assert m.info()["kernel"] == KIND_OF_OPTION[kernel]
        m.free()
    finally:
        ctx.set_option("slice_words", 0)
        ctx.set_option("graph", 1)
        ctx.set_option("kernel", 0)


@pytest.mark.parametrize("kernel", [2, 3, 4])
def test_trlwe_regions_persistent_kernels(ctx, oracle, kernel):
    """NUM_REGIONS = 10 (rotated slots gathered in shared memory) on both
    persistent kernels with a graph."""
    w = gpu.synth_model(seed=17, n_tags=150, n_targets=400, neighbours=6)
    n_rows = (3 * 150 + 9) // 10
    rows = random_rows(17, n_rows)
    ctx.set_option("kernel", kernel)
    try:
        m = gpu.TrlweModel(ctx, w.model, n_rows, 100, 10, 102)
        d_in = ctx.device_alloc(rows.nbytes)
        d_out = ctx.device_alloc(m.n_out * 8192)
        d_in.upload(rows)
        m.score_device(d_in.ptr, gpu.DENSE_TRLWE, d_out.ptr, gpu.DENSE_TRLWE)
        ctx.sync()
        got = d_out.download(dtype=np.int32).reshape(m.n_out, 2048)
        m.free()
    finally:
        ctx.set_option("kernel", 0)
    want, _ = oracle.trlwe_score(w.model.term_ptr, w.model.term_feat, w.model.term_coef, rows, 100, 10, 102)
    np.testing.assert_array_equal(got, want)


def test_large_neighbourhoods_fall_back_to_direct_kernel(ctx, oracle):
    """With splitting off, 50-neighbour outputs (150 window slots) do not fit
    a 2048-word slice window; the model is planned for the direct kernel and
    stays exact."""
    w = gpu.synth_model(seed=31, n_tags=200, n_targets=300, choices=[5, 50])
    rows = random_rows(9, 600)
    ctx.set_option("slice_words", 2048)
    ctx.set_option("split", 0)
    try:
        m = gpu.TrlweModel(ctx, w.model, 600, 1000, 1, 1024)
        assert m.info()["kernel"] == 1
        got = m.score(rows)
        m.free()
    finally:
        ctx.set_option("slice_words", 0)
        ctx.set_option("split", 1)
    want, _ = oracle.trlwe_score(w.model.term_ptr, w.model.term_feat, w.model.term_coef, rows, 1000, 1, 1024)
    np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("kernel,slice_words,regions", [(2, 2048, 1), (4, 2048, 1), (4, 512, 3), (3, 1024, 10),
                                                        (2, 256, 1)])
def test_split_neighbourhoods_device_and_host(ctx, oracle, kernel, slice_words, regions):
    """Neighbourhoods of up to 150 slots with windows of a few slots: the
    plan splits them into parts whose later launches add to the outputs
    (record layout with variance, device path with and without graph, host
    path and output ranges), bit-exact to the oracle."""
    rs = 1024 // regions
    ns = min(rs, 1000) - (1 if regions > 1 else 0)
    w = gpu.synth_model(seed=37 + regions, n_tags=120, n_targets=200, choices=[5, 50, 1, 20])
    n_rows = (3 * 120 + regions - 1) // regions
    rows = random_rows(11 + regions, n_rows)
    ctx.set_option("kernel", kernel)
    ctx.set_option("slice_words", slice_words)
    ctx.set_option("max_window_slots", 24)
    try:
        m = gpu.TrlweModel(ctx, w.model, n_rows, ns, regions, rs)
        want, _ = oracle.trlwe_score(w.model.term_ptr, w.model.term_feat, w.model.term_coef, rows, ns, regions, rs)
        for graph in (1, 0):
            ctx.set_option("graph", graph)
            np.testing.assert_array_equal(m.score(rows), want)
        info = m.info()
        assert info["kernel"] == KIND_OF_OPTION[kernel] and info["max_window_slots"] <= 24
        # host path (chunked, phases per chunk)
        lay = gpu.DENSE_TRLWE
        h_in, h_out = ctx.host_alloc(rows.nbytes), ctx.host_alloc(m.n_out * 8192)
        h_in.array[:] = rows.view(np.uint8).reshape(-1)
        m.score_host(h_in.ptr, lay, n_rows, h_out.ptr, lay)
        np.testing.assert_array_equal(np.frombuffer(h_out.array, np.int32).reshape(m.n_out, 2048), want)
        # output ranges
        d_in = ctx.device_alloc(rows.nbytes)
        d_in.upload(rows)
        for lo, hi in [(0, m.n_out), (7, 100), (301, 302)]:
            d_out = ctx.device_alloc((hi - lo) * 8192)
            m.score_range(lo, hi, 0, d_in.ptr, lay, 0, n_rows, d_out.ptr, lay)
            ctx.sync()
            np.testing.assert_array_equal(d_out.download(dtype=np.int32).reshape(hi - lo, 2048), want[lo:hi])
            d_out.free()
        d_in.free()
        h_in.free()
        h_out.free()
        m.free()
    finally:
        ctx.set_option("kernel", 0)
        ctx.set_option("slice_words", 0)
        ctx.set_option("max_window_slots", 0)
        ctx.set_option("graph", 1)


def test_trlwe_autotune_picks_a_correct_plan(ctx, oracle):
    w = gpu.synth_model(seed=4, n_tags=300, n_targets=1500, neighbours=5)
    rows = random_rows(6, 900)
    m = gpu.TrlweModel(ctx, w.model, 900, 1000, 1, 1024)
    got = m.score(rows)  # first call autotunes
    got2 = m.score(rows)
    want, _ = oracle.trlwe_score(w.model.term_ptr, w.model.term_feat, w.model.term_coef, rows, 1000, 1, 1024)
    np.testing.assert_array_equal(got, want)
    np.testing.assert_array_equal(got2, want)
    info = m.info()
    # a batched kind: window, pipe or warp-specialised at a TRLWE slice width,
    # or the tensor-core kernel at its 64-word slices
    assert (info["kernel"] in (0, 2, 3) and info["slice_words"] in (512, 1024, 2048)) or \
        (info["kernel"] == 4 and info["slice_words"] == 64)


@pytest.mark.parametrize("kernel,slice_words,split", [(0, 0, 1), (2, 128, 1), (3, 256, 1), (3, 512, 1), (1, 256, 1),
                                                      (4, 256, 1), (4, 512, 1), (4, 1024, 1), (4, 1024, 0)])
def test_lwe_vs_oracle_ranges(ctx, oracle, kernel, slice_words, split):
    # (4, 1024): a 10-neighbour output needs 30 slots of 4 KiB, more than one
    # ring stage holds: the plan splits it into parts, or, with splitting
    # off, falls back to the direct kernel.
    n, n_indiv, n_tags = 1024, 37, 60
    w = gpu.synth_model(seed=9, n_tags=n_tags, n_targets=90, choices=[5, 10, 2])
    n_feat = 3 * n_tags
    stride = gpu.lwe_row_words(n_indiv, n)
    d_in = ctx.device_alloc(n_feat * stride * 4)
    gpu.synth_lwe_device(ctx, 77, n, n_indiv, n_feat, d_in.ptr, stride)
    ctx.sync()
    rows = d_in.download(dtype=np.int32).reshape(n_feat, stride)
    ctx.set_option("kernel", kernel)
    ctx.set_option("slice_words", slice_words)
    ctx.set_option("split", split)
    try:
        m = gpu.LweModel(ctx, w.model, n_feat, n_indiv, n)
        for (lo, hi, ni) in [(0, m.n_out, n_indiv), (5, 131, n_indiv), (100, 101, n_indiv), (0, m.n_out, 11)]:
            ostride = gpu.lwe_row_words(ni, n)
            d_out = ctx.device_alloc((hi - lo) * ostride * 4)
            m.score_device(ni, d_in.ptr, stride, lo, hi, d_out.ptr, ostride)
            ctx.sync()
            got = d_out.download(dtype=np.int32).reshape(hi - lo, ostride)[:, :ni * (n + 1)]
            sub = rows if ni == n_indiv else np.ascontiguousarray(rows[:, :ni * (n + 1)])
            want = oracle.lwe_score(w.model.term_ptr, w.model.term_feat, w.model.term_coef, sub, ni, lo, hi, n=n)
            np.testing.assert_array_equal(got, want)
            d_out.free()
        if (kernel, slice_words, split) == (4, 1024, 0):
            assert m.info()["kernel"] == 1
        elif slice_words:
            assert m.info()["slice_words"] == slice_words
        m.free()
    finally:
        ctx.set_option("kernel", 0)
        ctx.set_option("slice_words", 0)
        ctx.set_option("split", 1)
    d_in.free()


def test_synth_lwe_matches_oracle_generator(ctx, oracle):
    n, n_indiv, n_feat = 1024, 5, 9
    stride = gpu.lwe_row_words(n_indiv, n)
    d = ctx.device_alloc(n_feat * stride * 4)
    gpu.synth_lwe_device(ctx, 1234, n, n_indiv, n_feat, d.ptr, stride)
    ctx.sync()
    rows = d.download(dtype=np.int32).reshape(n_feat, stride)
    for f in (0, 4, 8):
        want = oracle.synth_lwe_words(1234, n, n_indiv, f, 0, n_indiv * (n + 1))
        np.testing.assert_array_equal(rows[f, :n_indiv * (n + 1)], want)


def test_lwe_equals_sample_extract_of_trlwe(ctx, oracle):
    """Per-individual LWE scoring of SampleExtract_i(inputs) equals
    SampleExtract_i of the TRLWE scoring: the two layouts agree."""
    n_tags, n_indiv = 40, 6
    w = gpu.synth_model(seed=21, n_tags=n_tags, n_targets=30, neighbours=5)
    rows = random_rows(8, 3 * n_tags)
    m = gpu.TrlweModel(ctx, w.model, 3 * n_tags, n_indiv, 1, 1024)
    trl = m.score(rows)
    stride = gpu.lwe_row_words(n_indiv)
    lwe_in = np.zeros((3 * n_tags, stride), np.int32)
    for f in range(3 * n_tags):
        for i in range(n_indiv):
            lwe_in[f, i * 1025:(i + 1) * 1025] = oracle.sample_extract(rows[f], i)
    lm = gpu.LweModel(ctx, w.model, 3 * n_tags, n_indiv)
    d_in = ctx.device_alloc(lwe_in.nbytes)
    d_in.upload(lwe_in)
    d_out = ctx.device_alloc(lm.n_out * stride * 4)
    lm.score_device(n_indiv, d_in.ptr, stride, 0, lm.n_out, d_out.ptr, stride)
    ctx.sync()
    got = d_out.download(dtype=np.int32).reshape(lm.n_out, stride)
    for o in range(0, lm.n_out, 7):
        for i in range(n_indiv):
            np.testing.assert_array_equal(got[o, i * 1025:(i + 1) * 1025], oracle.sample_extract(trl[o], i))


def test_errors_are_statuses(ctx):
    w = gpu.synth_model(seed=1, n_tags=20, n_targets=10, neighbours=5)
    with pytest.raises(gpu.IdashError) as e:
        gpu.TrlweModel(ctx, w.model, 10, 1000, 1, 1024)  # features beyond 10 rows
    assert e.value.name == "IDASH_ERR_INDEX"
    with pytest.raises(gpu.IdashError) as e:
        gpu.TrlweModel(ctx, w.model, 60, 1000, 2, 1024)  # 2 * 1024 > N
    assert e.value.name == "IDASH_ERR_INVALID_ARGUMENT"
    m = gpu.TrlweModel(ctx, w.model, 60, 1000, 1, 1024)
    d = ctx.device_alloc(61 * 8192)
    bad = gpu.RowLayout(8200, 0, -1, -1)  # stride not a multiple of 16
    with pytest.raises(gpu.IdashError) as e:
        m.score_device(d.ptr, bad, d.ptr, gpu.DENSE_TRLWE)
    assert e.value.name == "IDASH_ERR_INVALID_ARGUMENT"
    with pytest.raises(gpu.IdashError):
        m.score_device(d.ptr + 4, gpu.DENSE_TRLWE, d.ptr, gpu.DENSE_TRLWE)  # misaligned payload
    ctx.sync()
