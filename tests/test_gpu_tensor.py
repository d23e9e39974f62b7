"""The tensor-core scoring kernel (score_tc.cu: exact digit products on
tcgen05, "kernel" option 5) against the oracle, bit for bit: TRLWE dense and
record layouts, the host path, output ranges, the per-individual LWE form
with row lengths that end inside a 64-column slice, the largest coefficients
the two-digit split admits, and the magnitude bound at the largest K."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

gpu = pytest.importorskip("idash2019_2_gb300.gpu")

TC_KIND = 4  # idash_model_info.kernel of the tensor-core kernel


@pytest.fixture(scope="module")
def ctx():
    c = gpu.Context(0)
    c.set_option("kernel", 5)
    yield c
    c.set_option("kernel", 0)
    c.close()


def rows_of(seed, n_rows, words=2048):
    rng = np.random.default_rng(seed)
    return rng.integers(0, 2 ** 32, size=(n_rows, words), dtype=np.uint64).astype(np.uint32).view(np.int32)


@pytest.mark.parametrize("seed,tags,targets,k,ns", [(1, 150, 400, 5, 1000), (2, 120, 90, 30, 1024), (3, 40, 7, 1, 17)])
def test_trlwe_device_and_host(ctx, oracle, seed, tags, targets, k, ns):
    w = gpu.synth_model(seed=seed, n_tags=tags, n_targets=targets, neighbours=k)
    n_rows = 3 * tags
    rows = rows_of(seed, n_rows)
    want, _ = oracle.trlwe_score(w.model.term_ptr, w.model.term_feat, w.model.term_coef, rows, ns, 1, 1024)
    m = gpu.TrlweModel(ctx, w.model, n_rows, ns, 1, 1024)
    assert m.info()["kernel"] == TC_KIND and m.info()["slice_words"] == 64
    d_in = ctx.device_alloc(rows.nbytes)
    d_out = ctx.device_alloc(m.n_out * 8192)
    d_in.upload(rows)
    for graph in (1, 0):
        ctx.set_option("graph", graph)
        d_out.zero()
        m.score_device(d_in.ptr, gpu.DENSE_TRLWE, d_out.ptr, gpu.DENSE_TRLWE)
        ctx.sync()
        np.testing.assert_array_equal(d_out.download(dtype=np.int32).reshape(m.n_out, 2048), want)
    ctx.set_option("graph", 1)
    np.testing.assert_array_equal(m.score(rows), want)  # host path (chunked)
    for lo, hi in [(0, m.n_out), (5, min(131, m.n_out)), (m.n_out - 1, m.n_out)]:
        d_r = ctx.device_alloc((hi - lo) * 8192)
        m.score_range(lo, hi, 0, d_in.ptr, gpu.DENSE_TRLWE, 0, n_rows, d_r.ptr, gpu.DENSE_TRLWE)
        ctx.sync()
        np.testing.assert_array_equal(d_r.download(dtype=np.int32).reshape(hi - lo, 2048), want[lo:hi])
        d_r.free()
    d_in.free()
    d_out.free()
    m.free()


def test_trlwe_records_with_variance(ctx, oracle):
    w = gpu.synth_model(seed=9, n_tags=100, n_targets=250, neighbours=7)
    csr, n_rows = w.model, 300
    rows = rows_of(9, n_rows)
    var = np.random.default_rng(2).random(n_rows) * 2.0 ** -50
    rec = np.zeros((n_rows, gpu.RECORD_BYTES // 4), np.int32)
    rec[:, 2:2050] = rows
    rec[:, 2050:2052] = var.view(np.int32).reshape(n_rows, 2)
    out_index = (np.arange(csr.n_out) * 3 + 11).astype(np.uint32)
    m = gpu.TrlweModel(ctx, csr, n_rows, 1000, 1, 1024, out_index=out_index)
    assert m.info()["kernel"] == TC_KIND
    d_in = ctx.device_alloc(rec.nbytes + 16)
    d_out = ctx.device_alloc(csr.n_out * gpu.RECORD_BYTES + 16)
    d_in.upload(rec, offset=8)
    m.score_device(d_in.ptr + 8, gpu.RECORD_IN, d_out.ptr + 8, gpu.RECORD_OUT)
    ctx.sync()
    got = d_out.download(nbytes=csr.n_out * gpu.RECORD_BYTES, offset=8, dtype=np.int32).reshape(csr.n_out, -1)
    want, want_var = oracle.trlwe_score(csr.term_ptr, csr.term_feat, csr.term_coef, rows, 1000, 1, 1024, in_var=var)
    np.testing.assert_array_equal(got[:, 2:2050], want)
    np.testing.assert_array_equal(np.ascontiguousarray(got[:, 2050:2052]).view(np.float64).ravel(), want_var)
    np.testing.assert_array_equal(got[:, 0].view(np.uint32), out_index)
    d_in.free()
    d_out.free()
    m.free()


@pytest.mark.parametrize("n_indiv,choices", [(37, [5, 10, 2]), (100, [5, 10, 20, 30, 50]), (1, [5])])
def test_lwe_ranges(ctx, oracle, n_indiv, choices):
    """Rows of n_indiv * 1025 words: 37 and 1 individual end inside a
    64-column slice (scalar stores there); 100 fill whole slices except the
    last."""
    n, n_tags = 1024, 200
    w = gpu.synth_model(seed=n_indiv, n_tags=n_tags, n_targets=150, choices=choices)
    n_feat = 3 * n_tags
    stride = gpu.lwe_row_words(n_indiv, n)
    d_in = ctx.device_alloc(n_feat * stride * 4)
    gpu.synth_lwe_device(ctx, 77, n, n_indiv, n_feat, d_in.ptr, stride)
    ctx.sync()
    rows = d_in.download(dtype=np.int32).reshape(n_feat, stride)
    m = gpu.LweModel(ctx, w.model, n_feat, n_indiv, n)
    for (lo, hi, ni) in [(0, m.n_out, n_indiv), (5, 131, n_indiv), (100, 101, n_indiv),
                         (0, m.n_out, max(1, n_indiv // 3))]:
        ostride = gpu.lwe_row_words(ni, n)
        d_out = ctx.device_alloc((hi - lo) * ostride * 4)
        m.score_device(ni, d_in.ptr, stride, lo, hi, d_out.ptr, ostride)
        ctx.sync()
        got = d_out.download(dtype=np.int32).reshape(hi - lo, ostride)[:, :ni * (n + 1)]
        sub = rows if ni == n_indiv else np.ascontiguousarray(rows[:, :ni * (n + 1)])
        want = oracle.lwe_score(w.model.term_ptr, w.model.term_feat, w.model.term_coef, sub, ni, lo, hi, n=n)
        np.testing.assert_array_equal(got, want)
        d_out.free()
    assert m.info()["kernel"] == TC_KIND
    m.free()
    d_in.free()


def _dense_model(n_out, n_rows, coef_fn, const=None):
    ptr = np.arange(n_out + 1, dtype=np.uint64) * (n_rows + (1 if const is not None else 0))
    feat, coef = [], []
    for o in range(n_out):
        feat += list(range(n_rows))
        coef += [coef_fn(o, r) for r in range(n_rows)]
        if const is not None:
            feat.append(0xFFFFFFFF)
            coef.append(const)
    return gpu.CSRModel(ptr, np.array(feat, np.uint32), np.array(coef, np.int64).astype(np.int32))


@pytest.mark.parametrize("c_pos,c_neg,k_rows", [
    (8064, -8320, 192),     # c0 = -128, |c1| = 32: K up to 192
    (32640, -32896, 112),   # c0 = -128, |c1| = 128: K up to 112
])
def test_extreme_digits_at_the_largest_k(ctx, oracle, c_pos, c_neg, k_rows):
    """Coefficients whose digits are at the extremes of the two-digit split,
    ciphertext words whose four digits are all -128 (0x7F7F7F80) or all 127
    (0x7F7F7F7F), over the largest K the exactness bound admits for that
    coefficient range: the accumulators reach about 94% of the 2^22 bound."""
    n_out = 130  # two blocks, the second of two outputs
    csr = _dense_model(n_out, k_rows, lambda o, r: c_neg if (o + r) % 7 else c_pos, const=-1)
    rows = np.full((k_rows, 2048), 0x7F7F7F80, np.uint32)
    rows[::5] = 0x7F7F7F7F
    rows = rows.view(np.int32)
    want, _ = oracle.trlwe_score(csr.term_ptr, csr.term_feat, csr.term_coef, rows, 1000, 1, 1024)
    m = gpu.TrlweModel(ctx, csr, k_rows, 1000, 1, 1024)
    assert m.info()["kernel"] == TC_KIND
    np.testing.assert_array_equal(m.score(rows), want)
    m.free()


def test_coefficients_beyond_two_digits_use_the_other_kernels(ctx, oracle):
    """A coefficient needing a third base-256 digit (the reference allows any
    int32) makes the tensor-core plan infeasible: the model is planned for
    another kernel and stays exact."""
    csr = _dense_model(6, 20, lambda o, r: 2_000_000_000 if r == 3 else 5)
    rows = rows_of(4, 20)
    for option in (5, 0):
        ctx.set_option("kernel", option)
        try:
            m = gpu.TrlweModel(ctx, csr, 20, 1000, 1, 1024)
            want, _ = oracle.trlwe_score(csr.term_ptr, csr.term_feat, csr.term_coef, rows, 1000, 1, 1024)
            np.testing.assert_array_equal(m.score(rows), want)
            assert m.info()["kernel"] != TC_KIND
            m.free()
        finally:
            ctx.set_option("kernel", 5)
