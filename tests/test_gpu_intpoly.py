"""Integer-polynomial x TRLWE scoring (two-prime NTT + CRT) against the
oracle's exact schoolbook product, bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

gpu = pytest.importorskip("idash2019_2_gb300.gpu")


@pytest.fixture(scope="module")
def ctx():
    c = gpu.Context(0)
    yield c
    c.close()


def _case(seed, n_out, n_rows, max_terms, max_abs=8192):
    rng = np.random.default_rng(seed)
    counts = rng.integers(1, max_terms + 1, size=n_out)
    ptr = np.concatenate([[0], np.cumsum(counts)]).astype(np.uint64)
    feat = rng.integers(0, n_rows, size=int(ptr[-1])).astype(np.uint32)
    poly = rng.integers(-max_abs, max_abs, size=(int(ptr[-1]), 1024)).astype(np.int16)
    rows = rng.integers(0, 2 ** 32, size=(n_rows, 2048), dtype=np.uint64).astype(np.uint32).view(np.int32)
    bias = rng.integers(-8192, 8192, size=n_out).astype(np.int32)
    return gpu.CSRModel(ptr, feat, np.zeros(int(ptr[-1]), np.int32)), poly, rows, bias


@pytest.mark.parametrize("seed,n_out,max_terms,ns,rs", [(1, 9, 4, 1000, 1024), (2, 7, 60, 700, 900)])
def test_intpoly_matches_schoolbook(ctx, oracle, seed, n_out, max_terms, ns, rs):
    csr, poly, rows, bias = _case(seed, n_out, 40, max_terms)
    m = gpu.IntpolyModel(ctx, csr, poly, 40, ns, rs, bias=bias)
    d_in = ctx.device_alloc(rows.nbytes)
    d_in.upload(rows)
    d_out = ctx.device_alloc(n_out * 8192)
    m.score_device(d_in.ptr, gpu.DENSE_TRLWE, 0, n_out, d_out.ptr, gpu.DENSE_TRLWE)
    ctx.sync()
    got = d_out.download(dtype=np.int32).reshape(n_out, 2048)
    want = oracle.intpoly_score(csr.term_ptr, csr.term_feat, poly, bias, rows, ns, rs, 0, n_out)
    np.testing.assert_array_equal(got, want)
    # a sub-range lands at row (o - out_begin)
    d_out.zero()
    m.score_device(d_in.ptr, gpu.DENSE_TRLWE, 2, 5, d_out.ptr, gpu.DENSE_TRLWE)
    ctx.sync()
    np.testing.assert_array_equal(d_out.download(nbytes=3 * 8192, dtype=np.int32).reshape(3, 2048), want[2:5])
    m.free()


def test_intpoly_output_groups_and_ranges(ctx, oracle):
    """Outputs that read the same rows in the same order (a target's three
    genotype models) are scored together; groups of 3, 2 and 1, an empty
    output, and ranges that cut groups in the middle all stay exact."""
    rng = np.random.default_rng(7)
    n_rows, lists = 30, []
    for size in (3, 1, 2, 3, 3, 1, 3):
        rows_of = rng.integers(0, n_rows, size=int(rng.integers(1, 25))).astype(np.uint32)
        lists += [rows_of] * size
    lists[4] = np.zeros(0, np.uint32)  # an output with no terms inside a would-be group
    ptr = np.concatenate([[0], np.cumsum([len(x) for x in lists])]).astype(np.uint64)
    feat = np.concatenate(lists).astype(np.uint32)
    poly = rng.integers(-8192, 8192, size=(len(feat), 1024)).astype(np.int16)
    rows = rng.integers(0, 2 ** 32, size=(n_rows, 2048), dtype=np.uint64).astype(np.uint32).view(np.int32)
    bias = rng.integers(-8192, 8192, size=len(lists)).astype(np.int32)
    n_out = len(lists)
    csr = gpu.CSRModel(ptr, feat, np.zeros(len(feat), np.int32))
    m = gpu.IntpolyModel(ctx, csr, poly, n_rows, 1000, 1024, bias=bias)
    want = oracle.intpoly_score(ptr, feat, poly, bias, rows, 1000, 1024, 0, n_out)
    d_in = ctx.device_alloc(rows.nbytes)
    d_in.upload(rows)
    for lo, hi in [(0, n_out), (1, 8), (4, 5), (5, n_out), (n_out - 1, n_out)]:
        d_out = ctx.device_alloc((hi - lo) * 8192)
        m.score_device(d_in.ptr, gpu.DENSE_TRLWE, lo, hi, d_out.ptr, gpu.DENSE_TRLWE)
        ctx.sync()
        np.testing.assert_array_equal(d_out.download(dtype=np.int32).reshape(hi - lo, 2048), want[lo:hi])
        d_out.free()
    d_in.free()
    m.free()


def test_constant_polynomials_equal_the_trlwe_form(ctx):
    """With every weight a constant polynomial, the product is the reference's
    tLweAddMulTo sum: the two kernels agree."""
    w = gpu.synth_model(seed=12, n_tags=60, n_targets=50, neighbours=5)
    csr = w.model
    rows = np.random.default_rng(3).integers(0, 2 ** 32, size=(180, 2048), dtype=np.uint64).astype(
        np.uint32).view(np.int32)
    want = gpu.TrlweModel(ctx, csr, 180, 1000, 1, 1024).score(rows)
    # split off the constant terms as the per-output bias
    ptr, feat, coef, bias, polys = [0], [], [], [], []
    for o in range(csr.n_out):
        b = 0
        for t in range(int(csr.term_ptr[o]), int(csr.term_ptr[o + 1])):
            if csr.term_feat[t] == 0xFFFFFFFF:
                b += int(csr.term_coef[t])
            else:
                feat.append(int(csr.term_feat[t]))
                p = np.zeros(1024, np.int16)
                p[0] = csr.term_coef[t]
                polys.append(p)
        bias.append(b)
        ptr.append(len(feat))
    icsr = gpu.CSRModel(np.array(ptr, np.uint64), np.array(feat, np.uint32), np.zeros(len(feat), np.int32))
    m = gpu.IntpolyModel(ctx, icsr, np.array(polys), 180, 1000, 1024, bias=np.array(bias, np.int32))
    d_in = ctx.device_alloc(rows.nbytes)
    d_in.upload(rows)
    d_out = ctx.device_alloc(csr.n_out * 8192)
    m.score_device(d_in.ptr, gpu.DENSE_TRLWE, 0, csr.n_out, d_out.ptr, gpu.DENSE_TRLWE)
    ctx.sync()
    np.testing.assert_array_equal(d_out.download(dtype=np.int32).reshape(csr.n_out, 2048), want)


def test_exactness_bounds_are_enforced(ctx):
    csr, poly, rows, bias = _case(5, 2, 10, 3)
    too_many = gpu.CSRModel(np.array([0, 200], np.uint64), np.zeros(200, np.uint32), np.zeros(200, np.int32))
    with pytest.raises(gpu.IdashError) as e:
        gpu.IntpolyModel(ctx, too_many, np.zeros((200, 1024), np.int16), 10, 1000, 1024)
    assert e.value.name == "IDASH_ERR_UNSUPPORTED"
    big = poly.copy()
    big[0, 5] = 9000  # beyond max_abs_coef = 8192
    with pytest.raises(gpu.IdashError):
        gpu.IntpolyModel(ctx, csr, big, 10, 1000, 1024)
    ctx.sync()


def test_set_weights_replaces_the_resident_transform(ctx, oracle):
    """New weights for the same terms, transformed on the device in place:
    the next product equals the schoolbook product with the new weights, and
    setting the first weights back restores the first result."""
    csr, poly, rows, bias = _case(5, 6, 20, 12)
    m = gpu.IntpolyModel(ctx, csr, poly, 20, 1000, 1024, bias=bias)
    poly2 = np.random.default_rng(6).integers(-8192, 8192, size=poly.shape).astype(np.int16)
    d_in = ctx.device_alloc(rows.nbytes)
    d_in.upload(rows)
    d_out = ctx.device_alloc(6 * 8192)
    d_poly = ctx.device_alloc(poly.nbytes)
    try:
        for weights in (poly2, poly):
            d_poly.upload(weights)
            m.set_weights(d_poly.ptr)
            m.score_device(d_in.ptr, gpu.DENSE_TRLWE, 0, 6, d_out.ptr, gpu.DENSE_TRLWE)
            ctx.sync()
            want = oracle.intpoly_score(csr.term_ptr, csr.term_feat, weights, bias, rows, 1000, 1024, 0, 6)
            np.testing.assert_array_equal(d_out.download(dtype=np.int32).reshape(6, 2048), want)
    finally:
        for b in (d_in, d_out, d_poly):
            b.free()
        m.free()
