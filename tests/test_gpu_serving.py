"""Serving (idash_serve_trlwe): continuous batching of imputation requests
against one resident model.  Each request's result is the same alone and in
the mix (bit for bit), the mix really overlaps requests on the device, the
outputs match the oracle, and requests beyond the HBM budget are refused."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

gpu = pytest.importorskip("idash2019_2_gb300.gpu")


@pytest.fixture(scope="module")
def served():
    ctx = gpu.Context(0)
    w = gpu.synth_model(seed=77, n_tags=300, n_targets=1000, neighbours=10)
    m = gpu.TrlweModel(ctx, w.model, 900, 1024, 1, 1024)
    rng = np.random.default_rng(5)
    reqs = []
    for i in range(10):
        length = int(rng.integers(20, 400))
        t0 = int(rng.integers(0, 1000 - length))
        # arriving together: four are admitted at once and share the device
        reqs.append(dict(arrival_s=0.0, n_indiv=int(rng.integers(1, 2600)), target_begin=t0,
                         target_end=t0 + length, seed=1000 + i))
    res, outs = m.serve(reqs, hbm_budget=2 << 30, max_inflight=4, keep_outputs=True)
    yield ctx, w, m, reqs, res, outs
    ctx.close()


def test_each_request_is_the_same_alone_and_in_the_mix(served):
    ctx, w, m, reqs, res, outs = served
    for i, r in enumerate(reqs):
        res1, out1 = m.serve([dict(r, arrival_s=0.0)], hbm_budget=2 << 30, max_inflight=1, keep_outputs=True)
        np.testing.assert_array_equal(outs[i], out1[0])
        assert res[i]["digest"] == res1[0]["digest"]


def test_digests_restate_on_the_host(served):
    ctx, w, m, reqs, res, outs = served
    lib = ctx.lib
    import ctypes as C
    for i in (0, 3):
        words = np.ascontiguousarray(outs[i]).view(np.uint32).ravel()
        d = lib.idash_digest_host(words.ctypes.data_as(C.POINTER(C.c_uint32)), words.size, 0)
        assert d == res[i]["digest"]


@pytest.mark.parametrize("slice_words", [128, 512])
def test_fused_digest_of_the_warp_specialised_kernel(served, slice_words):
    """With the warp-specialised kernel the scoring kernel takes the digest as
    it stores the outputs (no separate pass).  Its digests equal the host
    restatement over the outputs and the autotuned model's digests, and the
    outputs are the same."""
    ctx, w, m, reqs, res, outs = served
    import ctypes as C
    pick = (0, 2, 5)  # request 2 spans several TRLWE blocks (over 1,024 individuals)
    ctx.set_option("kernel", 4)
    ctx.set_option("slice_words", slice_words)
    try:
        m2 = gpu.TrlweModel(ctx, w.model, 900, 1024, 1, 1024)
        assert m2.info()["kernel"] == 3
        res2, outs2 = m2.serve([dict(reqs[i], arrival_s=0.0) for i in pick], hbm_budget=2 << 30, max_inflight=2,
                               keep_outputs=True)
        m2.free()
    finally:
        ctx.set_option("kernel", 0)
        ctx.set_option("slice_words", 0)
    assert sum(reqs[i]["n_indiv"] > 1024 for i in pick) >= 1
    for j, i in enumerate(pick):
        np.testing.assert_array_equal(outs2[j], outs[i])
        words = np.ascontiguousarray(outs2[j]).view(np.uint32).ravel()
        d = ctx.lib.idash_digest_host(words.ctypes.data_as(C.POINTER(C.c_uint32)), words.size, 0)
        assert d == res2[j]["digest"] == res[i]["digest"]


def _mix64(z):
    z = z + np.uint64(0x9E3779B97F4A7C15)
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


@pytest.mark.parametrize("row_words,stride,offset", [(2048, 8192, 0), (2046, 8196, 0), (2048, 8192, 4)])
def test_uniform_rows_restate_on_the_host(served, row_words, stride, offset):
    """The request ciphertext generator (16-byte stores on 16-byte aligned
    rows, 4-byte stores otherwise) against a numpy restatement: word j of
    global row r is the high half of mix64(key ^ (r * row_words + j)), with
    key = mix64(seed + mix64(7))."""
    ctx = served[0]
    seed, row_begin, n_rows = 0x1234567890ABCDEF, 37, 5
    d = ctx.device_alloc(n_rows * stride + 16)
    d.zero()
    gpu.synth_uniform_device(ctx, seed, row_begin, n_rows, row_words, d.ptr + offset, stride)
    ctx.sync()
    raw = d.download(dtype=np.uint8)[offset:offset + n_rows * stride].view(np.uint32).reshape(n_rows, stride // 4)
    d.free()
    with np.errstate(over="ignore"):
        key = _mix64(np.uint64(seed) + _mix64(np.uint64(7)))
        idx = (np.arange(row_begin, row_begin + n_rows, dtype=np.uint64)[:, None] * np.uint64(row_words) +
               np.arange(row_words, dtype=np.uint64)[None, :])
        want = (_mix64(key ^ idx) >> np.uint64(32)).astype(np.uint32)
    np.testing.assert_array_equal(raw[:, :row_words], want)
    assert not raw[:, row_words:].any()  # the stride's padding is untouched


def test_the_mix_overlaps_requests(served):
    ctx, w, m, reqs, res, outs = served
    spans = sorted((r["admit_s"], r["done_s"]) for r in res)
    most = max(sum(1 for a, d in spans if a <= t < d) for t, _ in spans)
    assert most >= 2, spans
    assert all(r["done_s"] >= r["admit_s"] - 1e-3 for r in res)


def test_every_served_request_matches_the_oracle(served, oracle):
    """Every request of the mix, every individual block, word for word."""
    ctx, w, m, reqs, res, outs = served
    for i in range(len(reqs)):
        r = reqs[i]
        o0, o1 = 3 * r["target_begin"], 3 * r["target_end"]
        lo, hi = m.input_rows(o0, o1)
        sub = w.model.slice_outputs(o0, o1)
        for b in range(outs[i].shape[0]):
            ns = min(1024, r["n_indiv"] - 1024 * b)
            d = ctx.device_alloc((hi - lo) * 8192)
            gpu.synth_uniform_device(ctx, gpu.request_block_seed(r["seed"], b), lo, hi - lo, 2048, d.ptr, 8192)
            ctx.sync()
            rows = np.zeros((900, 2048), np.int32)
            rows[lo:hi] = d.download(dtype=np.int32).reshape(hi - lo, 2048)
            d.free()
            want, _ = oracle.trlwe_score(sub.term_ptr, sub.term_feat, sub.term_coef, rows, ns, 1, 1024)
            np.testing.assert_array_equal(outs[i][b], want)


def test_requests_beyond_the_budget_are_refused(served):
    ctx, w, m, reqs, res, outs = served
    big = dict(arrival_s=0.0, n_indiv=3000, target_begin=0, target_end=1000, seed=1)
    with pytest.raises(gpu.IdashError) as e:
        m.serve([big], hbm_budget=64 << 20, max_inflight=2)
    assert e.value.name == "IDASH_ERR_ADMISSION"
