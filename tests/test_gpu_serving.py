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


# ------------------------------------------------------------ online server
def _rows_for(rng, shape):
    return rng.integers(0, 2 ** 32, size=shape, dtype=np.uint64).astype(np.uint32).view(np.int32)


def test_online_server_host_payloads_match_the_oracle(served, oracle):
    """Requests submitted one after another while earlier ones run, with
    their ciphertexts in host memory and their outputs copied back: every
    output word equals the oracle's, and each request's outputs and digest
    are the same when it is served alone."""
    import ctypes as C
    ctx, w, m, _, _, _ = served
    rng = np.random.default_rng(11)
    srv = gpu.Server(m, hbm_budget=1 << 30, max_inflight=6)
    reqs, tickets = [], []
    try:
        for i in range(12):
            length = int(rng.integers(10, 300))
            t0 = int(rng.integers(0, 1000 - length))
            n_indiv = int(rng.integers(1, 2200))
            in_shape, out_shape, lo = gpu.serve_input_shape(m, n_indiv, t0, t0 + length)
            h_in = _rows_for(rng, in_shape)
            h_out = np.zeros(out_shape, np.int32)
            tickets.append(srv.submit(n_indiv, t0, t0 + length, h_in=h_in, h_out=h_out))
            reqs.append((n_indiv, t0, t0 + length, h_in, h_out, lo))
            if i % 4 == 3:
                srv.wait(tickets[-2])  # later requests arrive while others are in flight
        res = [srv.wait(t) for t in tickets]
        launches = srv.launches()
        st = srv.stats()
    finally:
        srv.close()
    assert launches <= len(reqs)
    # the counters: every payload byte crossed once each way, device time was spent
    assert st["launches"] == launches and st["requests_done"] == len(reqs)
    assert st["h2d_bytes"] == sum(q[3].nbytes for q in reqs)
    assert st["d2h_bytes"] == sum(q[4].nbytes for q in reqs)
    assert 0 < st["busy_s"] < max(r["done_s"] for r in res)
    for (n_indiv, t0, t1, h_in, h_out, lo), r in zip(reqs, res):
        sub = w.model.slice_outputs(3 * t0, 3 * t1)
        for b in range(h_in.shape[0]):
            rows = np.zeros((900, 2048), np.int32)
            rows[lo:lo + h_in.shape[1]] = h_in[b]
            ns = min(1024, n_indiv - 1024 * b)
            want, _ = oracle.trlwe_score(sub.term_ptr, sub.term_feat, sub.term_coef, rows, ns, 1, 1024)
            np.testing.assert_array_equal(h_out[b], want)
        words = np.ascontiguousarray(h_out).view(np.uint32).ravel()
        assert r["digest"] == ctx.lib.idash_digest_host(words.ctypes.data_as(C.POINTER(C.c_uint32)), words.size, 0)
    # alone: one request at a time
    alone = gpu.Server(m, hbm_budget=1 << 30, max_inflight=1)
    try:
        for (n_indiv, t0, t1, h_in, h_out, lo), r in list(zip(reqs, res))[:4]:
            out1 = np.zeros_like(h_out)
            r1 = alone.wait(alone.submit(n_indiv, t0, t1, h_in=h_in, h_out=out1))
            np.testing.assert_array_equal(out1, h_out)
            assert r1["digest"] == r["digest"]
    finally:
        alone.close()


def test_online_server_lwe_form_in_segments(oracle):
    """The per-individual LWE form served: requests of different individual
    counts (different row strides) share launches, outputs come back in
    segments of 37 outputs; every word equals the oracle's."""
    import ctypes as C
    ctx = gpu.Context(0)
    try:
        n, n_tags = 1024, 200
        w = gpu.synth_model(seed=21, n_tags=n_tags, n_targets=300, neighbours=10)
        m = gpu.LweModel(ctx, w.model, 3 * n_tags, 40, n)
        rng = np.random.default_rng(3)
        srv = gpu.Server(m, hbm_budget=1 << 30, max_inflight=4, segment_outputs=37)
        reqs, tickets = [], []
        try:
            for i in range(7):
                length = int(rng.integers(5, 120))
                t0 = int(rng.integers(0, 300 - length))
                n_indiv = int(rng.integers(1, 41))
                in_shape, out_shape, lo = gpu.serve_input_shape(m, n_indiv, t0, t0 + length)
                h_in = _rows_for(rng, in_shape)
                h_out = np.zeros(out_shape, np.int32)
                tickets.append(srv.submit(n_indiv, t0, t0 + length, h_in=h_in, h_out=h_out))
                reqs.append((n_indiv, t0, t0 + length, h_in, h_out, lo))
            res = [srv.wait(t) for t in tickets]
        finally:
            srv.close()
        for (n_indiv, t0, t1, h_in, h_out, lo), r in zip(reqs, res):
            L = n_indiv * (n + 1)
            sub = w.model.slice_outputs(3 * t0, 3 * t1)
            rows = np.zeros((3 * n_tags, h_in.shape[1]), np.int32)
            rows[lo:lo + h_in.shape[0]] = h_in
            want = oracle.lwe_score(sub.term_ptr, sub.term_feat, sub.term_coef, rows, n_indiv, 0, sub.n_out, n=n)
            np.testing.assert_array_equal(h_out[:, :L], want)
            # the digest covers the valid words at their positions in the output layout
            exp = 0
            for row in range(h_out.shape[0]):
                words = np.ascontiguousarray(h_out[row, :L]).view(np.uint32)
                exp += ctx.lib.idash_digest_host(words.ctypes.data_as(C.POINTER(C.c_uint32)), L, row * h_out.shape[1])
            assert r["digest"] == exp % (1 << 64)
        m.free()
    finally:
        ctx.close()


def test_online_server_refuses_bad_requests(served):
    ctx, w, m, _, _, _ = served
    srv = gpu.Server(m, hbm_budget=64 << 20, max_inflight=2)
    try:
        with pytest.raises(gpu.IdashError) as e:
            srv.submit(3000, 0, 1000)  # more than the budget
        assert e.value.name == "IDASH_ERR_ADMISSION"
        with pytest.raises(gpu.IdashError) as e:
            srv.submit(10, 990, 1001)  # targets out of range
        assert e.value.name == "IDASH_ERR_INVALID_ARGUMENT"
        t = srv.submit(5, 0, 10, seed=9)
        r = srv.wait(t)
        assert r["done_s"] >= r["admit_s"] >= 0
        assert srv.poll(t)["digest"] == r["digest"]
    finally:
        srv.close()


def test_submits_from_several_threads_and_close_drains(served):
    """Four client threads submit and wait at once (the calls release the
    interpreter lock): every request's outputs and digest are right.  Then
    requests submitted and not waited for are finished by close."""
    import ctypes as C
    import threading
    ctx, w, m, _, _, _ = served
    srv = gpu.Server(m, hbm_budget=1 << 30, max_inflight=6)
    results, errors = {}, []

    def client(k):
        try:
            rng = np.random.default_rng(100 + k)
            for i in range(4):
                length = int(rng.integers(10, 200))
                t0 = int(rng.integers(0, 1000 - length))
                n_indiv = int(rng.integers(1, 1500))
                in_shape, out_shape, lo = gpu.serve_input_shape(m, n_indiv, t0, t0 + length)
                h_in = _rows_for(rng, in_shape)
                h_out = np.zeros(out_shape, np.int32)
                r = srv.wait(srv.submit(n_indiv, t0, t0 + length, h_in=h_in, h_out=h_out))
                results[(k, i)] = (n_indiv, t0, t0 + length, h_in, h_out, lo, r)
        except Exception as e:  # reported by the main thread
            errors.append(e)

    threads = [threading.Thread(target=client, args=(k,)) for k in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors and len(results) == 16
    for n_indiv, t0, t1, h_in, h_out, lo, r in results.values():
        words = np.ascontiguousarray(h_out).view(np.uint32).ravel()
        assert r["digest"] == ctx.lib.idash_digest_host(words.ctypes.data_as(C.POINTER(C.c_uint32)), words.size, 0)
    # one request per thread against the oracle
    for k in range(4):
        n_indiv, t0, t1, h_in, h_out, lo, _ = results[(k, 0)]
        sub = w.model.slice_outputs(3 * t0, 3 * t1)
        rows = np.zeros((900, 2048), np.int32)
        rows[lo:lo + h_in.shape[1]] = h_in[0]
        want, _ = oracle_trlwe(sub, rows, min(1024, n_indiv))
        np.testing.assert_array_equal(h_out[0], want)
    for i in range(8):
        srv.submit(50 + i, 10 * i, 10 * i + 300, seed=i + 1)
    srv.close()  # returns once the eight are scored
    assert srv.h is None


def oracle_trlwe(sub, rows, ns):
    import pyoracle
    return pyoracle.trlwe_score(sub.term_ptr, sub.term_feat, sub.term_coef, rows, ns, 1, 1024)
