"""idash_score_trlwe_noalloc: scoring for callers that cannot allocate device
memory (their framework owns the GPU's memory pool, or they sit at a
per-client memory limit, or they cannot take cudaMalloc's synchronisation).

The entry point is called through the C ABI on several models in a row and
each result is compared word for word with the oracle's restatement of the
reference loop (oracle/oracle.c, eval/idash.cpp:779-842): payloads, record
headers and the double variance.  The cases cover both kernels the entry
point can run: the batched window kernel, and the direct kernel it falls back
to when one output's slots exceed any window (30 neighbours = 90 slots, more
than the 83 a 256-word window holds).  The first case runs again last, so
what an earlier call left in the shared scratch array cannot leak into a
later result.  This file is collected last so a failure here stops a -x run
only after every other test has run; it also passes alone in a fresh process
(the first call on the device does the scratch set-up)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

gpu = pytest.importorskip("idash2019_2_gb300.gpu")
_lib = pytest.importorskip("idash2019_2_gb300._lib")

U32P, U64P, I32P = C.POINTER(C.c_uint32), C.POINTER(C.c_uint64), C.POINTER(C.c_int32)


def _noalloc(lib, params, csr, n_rows, d_in, in_layout, d_out, out_layout, out_index=None, row_of_index=None):
    tp = np.ascontiguousarray(csr.term_ptr, np.uint64)
    tf = np.ascontiguousarray(csr.term_feat, np.uint32)
    tc = np.ascontiguousarray(csr.term_coef, np.int32)
    oi = None if out_index is None else np.ascontiguousarray(out_index, np.uint32)
    ri = None if row_of_index is None else np.ascontiguousarray(row_of_index, np.uint32)
    return lib.idash_score_trlwe_noalloc(
        C.byref(params), csr.n_out, None if oi is None else oi.ctypes.data_as(U32P), tp.ctypes.data_as(U64P),
        tf.ctypes.data_as(U32P), tc.ctypes.data_as(I32P), 0 if ri is None else len(ri),
        None if ri is None else ri.ctypes.data_as(U32P), n_rows, C.c_void_p(d_in), C.byref(in_layout),
        C.c_void_p(d_out), C.byref(out_layout), None)


# (seed, tags, targets, neighbours, NUM_SAMPLES, NUM_REGIONS, REGION_SIZE, records, index maps)
CASES = [
    (41, 300, 900, 5, 1000, 1, 1024, False, False),   # window kernel, dense rows
    (42, 120, 250, 7, 100, 10, 102, True, False),     # window kernel, rotated regions, records
    (43, 200, 400, 5, 1000, 1, 1024, True, True),     # records at NUM_REGIONS 1, FeatIndex -> row map, indices
    (44, 100, 60, 30, 500, 1, 1024, False, True),     # direct-kernel fallback (90 slots per output)
    (41, 300, 900, 5, 1000, 1, 1024, False, False),   # the first case again
]


def _run_case(lib, ctx, oracle, seed, tags, targets, k, ns, regions, rs, records, maps):
    w = gpu.synth_model(seed=seed, n_tags=tags, n_targets=targets, neighbours=k)
    csr = w.model
    n_rows = (3 * tags + regions - 1) // regions
    rng = np.random.default_rng(seed)
    rows = rng.integers(0, 2 ** 32, size=(n_rows, 2048), dtype=np.uint64).astype(np.uint32).view(np.int32)
    in_var = rng.random(n_rows) * 2.0 ** -40
    # FeatIndex i is held at input row perm[i] when the case maps indices
    perm = rng.permutation(n_rows).astype(np.uint32) if maps else np.arange(n_rows, dtype=np.uint32)
    out_index = (rng.permutation(csr.n_out) * 7 + 3).astype(np.uint32) if maps else None
    held = np.empty_like(rows)
    held[perm] = rows
    lay_in = gpu.RECORD_IN if records else gpu.DENSE_TRLWE
    lay_out = gpu.RECORD_OUT if records else gpu.DENSE_TRLWE
    stride = lay_in.row_stride
    base = 8 if records else 0  # record payloads sit at +8 of a 16-byte aligned base
    img = np.zeros(n_rows * stride // 4 + 4, np.int32)
    view = img[base // 4: base // 4 + n_rows * stride // 4].reshape(n_rows, stride // 4)
    p0 = 2 if records else 0
    view[:, p0:p0 + 2048] = held
    if records:
        vv = np.empty_like(in_var)
        vv[perm] = in_var
        view[:, 2050:2052] = vv.view(np.int32).reshape(n_rows, 2)
    d_in = ctx.device_alloc(img.nbytes)
    d_out = ctx.device_alloc(csr.n_out * stride + 16)
    try:
        d_in.upload(img)
        d_out.upload(np.full((csr.n_out * stride + 16) // 4, -1, np.int32))  # stale bytes everywhere
        ctx.sync()
        params = gpu.TrlweParams(1024, 1, ns, regions, rs, 1 << 18, 42)
        code = _noalloc(lib, params, csr, n_rows, d_in.ptr + base, lay_in, d_out.ptr + base, lay_out,
                        out_index=out_index, row_of_index=perm if maps else None)
        assert code == 0, lib.idash_last_error(None)
        got = d_out.download().view(np.int32)
    finally:
        d_in.free()
        d_out.free()
    want, want_var = oracle.trlwe_score(csr.term_ptr, csr.term_feat, csr.term_coef, rows, ns, regions, rs,
                                        in_var=in_var if records else None)
    recs = got[base // 4: base // 4 + csr.n_out * stride // 4].reshape(csr.n_out, stride // 4)
    np.testing.assert_array_equal(recs[:, p0:p0 + 2048], want)
    if records:
        idx = recs[:, 0].view(np.uint32)
        np.testing.assert_array_equal(idx, out_index if out_index is not None else np.arange(csr.n_out))
        assert np.all(recs[:, 1] == 42)
        got_var = np.ascontiguousarray(recs[:, 2050:2052]).view(np.float64).ravel()
        np.testing.assert_array_equal(got_var, want_var)


def test_noalloc_matches_oracle_over_consecutive_calls(oracle):
    lib = _lib.load()
    ctx = gpu.Context(0)
    try:
        for case in CASES:
            _run_case(lib, ctx, oracle, *case)
    finally:
        ctx.close()


def test_noalloc_refuses_models_beyond_its_scratch():
    lib = _lib.load()
    ctx = gpu.Context(0)
    try:
        # 1,200,000 outputs with 16 terms each: plan tables of about 100 MiB
        n_out, per = 1_200_000, 16
        ptr = np.arange(n_out + 1, dtype=np.uint64) * per
        feat = np.tile(np.arange(per, dtype=np.uint32), n_out)
        coef = np.ones(n_out * per, np.int32)
        csr = gpu.CSRModel(ptr, feat, coef)
        d = ctx.device_alloc(64 * 8192)
        params = gpu.TrlweParams(1024, 1, 1000, 1, 1024, 1 << 18, 42)
        code = _noalloc(lib, params, csr, 64, d.ptr, gpu.DENSE_TRLWE, d.ptr, gpu.DENSE_TRLWE)
        assert _lib.STATUS[code] == "IDASH_ERR_INVALID_ARGUMENT"
        assert b"64 MiB" in lib.idash_last_error(None)
        d.free()
    finally:
        ctx.close()
