"""idash_score_trlwe_noalloc: scoring for callers that cannot allocate device
memory (their framework owns the GPU's memory pool, or they sit at a
per-client memory limit, or they cannot take cudaMalloc's synchronisation).

The entry point is called through the C ABI, twice in a row with different
models, and each result must equal the regular entry point's
(idash_score_trlwe_device) bit for bit.  This file is collected last so a
failure here stops a -x run only after every other test has run; it also
passes alone in a fresh process (the first call on the device does the
scratch set-up)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

gpu = pytest.importorskip("idash2019_2_gb300.gpu")
_lib = pytest.importorskip("idash2019_2_gb300._lib")


def _rows(seed, n_rows):
    rng = np.random.default_rng(seed)
    return rng.integers(0, 2 ** 32, size=(n_rows, 2048), dtype=np.uint64).astype(np.uint32).view(np.int32)


def _noalloc(lib, params, csr, n_rows, d_in, in_layout, d_out, out_layout):
    tp = np.ascontiguousarray(csr.term_ptr, np.uint64)
    tf = np.ascontiguousarray(csr.term_feat, np.uint32)
    tc = np.ascontiguousarray(csr.term_coef, np.int32)
    return lib.idash_score_trlwe_noalloc(
        C.byref(params), csr.n_out, tp.ctypes.data_as(C.POINTER(C.c_uint64)),
        tf.ctypes.data_as(C.POINTER(C.c_uint32)), tc.ctypes.data_as(C.POINTER(C.c_int32)), n_rows,
        C.c_void_p(d_in), C.byref(in_layout), C.c_void_p(d_out), C.byref(out_layout), None)


CASES = [
    # (seed, tags, targets, neighbours, NUM_SAMPLES, NUM_REGIONS, REGION_SIZE, record layout)
    (41, 300, 900, 5, 1000, 1, 1024, False),
    (42, 120, 250, 7, 100, 10, 102, True),
]


def test_noalloc_matches_device_entry_point_twice():
    lib = _lib.load()
    ctx = gpu.Context(0)
    try:
        for seed, tags, targets, k, ns, regions, rs, records in CASES:
            w = gpu.synth_model(seed=seed, n_tags=tags, n_targets=targets, neighbours=k)
            n_rows = (3 * tags + regions - 1) // regions
            params = gpu.TrlweParams(1024, 1, ns, regions, rs, 1 << 18, 42)
            lay_in = gpu.RECORD_IN if records else gpu.DENSE_TRLWE
            lay_out = gpu.RECORD_OUT if records else gpu.DENSE_TRLWE
            stride = lay_in.row_stride
            base = 8 if records else 0  # record payloads sit at +8 of a 16-byte aligned base
            rows = _rows(seed, n_rows)
            img = np.zeros(n_rows * stride // 4 + 4, np.int32)
            view = img[base // 4: base // 4 + n_rows * stride // 4].reshape(n_rows, stride // 4)
            view[:, 2 if records else 0:(2 if records else 0) + 2048] = rows
            if records:
                view[:, 2050:2052] = np.array([2.0 ** -50], np.float64).view(np.int32)
            d_in = ctx.device_alloc(img.nbytes)
            d_in.upload(img)
            out_bytes = w.model.n_out * stride + 16
            d_ref = ctx.device_alloc(out_bytes)
            d_new = ctx.device_alloc(out_bytes)
            m = gpu.TrlweModel(ctx, w.model, n_rows, ns, regions, rs)
            m.score_device(d_in.ptr + base, lay_in, d_ref.ptr + base, lay_out)
            ctx.sync()
            want = d_ref.download()
            m.free()
            d_new.zero()
            ctx.sync()
            code = _noalloc(lib, params, w.model, n_rows, d_in.ptr + base, lay_in, d_new.ptr + base, lay_out)
            assert code == 0, lib.idash_last_error(None)
            got = d_new.download()
            np.testing.assert_array_equal(got, want)
            for b in (d_in, d_ref, d_new):
                b.free()
    finally:
        ctx.close()


def test_noalloc_refuses_models_beyond_its_scratch():
    lib = _lib.load()
    ctx = gpu.Context(0)
    try:
        # 450,000 outputs with 16 terms each: a plan of about 40 MB
        n_out, per = 450_000, 16
        ptr = np.arange(n_out + 1, dtype=np.uint64) * per
        feat = np.tile(np.arange(per, dtype=np.uint32), n_out)
        coef = np.ones(n_out * per, np.int32)
        csr = gpu.CSRModel(ptr, feat, coef)
        d = ctx.device_alloc(64 * 8192)
        params = gpu.TrlweParams(1024, 1, 1000, 1, 1024, 1 << 18, 42)
        code = _noalloc(lib, params, csr, 64, d.ptr, gpu.DENSE_TRLWE, d.ptr, gpu.DENSE_TRLWE)
        assert _lib.STATUS[code] == "IDASH_ERR_INVALID_ARGUMENT"
        assert b"32 MiB" in lib.idash_last_error(None)
        d.free()
    finally:
        ctx.close()
