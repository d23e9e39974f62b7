"""Python face of the C ABI, for tests, smoke() and bench.py.

Mirrors the reference's cloud-step roles (eval/idash.h): a Model flattened to
CSR, EncryptedData as rows of TRLWE ciphertexts, EncryptedPredictions as
output rows.  All compute goes through libidash_gpu.so; host arrays are numpy.
"""
from __future__ import annotations

import ctypes as C
import weakref
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import IdashError, RowLayout, TrlweParams, LweParams, check

N_DEFAULT = 1024
ONE_IN_T32 = 1 << 18                   # dtot32(2^-14), eval/idash.cpp:39
RECORD_BYTES = 8 + 2 * 1024 * 4 + 8    # uint32 index | int32 tag | 2N int32 | double
RECORD_TAG = 42
DENSE_TRLWE = RowLayout(2 * 1024 * 4, 0, -1, -1)
RECORD_IN = RowLayout(RECORD_BYTES, 8, 8 + 2 * 1024 * 4, -1)
RECORD_OUT = RowLayout(RECORD_BYTES, 8, 8 + 2 * 1024 * 4, 0)


def _p(arr, ctype):
    return arr.ctypes.data_as(C.POINTER(ctype)) if arr is not None else None


class Context:
    """One GPU: stream, scratch and error word (idash_open)."""

    def __init__(self, device: int = 0):
        self.lib = _lib.load()
        h = C.c_void_p()
        code = self.lib.idash_open(C.byref(h), device)
        if code != 0:
            raise IdashError(code, (self.lib.idash_last_error(None) or b"").decode())
        self.h = h
        self._owned = weakref.WeakSet()  # models and buffers to release before the context

    def _own(self, obj):
        self._owned.add(obj)

    def close(self):
        if self.h:
            for obj in list(self._owned):
                obj.free()
            self.lib.idash_close(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, code):
        check(code, self.h)

    def set_option(self, name: str, value: int):
        self.check(self.lib.idash_set_option(self.h, name.encode(), int(value)))

    def get_option(self, name: str) -> int:
        v = C.c_int64()
        self.check(self.lib.idash_get_option(self.h, name.encode(), C.byref(v)))
        return v.value

    def stats(self) -> dict:
        s = _lib.Stats()
        self.check(self.lib.idash_get_stats(self.h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in s._fields_}

    @property
    def stream(self) -> int:
        return self.lib.idash_stream(self.h) or 0

    def sync(self):
        self.check(self.lib.idash_sync(self.h))

    # memory
    def device_alloc(self, nbytes: int) -> "DeviceBuffer":
        return DeviceBuffer(self, nbytes)

    def host_alloc(self, nbytes: int) -> "HostBuffer":
        return HostBuffer(self, nbytes)


class DeviceBuffer:
    def __init__(self, ctx: Context, nbytes: int):
        self.ctx, self.nbytes = ctx, int(nbytes)
        p = C.c_void_p()
        ctx.check(ctx.lib.idash_device_alloc(ctx.h, self.nbytes, C.byref(p)))
        self.ptr = p.value
        ctx._own(self)

    def free(self):
        if self.ptr and self.ctx.h:
            self.ctx.check(self.ctx.lib.idash_device_free(self.ctx.h, C.c_void_p(self.ptr)))
        self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def upload(self, arr: np.ndarray, offset: int = 0):
        arr = np.ascontiguousarray(arr)
        assert offset + arr.nbytes <= self.nbytes
        self.ctx.check(self.ctx.lib.idash_copy_h2d(self.ctx.h, C.c_void_p(self.ptr + offset),
                                                   arr.ctypes.data_as(C.c_void_p), arr.nbytes))

    def download(self, nbytes: int | None = None, offset: int = 0, dtype=np.uint8) -> np.ndarray:
        nbytes = self.nbytes - offset if nbytes is None else nbytes
        out = np.empty(nbytes // np.dtype(dtype).itemsize, dtype=dtype)
        self.ctx.check(self.ctx.lib.idash_copy_d2h(self.ctx.h, out.ctypes.data_as(C.c_void_p),
                                                   C.c_void_p(self.ptr + offset), out.nbytes))
        return out

    def zero(self):
        self.ctx.check(self.ctx.lib.idash_memset_device(self.ctx.h, C.c_void_p(self.ptr), 0, self.nbytes))


class HostBuffer:
    """Page-locked host memory exposed as a numpy array."""

    def __init__(self, ctx: Context, nbytes: int):
        self.ctx, self.nbytes = ctx, int(nbytes)
        p = C.c_void_p()
        ctx.check(ctx.lib.idash_host_alloc(ctx.h, self.nbytes, C.byref(p)))
        self.ptr = p.value
        ctx._own(self)
        self.array = np.ctypeslib.as_array((C.c_uint8 * self.nbytes).from_address(self.ptr))

    def free(self):
        if self.ptr and self.ctx.h:
            self.array = None
            self.ctx.check(self.ctx.lib.idash_host_free(self.ctx.h, C.c_void_p(self.ptr)))
        self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


@dataclass
class CSRModel:
    """A Model (eval/idash.h:129-134) flattened: output o's terms are
    term_feat/term_coef[term_ptr[o]:term_ptr[o+1]]; constant = 0xFFFFFFFF."""
    term_ptr: np.ndarray   # uint64 [n_out + 1]
    term_feat: np.ndarray  # uint32
    term_coef: np.ndarray  # int32

    @property
    def n_out(self) -> int:
        return len(self.term_ptr) - 1

    def slice_outputs(self, lo: int, hi: int) -> "CSRModel":
        a, b = int(self.term_ptr[lo]), int(self.term_ptr[hi])
        return CSRModel((self.term_ptr[lo:hi + 1] - a).astype(np.uint64), self.term_feat[a:b].copy(),
                        self.term_coef[a:b].copy())


@dataclass
class SynthWorkload:
    model: CSRModel
    tag_pos: np.ndarray
    target_pos: np.ndarray
    window_start: np.ndarray
    window_len: np.ndarray


def synth_model(seed: int, n_tags: int, n_targets: int, neighbours: int = 5, choices=None) -> SynthWorkload:
    """Seeded synthetic imputation model (idash_synth_model; host only)."""
    lib = _lib.load()
    spec = _lib.SynthSpec()
    spec.seed, spec.n_tags, spec.n_targets = seed, n_tags, n_targets
    if choices:
        spec.neighbours, spec.n_choices = 0, len(choices)
        for i, c in enumerate(choices):
            spec.choices[i] = c
    else:
        spec.neighbours, spec.n_choices = neighbours, 0
    m = _lib.SynthModel()
    check(lib.idash_synth_model(C.byref(spec), C.byref(m)))
    try:
        n_out, nt = m.n_out, m.n_terms
        arr = np.ctypeslib.as_array
        w = SynthWorkload(
            CSRModel(arr(m.term_ptr, (n_out + 1,)).copy(), arr(m.term_feat, (nt,)).copy(),
                     arr(m.term_coef, (nt,)).copy()),
            arr(m.tag_pos, (n_tags,)).copy(),
            arr(m.target_pos, (n_targets,)).copy() if n_targets else np.zeros(0, np.uint64),
            arr(m.window_start, (n_targets,)).copy() if n_targets else np.zeros(0, np.uint32),
            arr(m.window_len, (n_targets,)).copy() if n_targets else np.zeros(0, np.uint32))
    finally:
        lib.idash_synth_model_free(C.byref(m))
    return w


class TrlweModel:
    """A resident TRLWE model (idash_model_trlwe): the cloud_compute_score
    drop-in (eval/idash.cpp:763-848)."""

    def __init__(self, ctx: Context, csr: CSRModel, n_in_rows: int, num_samples: int, num_regions: int,
                 region_size: int, N: int = N_DEFAULT, one_t32: int = ONE_IN_T32, out_index=None, out_row=None,
                 row_of_index=None, record_tag: int = RECORD_TAG):
        self.ctx, self.csr, self.N = ctx, csr, N
        self.params = TrlweParams(N, 1, num_samples, num_regions, region_size, one_t32, record_tag)
        self._keep = [np.ascontiguousarray(csr.term_ptr, np.uint64), np.ascontiguousarray(csr.term_feat, np.uint32),
                      np.ascontiguousarray(csr.term_coef, np.int32)]
        oi = None if out_index is None else np.ascontiguousarray(out_index, np.uint32)
        orow = None if out_row is None else np.ascontiguousarray(out_row, np.uint32)
        ri = None if row_of_index is None else np.ascontiguousarray(row_of_index, np.uint32)
        self._keep += [oi, orow, ri]
        h = C.c_void_p()
        ctx.check(ctx.lib.idash_model_trlwe(
            ctx.h, C.byref(h), C.byref(self.params), csr.n_out, _p(oi, C.c_uint32), _p(orow, C.c_uint32),
            _p(self._keep[0], C.c_uint64), _p(self._keep[1], C.c_uint32), _p(self._keep[2], C.c_int32),
            0 if ri is None else len(ri), _p(ri, C.c_uint32), n_in_rows))
        self.h = h
        self.n_out = csr.n_out
        self.n_in_rows = n_in_rows
        ctx._own(self)

    def free(self):
        if self.h and self.ctx.h:
            self.ctx.lib.idash_model_free(self.h)
        self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def info(self) -> dict:
        i = _lib.ModelInfo()
        self.ctx.check(self.ctx.lib.idash_model_get_info(self.h, C.byref(i)))
        return {k: getattr(i, k) for k, _ in i._fields_}

    def replan(self):
        self.ctx.check(self.ctx.lib.idash_model_replan(self.h))

    def score_device(self, d_in: int, in_layout: RowLayout, d_out: int, out_layout: RowLayout, stream=None):
        self.ctx.check(self.ctx.lib.idash_score_trlwe_device(
            self.h, C.c_void_p(d_in), C.byref(in_layout), C.c_void_p(d_out), C.byref(out_layout),
            C.c_void_p(stream) if stream else None))

    def score_host(self, h_in_ptr: int, in_layout: RowLayout, n_in_rows: int, h_out_ptr: int,
                   out_layout: RowLayout):
        self.ctx.check(self.ctx.lib.idash_score_trlwe_host(
            self.h, C.c_void_p(h_in_ptr), C.byref(in_layout), n_in_rows, C.c_void_p(h_out_ptr),
            C.byref(out_layout)))

    def score_range(self, out_begin: int, out_end: int, num_samples: int, d_in: int, in_layout: RowLayout,
                    in_row_base: int, n_in_rows: int, d_out: int, out_layout: RowLayout, stream=None):
        self.ctx.check(self.ctx.lib.idash_score_trlwe_range(
            self.h, out_begin, out_end, num_samples, C.c_void_p(d_in), C.byref(in_layout), in_row_base, n_in_rows,
            C.c_void_p(d_out), C.byref(out_layout), C.c_void_p(stream) if stream else None))

    def input_rows(self, out_begin: int, out_end: int) -> tuple[int, int]:
        lo, hi = C.c_uint64(), C.c_uint64()
        self.ctx.check(self.ctx.lib.idash_model_input_rows(self.h, out_begin, out_end, C.byref(lo), C.byref(hi)))
        return lo.value, hi.value

    def serve(self, requests, hbm_budget: int, max_inflight: int, keep_outputs: bool = False):
        """Runs idash_serve_trlwe over `requests` (dicts with arrival_s,
        n_indiv, target_begin, target_end, seed).  Returns (results, outputs);
        outputs[i] is request i's int32 [blocks, outputs, 2N] array when
        keep_outputs, else None."""
        n = len(requests)
        reqs = (_lib.Request * max(n, 1))()
        for i, r in enumerate(requests):
            reqs[i] = _lib.Request(r["arrival_s"], r["n_indiv"], 0, r["target_begin"], r["target_end"], r["seed"])
        res = (_lib.RequestResult * max(n, 1))()
        cfg = _lib.ServeConfig(hbm_budget, max_inflight, 0)
        outs, ptrs = None, None
        if keep_outputs:
            rs = self.params.region_size
            outs = [np.zeros(((r["n_indiv"] + rs - 1) // rs, 3 * (r["target_end"] - r["target_begin"]), 2 * self.N),
                             np.int32) for r in requests]
            ptrs = (C.c_void_p * max(n, 1))(*[o.ctypes.data for o in outs])
        self.ctx.check(self.ctx.lib.idash_serve_trlwe(self.h, C.byref(cfg), reqs, n, res, ptrs))
        return [{k: getattr(res[i], k) for k, _ in res[i]._fields_} for i in range(n)], outs

    def score(self, rows: np.ndarray) -> np.ndarray:
        """Convenience: dense int32 [n_rows, 2N] in -> [n_out, 2N] out, via the
        host-memory path."""
        rows = np.ascontiguousarray(rows, dtype=np.int32)
        assert rows.shape[1] == 2 * self.N
        out = np.empty((self.n_out, 2 * self.N), dtype=np.int32)
        lay = RowLayout(2 * self.N * 4, 0, -1, -1)
        self.score_host(rows.ctypes.data, lay, rows.shape[0], out.ctypes.data, lay)
        return out


class LweModel:
    """A resident per-individual LWE model (idash_model_lwe)."""

    def __init__(self, ctx: Context, csr: CSRModel, n_feat_rows: int, n_indiv: int, n: int = 1024,
                 one_t32: int = ONE_IN_T32):
        self.ctx, self.csr, self.n, self.n_indiv = ctx, csr, n, n_indiv
        self.params = LweParams(n, n_indiv, one_t32)
        self._keep = [np.ascontiguousarray(csr.term_ptr, np.uint64), np.ascontiguousarray(csr.term_feat, np.uint32),
                      np.ascontiguousarray(csr.term_coef, np.int32)]
        h = C.c_void_p()
        ctx.check(ctx.lib.idash_model_lwe(ctx.h, C.byref(h), C.byref(self.params), csr.n_out,
                                          _p(self._keep[0], C.c_uint64), _p(self._keep[1], C.c_uint32),
                                          _p(self._keep[2], C.c_int32), n_feat_rows))
        self.h = h
        self.n_out = csr.n_out
        ctx._own(self)

    def free(self):
        if self.h and self.ctx.h:
            self.ctx.lib.idash_model_free(self.h)
        self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def input_rows(self, out_begin: int, out_end: int) -> tuple[int, int]:
        lo, hi = C.c_uint64(), C.c_uint64()
        self.ctx.check(self.ctx.lib.idash_model_input_rows(self.h, out_begin, out_end, C.byref(lo), C.byref(hi)))
        return lo.value, hi.value

    def info(self) -> dict:
        i = _lib.ModelInfo()
        self.ctx.check(self.ctx.lib.idash_model_get_info(self.h, C.byref(i)))
        return {k: getattr(i, k) for k, _ in i._fields_}

    def score_device(self, n_indiv: int, d_in: int, in_stride_words: int, out_begin: int, out_end: int,
                     d_out: int, out_stride_words: int, stream=None):
        self.ctx.check(self.ctx.lib.idash_score_lwe_device(
            self.h, n_indiv, C.c_void_p(d_in), in_stride_words, out_begin, out_end, C.c_void_p(d_out),
            out_stride_words, C.c_void_p(stream) if stream else None))


class IntpolyModel:
    """A resident integer-polynomial x TRLWE model (idash_model_intpoly)."""

    def __init__(self, ctx: Context, csr: CSRModel, term_poly, n_in_rows: int, num_samples: int,
                 region_size: int, bias=None, N: int = N_DEFAULT, one_t32: int = ONE_IN_T32,
                 max_abs_coef: int = 8192, poly_on_device: bool = False):
        self.ctx, self.csr, self.N = ctx, csr, N
        self.params = _lib.IntpolyParams(N, num_samples, region_size, one_t32, max_abs_coef)
        keep = [np.ascontiguousarray(csr.term_ptr, np.uint64), np.ascontiguousarray(csr.term_feat, np.uint32)]
        b = None if bias is None else np.ascontiguousarray(bias, np.int32)
        if poly_on_device:
            poly_ptr = C.c_void_p(term_poly)
        else:
            tp = np.ascontiguousarray(term_poly, np.int16)
            keep.append(tp)
            poly_ptr = tp.ctypes.data_as(C.c_void_p)
        h = C.c_void_p()
        ctx.check(ctx.lib.idash_model_intpoly(ctx.h, C.byref(h), C.byref(self.params), csr.n_out,
                                              _p(keep[0], C.c_uint64), _p(keep[1], C.c_uint32), _p(b, C.c_int32),
                                              n_in_rows, poly_ptr, 1 if poly_on_device else 0))
        self.h = h
        self.n_out = csr.n_out
        ctx._own(self)

    def free(self):
        if self.h and self.ctx.h:
            self.ctx.lib.idash_model_free(self.h)
        self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def set_weights(self, d_term_poly: int, stream=None):
        """New int16 weight polynomials (device memory, [terms][N]) for the
        same terms, transformed into the resident form asynchronously."""
        self.ctx.check(self.ctx.lib.idash_model_intpoly_set_weights(self.h, C.c_void_p(d_term_poly),
                                                                    C.c_void_p(stream) if stream else None))

    def score_device(self, d_in: int, in_layout: RowLayout, out_begin: int, out_end: int, d_out: int,
                     out_layout: RowLayout, stream=None):
        self.ctx.check(self.ctx.lib.idash_score_intpoly_device(
            self.h, C.c_void_p(d_in), C.byref(in_layout), out_begin, out_end, C.c_void_p(d_out), C.byref(out_layout),
            C.c_void_p(stream) if stream else None))


class Server:
    """An online serving engine over one resident model (idash_server_*):
    submit requests at any time, poll or wait for their results."""

    def __init__(self, model, hbm_budget: int, max_inflight: int, segment_outputs: int = 0):
        self.ctx, self.model = model.ctx, model
        lib = self.ctx.lib
        cfg = _lib.ServeConfig(hbm_budget, max_inflight, segment_outputs)
        h = C.c_void_p()
        self.ctx.check(lib.idash_server_open(model.h, C.byref(cfg), C.byref(h)))
        self.h = h
        self._keep = {}

    def submit(self, n_indiv: int, target_begin: int, target_end: int, h_in=None, h_out=None, seed: int = 0) -> int:
        """h_in / h_out: numpy arrays (kept alive until the request is waited
        for) or None (inputs generated from seed / digest only)."""
        r = _lib.ServeRequest(n_indiv, 0, target_begin, target_end,
                              None if h_in is None else h_in.ctypes.data, None if h_out is None else h_out.ctypes.data,
                              seed)
        t = C.c_uint64()
        code = self.ctx.lib.idash_server_submit(self.h, C.byref(r), C.byref(t))
        if code != 0:
            raise IdashError(code, (self.ctx.lib.idash_server_last_error(self.h) or b"").decode())
        self._keep[t.value] = (h_in, h_out)
        return t.value

    def poll(self, ticket: int):
        res = _lib.RequestResult()
        code = self.ctx.lib.idash_server_poll(self.h, ticket, C.byref(res))
        if code == 11:
            return None
        if code != 0:
            raise IdashError(code, (self.ctx.lib.idash_server_last_error(self.h) or b"").decode())
        return {k: getattr(res, k) for k, _ in res._fields_}

    def wait(self, ticket: int) -> dict:
        res = _lib.RequestResult()
        code = self.ctx.lib.idash_server_wait(self.h, ticket, C.byref(res))
        if code != 0:
            raise IdashError(code, (self.ctx.lib.idash_server_last_error(self.h) or b"").decode())
        self._keep.pop(ticket, None)
        return {k: getattr(res, k) for k, _ in res._fields_}

    def launches(self) -> int:
        return self.ctx.lib.idash_server_launches(self.h)

    def stats(self) -> dict:
        """launches, requests_done, busy_s (device time of the scoring
        launches), h2d_bytes and d2h_bytes since the server opened."""
        st = _lib.ServerStats()
        self.ctx.check(self.ctx.lib.idash_server_get_stats(self.h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in st._fields_}

    def close(self):
        if self.h:
            h, self.h = self.h, None
            self.ctx.check(self.ctx.lib.idash_server_close(h))
            self._keep.clear()


def serve_input_shape(model, n_indiv: int, target_begin: int, target_end: int):
    """(input rows shape, output rows shape, first input row) of a served
    request: TRLWE (blocks, rows, 2N) int32, LWE (rows, stride) int32."""
    lo, hi = model.input_rows(3 * target_begin, 3 * target_end)
    n_out = 3 * (target_end - target_begin)
    if isinstance(model, LweModel):
        stride = lwe_row_words(n_indiv, model.n)
        return (hi - lo, stride), (n_out, stride), lo
    rs = model.params.region_size
    blocks = (n_indiv + rs - 1) // rs
    return (blocks, hi - lo, 2 * model.N), (blocks, n_out, 2 * model.N), lo


def synth_int16_device(ctx: Context, seed: int, n: int, max_abs: int, d_out: int):
    ctx.check(ctx.lib.idash_synth_int16_device(ctx.h, seed, n, max_abs, C.c_void_p(d_out), None))


def lwe_row_words(n_indiv: int, n: int = 1024) -> int:
    """Row stride (int32 words) of a per-individual LWE row: n_indiv*(n+1) rounded to 4."""
    return (n_indiv * (n + 1) + 3) // 4 * 4


def synth_trlwe_device(ctx: Context, seed: int, params: TrlweParams, n_tags: int, d_out: int,
                       layout: RowLayout):
    ctx.check(ctx.lib.idash_synth_trlwe_device(ctx.h, seed, C.byref(params), n_tags, C.c_void_p(d_out),
                                               C.byref(layout), None))


def synth_uniform_device(ctx: Context, seed: int, row_begin: int, n_rows: int, row_words: int, d_out: int,
                         row_stride: int):
    ctx.check(ctx.lib.idash_synth_uniform_device(ctx.h, seed, row_begin, n_rows, row_words, C.c_void_p(d_out),
                                                 row_stride, None))


def request_block_seed(seed: int, block: int) -> int:
    """Seed of individual block `block` of a serving request (idash_serve_trlwe)."""
    return (seed * 0x9E3779B97F4A7C15 + block) & ((1 << 64) - 1)


def synth_lwe_device(ctx: Context, seed: int, n: int, n_indiv: int, n_feat_rows: int, d_out: int,
                     row_stride_words: int):
    ctx.check(ctx.lib.idash_synth_lwe_device(ctx.h, seed, n, n_indiv, n_feat_rows, C.c_void_p(d_out),
                                             row_stride_words, None))


def cloud_files(params_file: str, model_dir: str, data_file: str, pred_file: str, device: int = 0) -> dict:
    """The whole cloud step on files (idash_cloud_files): eval/cloud.cpp's flow."""
    lib = _lib.load()
    rep = _lib.CloudReport()
    err = C.create_string_buffer(1024)
    code = lib.idash_cloud_files(device, params_file.encode(), model_dir.encode(), data_file.encode(),
                                 pred_file.encode(), C.byref(rep), err, len(err))
    if code != 0:
        raise IdashError(code, err.value.decode(errors="replace"))
    return {k: getattr(rep, k) for k, _ in rep._fields_}


def decrypt_device(ctx: Context, key: np.ndarray, d_in: int, layout: RowLayout, n_rows: int, num_samples: int,
                   d_out: int, stream=None):
    """Phase b - a*s of n_rows TRLWE rows at coefficients [0, num_samples),
    as float t32tod (idash_decrypt_trlwe_device); d_out: n_rows x num_samples
    float32."""
    key = np.ascontiguousarray(key, np.int32)
    ctx.check(ctx.lib.idash_decrypt_trlwe_device(ctx.h, _p(key, C.c_int32), len(key), C.c_void_p(d_in),
                                                 C.byref(layout), n_rows, num_samples, C.c_void_p(d_out),
                                                 C.c_void_p(stream) if stream else None))


def decrypt_files(keys_file: str, pred_file: str, csv_file: str, by_position: bool, device: int = 0) -> dict:
    """eval/decrypt.cpp's flow on files (idash_decrypt_files)."""
    lib = _lib.load()
    rep = _lib.DecryptReport()
    err = C.create_string_buffer(1024)
    code = lib.idash_decrypt_files(device, keys_file.encode(), pred_file.encode(), csv_file.encode(),
                                   1 if by_position else 0, C.byref(rep), err, len(err))
    if code != 0:
        raise IdashError(code, err.value.decode(errors="replace"))
    return {k: getattr(rep, k) for k, _ in rep._fields_}


def synth_key(seed: int, N: int = 1024) -> np.ndarray:
    """The binary key the synthetic generators encrypt under."""
    out = np.zeros(N, np.int32)
    _lib.load().idash_synth_key(seed, N, _p(out, C.c_int32))
    return out


def encrypt_params(num_samples: int, num_regions: int, region_size: int, alpha: float = 2.0 ** -25,
                   N: int = 1024) -> "_lib.EncryptParams":
    """Encryption parameters with the reference's message encodings
    (ONE_IN_T32 and the NaN one-hot values, eval/idash.cpp:29-45)."""
    def dtot32(d):
        return int(((d - int(d)) * 4294967296.0)) & 0xFFFFFFFF

    p = _lib.EncryptParams()
    p.N, p.k, p.num_samples, p.num_regions, p.region_size = N, 1, num_samples, num_regions, region_size
    p.one_t32 = dtot32(1.0 / 16384)
    for v, frac in enumerate((3.0 / 6.0, 2.0 / 6.0, 1.0 / 6.0)):
        p.nan_t32[v] = dtot32(frac / 16384)
    p.record_tag = 42
    p.alpha = alpha
    return p


def encrypt_device(ctx: Context, params, key: np.ndarray, seed: int, n_rows: int, d_slot_src: int, d_geno: int,
                   geno_stride: int, d_out: int, layout: RowLayout, d_row_index: int = 0, d_row_out: int = 0,
                   d_noise: int = 0, stream=None):
    """Fresh TRLWE encryptions with one-hot messages (idash_encrypt_trlwe_device)."""
    key = np.ascontiguousarray(key, np.int32)
    vp = lambda x: C.c_void_p(x) if x else None
    ctx.check(ctx.lib.idash_encrypt_trlwe_device(ctx.h, C.byref(params), _p(key, C.c_int32), seed, n_rows,
                                                 vp(d_slot_src), vp(d_geno), geno_stride, vp(d_row_index),
                                                 vp(d_row_out), C.c_void_p(d_out), C.byref(layout), vp(d_noise),
                                                 vp(stream)))


def encrypt_files(keys_file: str, challenge_file: str, data_file: str, seed: int, device: int = 0) -> dict:
    """eval/encrypt.cpp's flow on files (idash_encrypt_files)."""
    lib = _lib.load()
    rep = _lib.EncryptReport()
    err = C.create_string_buffer(1024)
    code = lib.idash_encrypt_files(device, keys_file.encode(), challenge_file.encode(), data_file.encode(), seed,
                                   C.byref(rep), err, len(err))
    if code != 0:
        raise IdashError(code, err.value.decode(errors="replace"))
    return {k: getattr(rep, k) for k, _ in rep._fields_}
