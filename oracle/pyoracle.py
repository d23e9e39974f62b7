"""pyoracle — TEST INFRASTRUCTURE ONLY (checker for tests/, smoke() and the
CPU-baseline leg of bench.py; nothing in the product imports it).

numpy/ctypes glue around liboracle.so (the C restatement in oracle.c) plus
readers of the reference's file formats and two restatements used for
semantic checks:
  phase()          tLwePhase (eval/idash.cpp:714): b - a*s mod X^N+1
  plaintext_score  compute_score (eval/idash.cpp:888-927) in exact integers
"""
from __future__ import annotations

import ctypes as C
import os
import struct
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
CONST = 0xFFFFFFFF
N = 1024
ONE_IN_T32 = 1 << 18

_lib = None


def build() -> None:
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        u64p, u32p, i32p, i16p, f64p = (C.POINTER(C.c_uint64), C.POINTER(C.c_uint32), C.POINTER(C.c_int32),
                                         C.POINTER(C.c_int16), C.POINTER(C.c_double))
        L.oracle_trlwe_score.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_int32, C.c_uint64,
                                         u64p, u32p, i32p, u32p, C.c_uint64, C.c_uint64, i32p, f64p, i32p, f64p,
                                         C.c_int]
        L.oracle_lwe_score.argtypes = [C.c_uint32, C.c_uint32, C.c_int32, C.c_uint64, u64p, u32p, i32p,
                                       C.c_uint64, i32p, C.c_uint64, C.c_uint64, C.c_uint64, i32p, C.c_uint64,
                                       C.c_int]
        L.oracle_intpoly_score.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32, C.c_int32, C.c_uint64, u64p, u32p,
                                           i16p, i32p, C.c_uint64, i32p, C.c_uint64, C.c_uint64, i32p, C.c_int]
        L.oracle_sample_extract.argtypes = [C.c_uint32, i32p, C.c_uint32, i32p]
        L.oracle_sample_extract.restype = None
        L.oracle_trlwe_decrypt.argtypes = [C.c_uint32, i32p, C.c_uint64, C.c_uint64, i32p, C.c_uint32,
                                           C.POINTER(C.c_float), C.c_int]
        L.oracle_trlwe_decrypt.restype = None
        L.oracle_hash32.argtypes = [C.c_uint64, C.c_uint64, C.c_uint64]
        L.oracle_hash32.restype = C.c_uint32
        L.oracle_synth_lwe_words.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint64, C.c_uint64,
                                             C.c_uint64, i32p]
        L.oracle_synth_lwe_words.restype = None
        L.oracle_synth_model.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, u32p,
                                         C.POINTER(SynthModel)]
        L.oracle_synth_model_free.argtypes = [C.POINTER(SynthModel)]
        L.oracle_synth_model_free.restype = None
        _lib = L
    return _lib


class SynthModel(C.Structure):
    _fields_ = [("n_out", C.c_uint64), ("n_terms", C.c_uint64), ("term_ptr", C.POINTER(C.c_uint64)),
                ("term_feat", C.POINTER(C.c_uint32)), ("term_coef", C.POINTER(C.c_int32)),
                ("window_start", C.POINTER(C.c_uint32)), ("window_len", C.POINTER(C.c_uint32))]


def synth_model(seed, n_tags, n_targets, neighbours=5, choices=None):
    """The seeded synthetic model (oracle_synth_model): returns
    (term_ptr, term_feat, term_coef, window_start, window_len) arrays."""
    ch = None if not choices else np.ascontiguousarray(choices, np.uint32)
    m = SynthModel()
    rc = lib().oracle_synth_model(seed, n_tags, n_targets, 0 if ch is not None else neighbours,
                                  0 if ch is None else len(ch), _p(ch, C.c_uint32), C.byref(m))
    if rc != 0:
        raise ValueError("oracle_synth_model failed")
    try:
        arr = np.ctypeslib.as_array
        out = (arr(m.term_ptr, (m.n_out + 1,)).copy(), arr(m.term_feat, (m.n_terms,)).copy(),
               arr(m.term_coef, (m.n_terms,)).copy(),
               arr(m.window_start, (n_targets,)).copy() if n_targets else np.zeros(0, np.uint32),
               arr(m.window_len, (n_targets,)).copy() if n_targets else np.zeros(0, np.uint32))
    finally:
        lib().oracle_synth_model_free(C.byref(m))
    return out


def _p(a, t):
    return None if a is None else a.ctypes.data_as(C.POINTER(t))


def trlwe_score(term_ptr, term_feat, term_coef, rows, num_samples, num_regions, region_size, in_var=None,
                row_of_index=None, one_t32=ONE_IN_T32, n_threads=0):
    """Oracle B, TRLWE form: returns (out [n_out, 2N] int32, out_var [n_out])."""
    tp = np.ascontiguousarray(term_ptr, np.uint64)
    tf = np.ascontiguousarray(term_feat, np.uint32)
    tc = np.ascontiguousarray(term_coef, np.int32)
    rows = np.ascontiguousarray(rows, np.int32)
    n_out = len(tp) - 1
    out = np.zeros((n_out, rows.shape[1]), np.int32)
    ov = np.zeros(n_out, np.float64)
    iv = None if in_var is None else np.ascontiguousarray(in_var, np.float64)
    ri = None if row_of_index is None else np.ascontiguousarray(row_of_index, np.uint32)
    rc = lib().oracle_trlwe_score(rows.shape[1] // 2, num_samples, num_regions, region_size, one_t32, n_out,
                                  _p(tp, C.c_uint64), _p(tf, C.c_uint32), _p(tc, C.c_int32), _p(ri, C.c_uint32),
                                  0 if ri is None else len(ri), rows.shape[0], _p(rows, C.c_int32),
                                  _p(iv, C.c_double), _p(out, C.c_int32), _p(ov, C.c_double), n_threads)
    if rc != 0:
        raise ValueError(f"oracle_trlwe_score failed ({rc})")
    return out, ov


def lwe_score(term_ptr, term_feat, term_coef, rows, n_indiv, out_begin, out_end, n=N, one_t32=ONE_IN_T32,
              n_threads=0):
    """Oracle B, per-individual LWE form.  rows: int32 [n_feat, stride]."""
    tp = np.ascontiguousarray(term_ptr, np.uint64)
    tf = np.ascontiguousarray(term_feat, np.uint32)
    tc = np.ascontiguousarray(term_coef, np.int32)
    rows = np.ascontiguousarray(rows, np.int32)
    L = n_indiv * (n + 1)
    out = np.zeros((out_end - out_begin, L), np.int32)
    rc = lib().oracle_lwe_score(n, n_indiv, one_t32, len(tp) - 1, _p(tp, C.c_uint64), _p(tf, C.c_uint32),
                                _p(tc, C.c_int32), rows.shape[0], _p(rows, C.c_int32), rows.shape[1], out_begin,
                                out_end, _p(out, C.c_int32), L, n_threads)
    if rc != 0:
        raise ValueError(f"oracle_lwe_score failed ({rc})")
    return out


def intpoly_score(term_ptr, term_feat, term_poly, bias, rows, num_samples, region_size, out_begin, out_end,
                  one_t32=ONE_IN_T32, n_threads=0):
    """Oracle B, integer-polynomial form (exact schoolbook negacyclic product)."""
    tp = np.ascontiguousarray(term_ptr, np.uint64)
    tf = np.ascontiguousarray(term_feat, np.uint32)
    tw = np.ascontiguousarray(term_poly, np.int16)
    b = np.ascontiguousarray(bias, np.int32)
    rows = np.ascontiguousarray(rows, np.int32)
    N = rows.shape[1] // 2
    out = np.zeros((out_end - out_begin, 2 * N), np.int32)
    rc = lib().oracle_intpoly_score(N, num_samples, region_size, one_t32, len(tp) - 1, _p(tp, C.c_uint64),
                                    _p(tf, C.c_uint32), _p(tw, C.c_int16), _p(b, C.c_int32), rows.shape[0],
                                    _p(rows, C.c_int32), out_begin, out_end, _p(out, C.c_int32), n_threads)
    if rc != 0:
        raise ValueError(f"oracle_intpoly_score failed ({rc})")
    return out


def sample_extract(trlwe_row: np.ndarray, slot: int) -> np.ndarray:
    row = np.ascontiguousarray(trlwe_row, np.int32)
    out = np.zeros(len(row) // 2 + 1, np.int32)
    lib().oracle_sample_extract(len(row) // 2, _p(row, C.c_int32), slot, _p(out, C.c_int32))
    return out


def trlwe_decrypt(rows: np.ndarray, key: np.ndarray, num_samples: int, n_threads: int = 0) -> np.ndarray:
    """Phase b - a*s of each TRLWE row at coefficients [0, num_samples) as
    float t32tod (decrypt_predictions, eval/idash.cpp:682-761); rows are
    [n][stride] int32 with a at word 0 and b at word N."""
    rows = np.ascontiguousarray(rows, np.int32)
    key = np.ascontiguousarray(key, np.int32)
    out = np.zeros((rows.shape[0], num_samples), np.float32)
    lib().oracle_trlwe_decrypt(len(key), _p(key, C.c_int32), rows.shape[0], rows.shape[1], _p(rows, C.c_int32),
                               num_samples, out.ctypes.data_as(C.POINTER(C.c_float)), n_threads or os.cpu_count())
    return out


def synth_lwe_words(seed, n, n_indiv, feature, w0, count):
    out = np.zeros(count, np.int32)
    lib().oracle_synth_lwe_words(seed, n, n_indiv, feature, w0, count, _p(out, C.c_int32))
    return out


# ---------------------------------------------------------------- file formats
RECORD = np.dtype([("idx", "<u4"), ("tag", "<i4"), ("coef", "<i4", (2 * N,)), ("var", "<f8")])


def read_records(path: str) -> np.ndarray:
    """encrypted_data.bin / encrypted_prediction.bin (eval/idash.cpp:540-556)."""
    raw = open(path, "rb").read()
    (count,) = struct.unpack_from("<Q", raw, 0)
    assert len(raw) == 8 + count * RECORD.itemsize, "record file size mismatch"
    return np.frombuffer(raw, dtype=RECORD, offset=8, count=count)


def read_params(path: str) -> dict:
    """params.bin (eval/idash.cpp:200-261)."""
    raw = open(path, "rb").read()
    hdr = struct.unpack_from("<7I", raw, 0)
    keys = ["NUM_SAMPLES", "NUM_INPUT_POSITIONS", "NUM_OUTPUT_POSITIONS", "NUM_INPUT_FEATURES",
            "NUM_OUTPUT_FEATURES", "NUM_REGIONS", "REGION_SIZE"]
    p = dict(zip(keys, hdr))
    off = 28
    p["in"] = {}
    for _ in range(p["NUM_INPUT_POSITIONS"]):
        pos, a, b, c = struct.unpack_from("<Q3I", raw, off)
        off += 20
        p["in"][pos] = (a, b, c)
    p["out"] = {}
    p["out_names"] = []
    for _ in range(p["NUM_OUTPUT_POSITIONS"]):
        (pos,) = struct.unpack_from("<Q", raw, off)
        off += 8
        end = raw.index(b"\0", off)
        name = raw[off:end].decode()
        off = end + 1
        a, b, c = struct.unpack_from("<3I", raw, off)
        off += 12
        p["out"][pos] = (a, b, c)
        p["out_names"].append((pos, name))
    return p


def read_model(params: dict, model_dir: str) -> dict:
    """<pos>_<snp>.hr files -> {out_bidx: [(in_bidx, coef), ...]} (later lines
    overwrite earlier ones, eval/parse_vw.cpp:24; eval/idash.cpp:66-114)."""
    model = {}
    for pos, bidx in params["out"].items():
        for snp in range(3):
            coefs = {}
            for line in open(os.path.join(model_dir, f"{pos}_{snp}.hr")):
                parts = line.split()
                if len(parts) >= 2:
                    coefs[parts[0]] = int(parts[1])
            terms = []
            for name, c in coefs.items():
                if name == "Constant":
                    terms.append((CONST, c))
                else:
                    ip, iv = name.split("_")
                    terms.append((params["in"][int(ip)][int(iv)], c))
            model[bidx[snp]] = terms
    return model


def model_csr(model: dict, order=None):
    outs = sorted(model) if order is None else list(order)
    ptr = [0]
    feat, coef = [], []
    for o in outs:
        for f, c in model[o]:
            feat.append(f)
            coef.append(c)
        ptr.append(len(feat))
    return (np.array(outs, np.uint32), np.array(ptr, np.uint64), np.array(feat, np.uint32),
            np.array(coef, np.int64).astype(np.uint32).view(np.int32))


def read_key(path: str, params_bytes: int | None = None) -> np.ndarray:
    """keys.bin: params.bin body then the tfhe_compat key record
    (tag, N, k, alpha_min, alpha_max, k*N int32)."""
    raw = open(path, "rb").read()
    # the key record is the trailing 12 + 16 + 4*N bytes (k = 1)
    rec = raw[len(raw) - (12 + 16 + 4 * N):]
    tag, n, k = struct.unpack_from("<3i", rec, 0)
    assert (tag, n, k) == (52, N, 1), "unexpected key record"
    return np.frombuffer(rec, dtype="<i4", offset=28, count=N).copy()


def negacyclic_mul(key: np.ndarray, a: np.ndarray) -> np.ndarray:
    """(key * a) mod (X^N + 1, 2^32) for a binary key, exact."""
    n = len(a)
    a64 = a.astype(np.int64)
    out = np.zeros(n, np.int64)
    for i in np.nonzero(key)[0]:
        out += np.concatenate([-a64[n - i:], a64[:n - i]]) if i else a64
    return (out & 0xFFFFFFFF).astype(np.uint32)


def phase(row: np.ndarray, key: np.ndarray) -> np.ndarray:
    """tLwePhase: b - a*s, as uint32 (eval/idash.cpp:714)."""
    a = row[:N].astype(np.uint32)
    b = row[N:].astype(np.uint32)
    return (b - negacyclic_mul(key, a)).astype(np.uint32)


def torus_to_double(x: np.ndarray) -> np.ndarray:
    """t32tod (eval/idash.cpp:718)."""
    return x.astype(np.uint32).view(np.int32).astype(np.float64) / 2.0 ** 32


def plaintext_scores(params: dict, model: dict, tags_file: str) -> dict:
    """compute_score (eval/idash.cpp:850-927): {out_bidx: scores[NUM_SAMPLES]}
    in units of the torus, from the plaintext genotypes."""
    ns = params["NUM_SAMPLES"]
    one = 2.0 ** -14
    nan_val = [3 / 6 * one, 2 / 6 * one, 1 / 6 * one]
    onehot = {}
    for line in open(tags_file):
        parts = line.split()
        pos = int(parts[1])
        if pos not in params["in"]:
            continue
        g = parts[4:4 + ns]
        for v in range(3):
            vals = np.array([(one if x == str(v) else 0.0) if x in ("0", "1", "2") else nan_val[v] for x in g])
            onehot[params["in"][pos][v]] = vals
    out = {}
    for o, terms in model.items():
        s = np.zeros(ns)
        for f, c in terms:
            s += c * (one if f == CONST else onehot[f])
        out[o] = s
    return out
