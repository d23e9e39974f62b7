"""ctypes binding of libidash_gpu.so (the C ABI in include/idash_gpu.h).

The library is built in-tree by idash2019_2_gb300.build.build().  Loading
fails loudly when it is missing: there is no CPU implementation behind this
module.
"""
from __future__ import annotations

import ctypes as C
import os
import re

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
LIB_PATH = os.path.join(PKG, "libidash_gpu.so")
HEADER = os.path.join(ROOT, "include", "idash_gpu.h")

u8p = C.POINTER(C.c_uint8)
u32p = C.POINTER(C.c_uint32)
u64p = C.POINTER(C.c_uint64)
i32p = C.POINTER(C.c_int32)
i16p = C.POINTER(C.c_int16)
vp = C.c_void_p
status_t = C.c_int

CONSTANT_FEATURE = 0xFFFFFFFF

STATUS = {
    0: "IDASH_OK", 1: "IDASH_ERR_INVALID_ARGUMENT", 2: "IDASH_ERR_CUDA", 3: "IDASH_ERR_OUT_OF_MEMORY",
    4: "IDASH_ERR_INDEX", 5: "IDASH_ERR_DEVICE_TIMEOUT", 6: "IDASH_ERR_IO", 7: "IDASH_ERR_FORMAT",
    8: "IDASH_ERR_UNSUPPORTED", 9: "IDASH_ERR_ADMISSION", 10: "IDASH_ERR_STATE", 11: "IDASH_PENDING",
}


class IdashError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"{STATUS.get(code, code)}: {message}")
        self.code = code
        self.name = STATUS.get(code, str(code))


class RowLayout(C.Structure):
    _fields_ = [("row_stride", C.c_uint64), ("payload_offset", C.c_uint64),
                ("variance_offset", C.c_int64), ("header_offset", C.c_int64)]


class TrlweParams(C.Structure):
    _fields_ = [("N", C.c_uint32), ("k", C.c_uint32), ("num_samples", C.c_uint32),
                ("num_regions", C.c_uint32), ("region_size", C.c_uint32), ("one_t32", C.c_int32),
                ("record_tag", C.c_int32)]


class LweParams(C.Structure):
    _fields_ = [("n", C.c_uint32), ("n_indiv", C.c_uint32), ("one_t32", C.c_int32)]


class IntpolyParams(C.Structure):
    _fields_ = [("N", C.c_uint32), ("num_samples", C.c_uint32), ("region_size", C.c_uint32),
                ("one_t32", C.c_int32), ("max_abs_coef", C.c_int32)]


class Stats(C.Structure):
    _fields_ = [("kernel_launches", C.c_uint64), ("graph_launches", C.c_uint64),
                ("h2d_bytes", C.c_uint64), ("d2h_bytes", C.c_uint64)]


class ModelInfo(C.Structure):
    _fields_ = [("n_out", C.c_uint64), ("n_terms", C.c_uint64), ("n_groups", C.c_uint64),
                ("n_blocks", C.c_uint64), ("n_slots", C.c_uint64), ("slice_words", C.c_uint32),
                ("max_window_slots", C.c_uint32), ("kernel", C.c_uint32), ("algorithmic_in_rows", C.c_uint64),
                ("dense_k", C.c_uint64)]


class SynthSpec(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("n_tags", C.c_uint32), ("n_targets", C.c_uint32),
                ("neighbours", C.c_uint32), ("n_choices", C.c_uint32), ("choices", C.c_uint32 * 8)]


class SynthModel(C.Structure):
    _fields_ = [("n_out", C.c_uint64), ("n_terms", C.c_uint64), ("term_ptr", u64p), ("term_feat", u32p),
                ("term_coef", i32p), ("tag_pos", u64p), ("target_pos", u64p), ("window_start", u32p),
                ("window_len", u32p)]


class Request(C.Structure):
    _fields_ = [("arrival_s", C.c_double), ("n_indiv", C.c_uint32), ("reserved", C.c_uint32),
                ("target_begin", C.c_uint64), ("target_end", C.c_uint64), ("seed", C.c_uint64)]


class RequestResult(C.Structure):
    _fields_ = [("admit_s", C.c_double), ("done_s", C.c_double), ("device_bytes", C.c_uint64),
                ("digest", C.c_uint64)]


class ServeConfig(C.Structure):
    _fields_ = [("hbm_budget", C.c_uint64), ("max_inflight", C.c_uint32), ("segment_outputs", C.c_uint32)]


class ServeRequest(C.Structure):
    _fields_ = [("n_indiv", C.c_uint32), ("reserved", C.c_uint32), ("target_begin", C.c_uint64),
                ("target_end", C.c_uint64), ("h_in", C.c_void_p), ("h_out", C.c_void_p), ("seed", C.c_uint64)]


class ServerStats(C.Structure):
    _fields_ = [("launches", C.c_uint64), ("requests_done", C.c_uint64), ("busy_s", C.c_double),
                ("h2d_bytes", C.c_uint64), ("d2h_bytes", C.c_uint64)]


class CloudReport(C.Structure):
    _fields_ = [("read_s", C.c_double), ("plan_s", C.c_double), ("score_s", C.c_double),
                ("write_s", C.c_double), ("n_in_records", C.c_uint64), ("n_out_records", C.c_uint64),
                ("model_from_cache", C.c_uint32), ("reserved", C.c_uint32)]


class DecryptReport(C.Structure):
    _fields_ = [("read_s", C.c_double), ("decrypt_s", C.c_double), ("write_s", C.c_double),
                ("n_records", C.c_uint64), ("n_lines", C.c_uint64)]


class EncryptParams(C.Structure):
    _fields_ = [("N", C.c_uint32), ("k", C.c_uint32), ("num_samples", C.c_uint32), ("num_regions", C.c_uint32),
                ("region_size", C.c_uint32), ("one_t32", C.c_int32), ("nan_t32", C.c_int32 * 3),
                ("record_tag", C.c_int32), ("alpha", C.c_double)]


class EncryptReport(C.Structure):
    _fields_ = [("read_s", C.c_double), ("encrypt_s", C.c_double), ("write_s", C.c_double),
                ("n_positions", C.c_uint64), ("n_records", C.c_uint64)]


# name -> (restype, argtypes); every function include/idash_gpu.h declares.
PROTOTYPES = {
    "idash_status_string": (C.c_char_p, [status_t]),
    "idash_abi_version": (C.c_int, []),
    "idash_open": (status_t, [C.POINTER(vp), C.c_int]),
    "idash_close": (None, [vp]),
    "idash_last_error": (C.c_char_p, [vp]),
    "idash_stream": (vp, [vp]),
    "idash_sync": (status_t, [vp]),
    "idash_set_option": (status_t, [vp, C.c_char_p, C.c_int64]),
    "idash_get_option": (status_t, [vp, C.c_char_p, C.POINTER(C.c_int64)]),
    "idash_get_stats": (status_t, [vp, C.POINTER(Stats)]),
    "idash_device_alloc": (status_t, [vp, C.c_size_t, C.POINTER(vp)]),
    "idash_device_free": (status_t, [vp, vp]),
    "idash_host_alloc": (status_t, [vp, C.c_size_t, C.POINTER(vp)]),
    "idash_host_free": (status_t, [vp, vp]),
    "idash_copy_h2d": (status_t, [vp, vp, vp, C.c_size_t]),
    "idash_copy_d2h": (status_t, [vp, vp, vp, C.c_size_t]),
    "idash_memset_device": (status_t, [vp, vp, C.c_int, C.c_size_t]),
    "idash_model_trlwe": (status_t, [vp, C.POINTER(vp), C.POINTER(TrlweParams), C.c_uint64, u32p, u32p, u64p,
                                     u32p, i32p, C.c_uint64, u32p, C.c_uint64]),
    "idash_score_trlwe_device": (status_t, [vp, vp, C.POINTER(RowLayout), vp, C.POINTER(RowLayout), vp]),
    "idash_score_trlwe_host": (status_t, [vp, vp, C.POINTER(RowLayout), C.c_uint64, vp, C.POINTER(RowLayout)]),
    "idash_model_lwe": (status_t, [vp, C.POINTER(vp), C.POINTER(LweParams), C.c_uint64, u64p, u32p, i32p,
                                   C.c_uint64]),
    "idash_score_lwe_device": (status_t, [vp, C.c_uint32, vp, C.c_uint64, C.c_uint64, C.c_uint64, vp,
                                          C.c_uint64, vp]),
    "idash_score_trlwe_range": (status_t, [vp, C.c_uint64, C.c_uint64, C.c_uint32, vp, C.POINTER(RowLayout),
                                           C.c_uint64, C.c_uint64, vp, C.POINTER(RowLayout), vp]),
    "idash_model_input_rows": (status_t, [vp, C.c_uint64, C.c_uint64, u64p, u64p]),
    "idash_server_open": (status_t, [vp, C.POINTER(ServeConfig), C.POINTER(vp)]),
    "idash_server_submit": (status_t, [vp, C.POINTER(ServeRequest), C.POINTER(C.c_uint64)]),
    "idash_server_poll": (status_t, [vp, C.c_uint64, C.POINTER(RequestResult)]),
    "idash_server_wait": (status_t, [vp, C.c_uint64, C.POINTER(RequestResult)]),
    "idash_server_launches": (C.c_uint64, [vp]),
    "idash_server_get_stats": (status_t, [vp, C.POINTER(ServerStats)]),
    "idash_server_close": (status_t, [vp]),
    "idash_server_last_error": (C.c_char_p, [vp]),
    "idash_serve_trlwe": (status_t, [vp, C.POINTER(ServeConfig), C.POINTER(Request), C.c_uint64,
                                     C.POINTER(RequestResult), C.POINTER(vp)]),
    "idash_digest_host": (C.c_uint64, [u32p, C.c_uint64, C.c_uint64]),
    "idash_synth_uniform_device": (status_t, [vp, C.c_uint64, C.c_uint64, C.c_uint64, C.c_uint32, vp, C.c_uint64,
                                              vp]),
    "idash_model_intpoly": (status_t, [vp, C.POINTER(vp), C.POINTER(IntpolyParams), C.c_uint64, u64p, u32p, i32p,
                                       C.c_uint64, vp, C.c_int]),
    "idash_model_intpoly_set_weights": (status_t, [vp, vp, vp]),
    "idash_score_intpoly_device": (status_t, [vp, vp, C.POINTER(RowLayout), C.c_uint64, C.c_uint64, vp,
                                              C.POINTER(RowLayout), vp]),
    "idash_synth_int16_device": (status_t, [vp, C.c_uint64, C.c_uint64, C.c_int32, vp, vp]),
    "idash_model_get_info": (status_t, [vp, C.POINTER(ModelInfo)]),
    "idash_model_replan": (status_t, [vp]),
    "idash_model_free": (None, [vp]),
    "idash_score_trlwe_noalloc": (status_t, [C.POINTER(TrlweParams), C.c_uint64, u32p, u64p, u32p, i32p,
                                             C.c_uint64, u32p, C.c_uint64, vp, C.POINTER(RowLayout), vp,
                                             C.POINTER(RowLayout), vp]),
    "idash_cloud_files": (status_t, [C.c_int, C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p,
                                     C.POINTER(CloudReport), C.c_char_p, C.c_size_t]),
    "idash_encrypt_trlwe_device": (status_t, [vp, C.POINTER(EncryptParams), i32p, C.c_uint64, C.c_uint64, vp,
                                              vp, C.c_uint32, vp, vp, vp, C.POINTER(RowLayout), vp, vp]),
    "idash_encrypt_files": (status_t, [C.c_int, C.c_char_p, C.c_char_p, C.c_char_p, C.c_uint64,
                                       C.POINTER(EncryptReport), C.c_char_p, C.c_size_t]),
    "idash_decrypt_trlwe_device": (status_t, [vp, i32p, C.c_uint32, vp, C.POINTER(RowLayout), C.c_uint64,
                                              C.c_uint32, vp, vp]),
    "idash_decrypt_files": (status_t, [C.c_int, C.c_char_p, C.c_char_p, C.c_char_p, C.c_int,
                                       C.POINTER(DecryptReport), C.c_char_p, C.c_size_t]),
    "idash_synth_key": (None, [C.c_uint64, C.c_uint32, i32p]),
    "idash_synth_model": (status_t, [C.POINTER(SynthSpec), C.POINTER(SynthModel)]),
    "idash_synth_model_free": (None, [C.POINTER(SynthModel)]),
    "idash_synth_lwe_device": (status_t, [vp, C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint64, vp, C.c_uint64,
                                          vp]),
    "idash_synth_trlwe_device": (status_t, [vp, C.c_uint64, C.POINTER(TrlweParams), C.c_uint32, vp,
                                            C.POINTER(RowLayout), vp]),
}


def declared_functions() -> list[str]:
    """Function names declared in include/idash_gpu.h."""
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(idash_[a-z0-9_]+)\s*\(", text)) - {"idash_status"})


_lib = None


def load() -> C.CDLL:
    """Loads the in-tree library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: run __graft_entry__.build() (nvcc, sm_103a) first")
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(code: int, ctx=None) -> None:
    if code != 0:
        lib = load()
        msg = lib.idash_last_error(ctx)
        raise IdashError(code, (msg or b"").decode(errors="replace"))
