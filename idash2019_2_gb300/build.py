"""In-tree build of the GB300 scoring library.

Compiles every CUDA/C++ source for sm_103a with nvcc (one process per
translation unit, in parallel) and links, inside the package directory:

  libidash_gpu.so   the C ABI declared in include/idash_gpu.h
  idash_cloud       the cloud CLI (eval/cloud.cpp's argv and output)
  idash_decrypt     the decryption CLI (eval/decrypt.cpp's argv and output)
  idash_encrypt     the encryption CLI (eval/encrypt.cpp's argv and output)

Objects go to idash2019_2_gb300/_build/ (git-ignored).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libidash_gpu.so")
CLI = os.path.join(PKG, "idash_cloud")
DECRYPT_CLI = os.path.join(PKG, "idash_decrypt")
ENCRYPT_CLI = os.path.join(PKG, "idash_encrypt")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O3",
                     "-I" + os.path.join(ROOT, "include"), "--expt-relaxed-constexpr"]

LIB_SOURCES = [
    "csrc/score_kernels.cu",
    "csrc/score_tc.cu",
    "csrc/synth.cu",
    "csrc/noalloc.cu",
    "csrc/noalloc_plan.cpp",
    "csrc/intpoly.cu",
    "csrc/server.cpp",
    "csrc/capi.cpp",
    "csrc/plan.cpp",
    "csrc/decrypt.cu",
    "csrc/encrypt.cu",
    "csrc/host/idash_host.cpp",
    "csrc/host/decrypt_host.cpp",
    "csrc/host/encrypt_host.cpp",
]
CLIS = {CLI: ["csrc/host/cloud_main.cpp"], DECRYPT_CLI: ["csrc/host/decrypt_main.cpp"],
        ENCRYPT_CLI: ["csrc/host/encrypt_main.cpp"]}


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the GB300 kernels cannot be built")


def _obj(src: str) -> str:
    return os.path.join(BUILD, src.replace("/", "_") + ".o")


def _deps_newer(target: str, srcs: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in srcs)


def _headers() -> list[str]:
    hs = [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    for d, _, fs in os.walk(CSRC):
        hs += [os.path.join(d, f) for f in fs if f.endswith((".hpp", ".cuh", ".h"))]
    return hs


def _compile(nvcc: str, src: str, verbose: bool) -> str:
    path = os.path.join(PKG, src)
    out = _obj(src)
    if not _deps_newer(out, [path] + _headers()):
        return out
    lang = ["-x", "cu"] if src.endswith(".cu") else []
    cmd = [nvcc, *NVCC_FLAGS, *lang, "-c", path, "-o", out]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return out


def build(verbose: bool = False) -> None:
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    srcs = LIB_SOURCES + [s for v in CLIS.values() for s in v]
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 2)) as ex:
        objs = dict(zip(srcs, ex.map(lambda s: _compile(nvcc, s, verbose), srcs)))
    lib_objs = [objs[s] for s in LIB_SOURCES]
    if _deps_newer(LIB, lib_objs):
        cmd = [nvcc, *ARCH, "-shared", "-o", LIB, *lib_objs, "-cudart", "static"]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)
    for exe, main_srcs in CLIS.items():
        exe_objs = lib_objs + [objs[s] for s in main_srcs]
        if _deps_newer(exe, exe_objs):
            cmd = [nvcc, *ARCH, "-o", exe, *exe_objs, "-cudart", "static"]
            if verbose:
                print(" ".join(cmd), flush=True)
            subprocess.run(cmd, check=True)


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
