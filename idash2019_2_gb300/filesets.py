"""Seeded input directories in the reference's cloud-step file formats, at
any scale, for measuring the file pipeline:

  params.bin          IdashParams (write_params_ostream, eval/idash.cpp:128-186)
  model/<pos>_<v>.hr  one model per output: "<tagpos>_<u> <coef>" lines and a
                      "Constant <coef>" line (read_model, eval/idash.cpp:66-114)
  encrypted_data.bin  uint64 count, then records of uint32 FeatIndex, int32
                      tag 42, 2N int32 TRLWE words, double variance
                      (write_encrypted_data, eval/idash.cpp:536-556)
  keys.bin, tags.txt  party A's inputs (optional): the secret key after the
                      params (eval/idash.cpp:474-502) and the tag genotypes
                      (read_plaintext_data, eval/idash.cpp:280-309)

Every target takes its `neighbours` nearest tags; coefficients are seeded
integers in [-8192, 8192).  The ciphertexts are uniformly random words (the
cloud step's arithmetic does not depend on them being encryptions).  All
loops are vectorised except the one write per model file.
"""
from __future__ import annotations

import os

import numpy as np

N = 1024
RECORD_TAG = 42


def _positions(rng, n_tags: int, n_targets: int):
    tag_pos = 1000 + 37 * np.arange(n_tags, dtype=np.int64) + rng.integers(0, 30, n_tags)
    lo, hi = int(tag_pos[0]) + 1, int(tag_pos[-1])
    tgt = np.sort(rng.integers(lo, max(hi, lo + 1), n_targets))
    tgt = tgt + np.arange(n_targets)  # distinct, still sorted
    return tag_pos, tgt


def _nearest(tag_pos, tgt, k: int) -> np.ndarray:
    """[n_targets, k] indices of each target's k nearest tags, ascending."""
    n = len(tag_pos)
    k = min(k, n)
    at = np.searchsorted(tag_pos, tgt)
    start = np.clip(at - k, 0, max(n - 2 * k, 0))
    cand = start[:, None] + np.arange(min(2 * k, n))[None, :]
    dist = np.abs(tag_pos[cand] - tgt[:, None])
    pick = np.argsort(dist, axis=1, kind="stable")[:, :k]
    return np.sort(np.take_along_axis(cand, pick, axis=1), axis=1)


def write_params(path: str, n_indiv: int, tag_pos, tgt) -> None:
    P, T = len(tag_pos), len(tgt)
    R = N // n_indiv
    hdr = np.array([n_indiv, P, T, 3 * P + 1, 3 * T, R, N // R], dtype="<u4").tobytes()
    ins = np.zeros(P, dtype=[("pos", "<u8"), ("f", "<u4", (3,))])
    ins["pos"] = tag_pos
    ins["f"] = 3 * np.arange(P, dtype=np.uint32)[:, None] + np.arange(3, dtype=np.uint32)[None, :]
    outs = []
    for i, pos in enumerate(tgt.tolist()):
        outs.append(int(pos).to_bytes(8, "little") + str(pos).encode() + b"\0" +
                    np.array([3 * i, 3 * i + 1, 3 * i + 2], dtype="<u4").tobytes())
    with open(path, "wb") as f:
        f.write(hdr)
        f.write(ins.tobytes())
        f.write(b"".join(outs))


def write_models(model_dir: str, rng, tag_pos, tgt, near) -> int:
    """One .hr file per output; returns the number of terms written."""
    os.makedirs(model_dir, exist_ok=True)
    T, k = near.shape
    coef = rng.integers(-8192, 8192, size=(T, 3, k, 3))
    coef[coef == 0] = 1
    const = rng.integers(-8192, 8192, size=(T, 3))
    names = np.char.add(np.char.add(tag_pos[near].astype(str)[:, :, None], "_"),
                        np.arange(3).astype(str)[None, None, :])  # [T, k, 3]
    terms = 0
    for ti in range(T):
        flat = names[ti].reshape(-1)
        for v in range(3):
            c = coef[ti, v].reshape(-1)
            body = "\n".join(f"{nm} {cv}" for nm, cv in zip(flat, c.tolist()))
            with open(os.path.join(model_dir, f"{int(tgt[ti])}_{v}.hr"), "w") as f:
                f.write(f"{body}\nConstant {int(const[ti, v])}\n")
            terms += len(c) + 1
    return terms


def write_ciphertexts(path: str, rng, n_rows: int, variance: float = 2.0 ** -50) -> None:
    rec = np.zeros(n_rows, dtype=[("idx", "<u4"), ("tag", "<i4"), ("coef", "<u4", (2 * N,)), ("var", "<f8")])
    rec["idx"] = np.arange(n_rows, dtype=np.uint32)
    rec["tag"] = RECORD_TAG
    rec["coef"] = rng.integers(0, 2 ** 32, size=(n_rows, 2 * N), dtype=np.uint64).astype(np.uint32)
    rec["var"] = variance
    with open(path, "wb") as f:
        f.write(np.uint64(n_rows).tobytes())
        f.write(rec.tobytes())


def write_keys(path: str, params_path: str, rng) -> np.ndarray:
    """keys.bin as the reference's keygen writes it (eval/idash.cpp:474-502):
    params.bin's bytes, then the TRLWE key record: int32 tag 52, N, k = 1,
    double alpha_min and alpha_max, N binary int32 coefficients."""
    key = rng.integers(0, 2, size=N).astype("<i4")
    with open(params_path, "rb") as f:
        params = f.read()
    with open(path, "wb") as f:
        f.write(params)
        f.write(np.array([52, N, 1], dtype="<i4").tobytes())
        f.write(np.array([2.0 ** -25, 2.0 ** -10], dtype="<f8").tobytes())
        f.write(key.tobytes())
    return key


def write_challenge(path: str, rng, tag_pos, n_indiv: int, missing: float = 0.05) -> None:
    """The tag genotypes (read_plaintext_data, eval/idash.cpp:280-309): per tag
    "22 <pos> <pos+1> rs<pos> <g_0> ... <g_{n-1}>", '.' for a missing value."""
    geno = rng.integers(0, 3, size=(len(tag_pos), n_indiv)).astype(np.uint8) + ord("0")
    geno[rng.random(size=geno.shape) < missing] = ord(".")
    cells = np.full((len(tag_pos), 2 * n_indiv), ord(" "), dtype=np.uint8)
    cells[:, 0::2] = geno
    cells[:, -1] = ord("\n")
    with open(path, "wb") as f:
        for i, pos in enumerate(tag_pos.tolist()):
            f.write(f"22 {pos} {pos + 1} rs{pos} ".encode())
            f.write(cells[i].tobytes())


def write_cloud_inputs(d: str, seed: int, n_indiv: int, n_tags: int, n_targets: int, neighbours: int = 5,
                       party_a: bool = False) -> dict:
    """params.bin, model/ and encrypted_data.bin for one cloud step in `d`;
    with party_a, also keys.bin and the tag genotypes file tags.txt."""
    os.makedirs(d, exist_ok=True)
    rng = np.random.default_rng(seed)
    tag_pos, tgt = _positions(rng, n_tags, n_targets)
    near = _nearest(tag_pos, tgt, neighbours)
    write_params(os.path.join(d, "params.bin"), n_indiv, tag_pos, tgt)
    terms = write_models(os.path.join(d, "model"), rng, tag_pos, tgt, near)
    R = N // n_indiv
    n_rows = (3 * n_tags + R - 1) // R
    write_ciphertexts(os.path.join(d, "encrypted_data.bin"), rng, n_rows)
    if party_a:
        write_keys(os.path.join(d, "keys.bin"), os.path.join(d, "params.bin"), rng)
        write_challenge(os.path.join(d, "tags.txt"), rng, tag_pos, n_indiv)
    return {"outputs": 3 * n_targets, "terms": terms, "in_records": n_rows}
