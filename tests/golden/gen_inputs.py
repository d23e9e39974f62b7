"""Seeded inputs in the reference's own file formats, for parity tests.

Writes, for a synthetic imputation problem:
  tags.txt / targets.txt      challenge-format genotype and target files
                              (parsed by eval/idash.cpp:280-312, :315-423)
  model/<pos>_<snp>.hr        discretised models (eval/parse_vw.cpp:8-30)
  params.bin                  eval/idash.cpp:128-186 layout
  encrypted_data.bin          eval/idash.cpp:540-556 layout, records in a
                              shuffled order (uniformly random ciphertexts)

All randomness comes from a splitmix64 counter hash, so the same files are
produced on any machine (numpy only; no reference code is needed to run it).
"""
from __future__ import annotations

import os
import struct

import numpy as np

RECORD_TAG = 42
N = 1024
_M64 = (1 << 64) - 1


def _mix64(z: np.ndarray) -> np.ndarray:
    z = (z + np.uint64(0x9E3779B97F4A7C15)) & np.uint64(_M64)
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def hash64(seed: int, stream: int, idx) -> np.ndarray:
    with np.errstate(over="ignore"):
        key = _mix64(np.uint64(seed & _M64) + _mix64(np.array([stream], dtype=np.uint64)))[0]
        return _mix64(np.asarray(idx, dtype=np.uint64) ^ key)


def hash_u32(seed, stream, idx):
    return (hash64(seed, stream, idx) >> np.uint64(32)).astype(np.uint32)


def make_problem(seed: int, n_indiv: int, n_tags: int, n_targets: int, neighbours, nan_rate: float = 0.05):
    """Positions, genotypes, windows and integer models."""
    p = np.arange(n_tags, dtype=np.uint64)
    tag_pos = (1000 + 37 * p + hash_u32(seed, 1, p) % 30).astype(np.int64)
    t = np.arange(n_targets, dtype=np.uint64)
    span = int(tag_pos[-1] - tag_pos[0])
    tgt = np.sort(tag_pos[0] + 1 + (hash64(seed, 2, t) % np.uint64(max(span - 1, 1))).astype(np.int64))
    # distinct target positions
    for i in range(1, len(tgt)):
        if tgt[i] <= tgt[i - 1]:
            tgt[i] = tgt[i - 1] + 1
    geno = (hash_u32(seed, 3, np.arange(n_tags * n_indiv, dtype=np.uint64)) % 3).astype(np.int8)
    nan = (hash_u32(seed, 4, np.arange(n_tags * n_indiv, dtype=np.uint64)) % 10000) < int(nan_rate * 10000)
    geno[nan] = -1
    geno = geno.reshape(n_tags, n_indiv)
    models = []  # per target: 3 lists of (name, coef)
    for ti in range(n_targets):
        k = neighbours if isinstance(neighbours, int) else neighbours[ti % len(neighbours)]
        order = np.argsort(np.abs(tag_pos - tgt[ti]), kind="stable")[:k]
        per_snp = []
        for v in range(3):
            o = 3 * ti + v
            terms = []
            for q, tp in enumerate(sorted(order)):
                for u in range(3):
                    c = int(hash_u32(seed, 5, o * 3 * 64 + q * 3 + u)) % 16384 - 8192
                    if c != 0:
                        terms.append((f"{tag_pos[tp]}_{u}", c))
            terms.append(("Constant", int(hash_u32(seed, 6, o)) % 16384 - 8192))
            per_snp.append(terms)
        models.append(per_snp)
    return tag_pos, tgt, geno, models


def write_text_inputs(d: str, tag_pos, tgt, geno, models):
    os.makedirs(os.path.join(d, "model"), exist_ok=True)
    with open(os.path.join(d, "tags.txt"), "w") as f:
        for i, pos in enumerate(tag_pos):
            g = " ".join("." if x < 0 else str(int(x)) for x in geno[i])
            f.write(f"22 {pos} {pos + 1} rs{pos} {g}\n")
    with open(os.path.join(d, "targets.txt"), "w") as f:
        for pos in tgt:
            f.write(f"{pos}\n")
    for ti, pos in enumerate(tgt):
        for v in range(3):
            with open(os.path.join(d, "model", f"{pos}_{v}.hr"), "w") as f:
                for name, c in models[ti][v]:
                    f.write(f"{name} {c}\n")


def write_params(path: str, n_indiv: int, tag_pos, tgt):
    R = N // n_indiv
    RS = N // R
    P, T = len(tag_pos), len(tgt)
    with open(path, "wb") as f:
        f.write(struct.pack("<7I", n_indiv, P, T, 3 * P + 1, 3 * T, R, RS))
        for i, pos in enumerate(tag_pos):
            f.write(struct.pack("<Q3I", int(pos), 3 * i, 3 * i + 1, 3 * i + 2))
        for i, pos in enumerate(tgt):
            f.write(struct.pack("<Q", int(pos)) + str(int(pos)).encode() + b"\0")
            f.write(struct.pack("<3I", 3 * i, 3 * i + 1, 3 * i + 2))
    return R, RS


def write_random_ciphertexts(path: str, seed: int, n_rows: int, variance: float = 2.0 ** -50):
    """encrypted_data.bin with uniformly random TRLWE payloads, records in a
    seeded shuffled order."""
    order = np.argsort(hash64(seed, 7, np.arange(n_rows, dtype=np.uint64)), kind="stable")
    rec = np.zeros(n_rows, dtype=[("idx", "<u4"), ("tag", "<i4"), ("coef", "<u4", (2 * N,)), ("var", "<f8")])
    rec["idx"] = order.astype(np.uint32)
    rec["tag"] = RECORD_TAG
    words = hash_u32(seed, 8, np.arange(n_rows * 2 * N, dtype=np.uint64)).reshape(n_rows, 2 * N)
    rec["coef"] = words[order]
    rec["var"] = variance
    with open(path, "wb") as f:
        f.write(struct.pack("<Q", n_rows))
        f.write(rec.tobytes())


def write_random_case(d: str, seed: int, n_indiv: int, n_tags: int, n_targets: int, neighbours) -> None:
    """A complete cloud-step input directory with random ciphertexts."""
    os.makedirs(d, exist_ok=True)
    tag_pos, tgt, geno, models = make_problem(seed, n_indiv, n_tags, n_targets, neighbours)
    write_text_inputs(d, tag_pos, tgt, geno, models)
    R, _ = write_params(os.path.join(d, "params.bin"), n_indiv, tag_pos, tgt)
    write_random_ciphertexts(os.path.join(d, "encrypted_data.bin"), seed, (3 * n_tags + R - 1) // R)


# Medium cases pinned by the SHA-256 of the reference's encrypted_prediction.bin.
HASHED_CASES = {
    "rand_r1_i1000": dict(seed=11, n_indiv=1000, n_tags=300, n_targets=1000, neighbours=5),
    "rand_r4_i250": dict(seed=12, n_indiv=250, n_tags=200, n_targets=600, neighbours=[5, 10, 20, 3]),
    "rand_r10_i100": dict(seed=13, n_indiv=100, n_tags=500, n_targets=2000, neighbours=5),
}
