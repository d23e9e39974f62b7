"""One scoring batch split across ranks, one process per GPU.

The reference scores a batch in one process (eval/cloud.cpp:3-28, the loop of
eval/idash.cpp:779-842).  The step partitions with no exchange in the data
path, in either of two ways:

  by targets      rank r scores a contiguous range of targets (outputs
                  3*t_lo .. 3*t_hi) and needs only the input rows those
                  outputs read: its own tags plus a halo of at most one
                  neighbourhood on each side;
  by individuals  TRLWE blocks of REGION_SIZE individuals are independent
                  ciphertexts, so rank r takes whole blocks (and the LWE form
                  splits a row's samples the same way), with no halo.

Each rank's outputs are its range's rows in order; concatenating the ranks'
outputs in rank order gives the one-rank bytes.  The host functions here are
plain numpy; score_target_shard runs a rank's part on its GPU.
"""
from __future__ import annotations

import numpy as np

CONSTANT_FEATURE = 0xFFFFFFFF


def even_ranges(n: int, world: int) -> list[tuple[int, int]]:
    """[0, n) as `world` contiguous ranges whose sizes differ by at most one."""
    if world < 1:
        raise ValueError("world must be at least 1")
    q, r = divmod(n, world)
    out, lo = [], 0
    for k in range(world):
        hi = lo + q + (1 if k < r else 0)
        out.append((lo, hi))
        lo = hi
    return out


def target_shard(n_targets: int, world: int, rank: int) -> tuple[int, int]:
    """Rank `rank`'s targets [t_lo, t_hi)."""
    return even_ranges(n_targets, world)[rank]


def block_shard(n_indiv: int, region_size: int, world: int, rank: int) -> tuple[int, int]:
    """Rank `rank`'s TRLWE blocks [b_lo, b_hi) of REGION_SIZE individuals."""
    n_blocks = (n_indiv + region_size - 1) // region_size
    return even_ranges(n_blocks, world)[rank]


def input_row_range(term_ptr, term_feat, out_lo: int, out_hi: int, num_regions: int = 1) -> tuple[int, int]:
    """The input rows [row_lo, row_hi) that outputs [out_lo, out_hi) read
    (feature f is held in row f // num_regions; constant terms read none);
    (0, 0) when they read no row."""
    a, b = int(term_ptr[out_lo]), int(term_ptr[out_hi])
    f = np.asarray(term_feat[a:b], np.uint64)
    f = f[f != CONSTANT_FEATURE]
    if f.size == 0:
        return 0, 0
    rows = f // num_regions
    return int(rows.min()), int(rows.max()) + 1


def shard_model(term_ptr, term_feat, term_coef, out_lo: int, out_hi: int, row_lo: int, num_regions: int = 1):
    """Outputs [out_lo, out_hi) as a model of their own over the input rows
    from row_lo on: (term_ptr, term_feat, term_coef) with every feature
    moved down by row_lo * num_regions (its region is kept)."""
    a, b = int(term_ptr[out_lo]), int(term_ptr[out_hi])
    ptr = (np.asarray(term_ptr[out_lo:out_hi + 1], np.uint64) - np.uint64(a)).astype(np.uint64)
    feat = np.array(term_feat[a:b], np.uint32)
    live = feat != CONSTANT_FEATURE
    feat[live] -= np.uint32(row_lo * num_regions)
    return ptr, feat, np.array(term_coef[a:b], np.int32)


def merge(parts) -> np.ndarray:
    """The ranks' output rows, in rank order, as one array."""
    return np.concatenate([np.asarray(p) for p in parts], axis=0)


def score_target_shard(model, rows: np.ndarray, n_targets: int, world: int, rank: int, num_samples: int):
    """This rank's outputs on its GPU: a TrlweModel of the whole model
    (resident on every rank) scores outputs 3*t_lo .. 3*t_hi from only the
    input rows they read, copied in from `rows` (the batch's dense int32
    [n_rows, 2N] rows on the host).  Returns int32 [outputs, 2N]."""
    from . import gpu
    t_lo, t_hi = target_shard(n_targets, world, rank)
    o_lo, o_hi = 3 * t_lo, 3 * t_hi
    r_lo, r_hi = model.input_rows(o_lo, o_hi)
    ctx, lay = model.ctx, gpu.DENSE_TRLWE
    width = rows.shape[1]
    d_in = ctx.device_alloc(max(r_hi - r_lo, 1) * width * 4)
    d_out = ctx.device_alloc(max(o_hi - o_lo, 1) * width * 4)
    try:
        if r_hi > r_lo:
            d_in.upload(np.ascontiguousarray(rows[r_lo:r_hi], np.int32))
        model.score_range(o_lo, o_hi, num_samples, d_in.ptr, lay, r_lo, r_hi - r_lo, d_out.ptr, lay)
        ctx.sync()
        return d_out.download(nbytes=(o_hi - o_lo) * width * 4, dtype=np.int32).reshape(o_hi - o_lo, width)
    finally:
        d_in.free()
        d_out.free()
