"""One batch split across two gloo ranks on CPU (idash2019_2_gb300/shard.py),
the oracle standing in for each rank's GPU: every rank scores its part from
only the input rows it needs, rank 0 gathers the parts, and the merged
outputs equal the one-rank outputs byte for byte.  Covers the split by
targets (a halo of input rows at the range edges, TRLWE with NUM_REGIONS 1
and 10, the LWE form) and the split by individuals (whole TRLWE blocks, and
LWE samples).  Not run on GPUs: one GPU is available."""
import os
import socket
import sys

import numpy as np
import pytest

from conftest import ROOT

torch = pytest.importorskip("torch")

SEED, TAGS, TARGETS = 5, 60, 211


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _model():
    import pyoracle
    ptr, feat, coef, _, _ = pyoracle.synth_model(SEED, TAGS, TARGETS, choices=[1, 5, 12])
    return ptr, feat, coef


def _rows(n_rows, width, seed=3):
    rng = np.random.default_rng(seed)
    return rng.integers(0, 2 ** 32, size=(n_rows, width), dtype=np.uint64).astype(np.uint32).view(np.int32)


def _trlwe_whole(regions):
    import pyoracle
    ptr, feat, coef = _model()
    rs = 1024 // regions
    rows = _rows((3 * TAGS + regions - 1) // regions, 2048)
    return pyoracle.trlwe_score(ptr, feat, coef, rows, min(rs, 1000) - (1 if regions > 1 else 0), regions, rs)[0]


def _part_trlwe_targets(world, rank, regions):
    import pyoracle
    from idash2019_2_gb300 import shard
    ptr, feat, coef = _model()
    rs = 1024 // regions
    ns = min(rs, 1000) - (1 if regions > 1 else 0)
    rows = _rows((3 * TAGS + regions - 1) // regions, 2048)
    t_lo, t_hi = shard.target_shard(TARGETS, world, rank)
    o_lo, o_hi = 3 * t_lo, 3 * t_hi
    r_lo, r_hi = shard.input_row_range(ptr, feat, o_lo, o_hi, regions)
    assert r_hi - r_lo < rows.shape[0]  # a strict part of the rows: the split needs only its halo
    p, f, c = shard.shard_model(ptr, feat, coef, o_lo, o_hi, r_lo, regions)
    return pyoracle.trlwe_score(p, f, c, rows[r_lo:r_hi], ns, regions, rs)[0]


def _lwe_inputs(n_indiv):
    ptr, feat, coef = _model()
    width = (n_indiv * 1025 + 3) // 4 * 4
    return ptr, feat, coef, _rows(3 * TAGS, width, seed=4)


def _part_lwe_targets(world, rank, n_indiv):
    import pyoracle
    from idash2019_2_gb300 import shard
    ptr, feat, coef, rows = _lwe_inputs(n_indiv)
    t_lo, t_hi = shard.target_shard(TARGETS, world, rank)
    r_lo, r_hi = shard.input_row_range(ptr, feat, 3 * t_lo, 3 * t_hi)
    p, f, c = shard.shard_model(ptr, feat, coef, 3 * t_lo, 3 * t_hi, r_lo)
    return pyoracle.lwe_score(p, f, c, rows[r_lo:r_hi], n_indiv, 0, 3 * (t_hi - t_lo))


def _part_lwe_individuals(world, rank, n_indiv):
    """Individuals [i_lo, i_hi): their samples' columns of every row."""
    import pyoracle
    from idash2019_2_gb300 import shard
    ptr, feat, coef, rows = _lwe_inputs(n_indiv)
    i_lo, i_hi = shard.even_ranges(n_indiv, world)[rank]
    cols = rows[:, i_lo * 1025:i_hi * 1025]
    return pyoracle.lwe_score(ptr, feat, coef, cols, i_hi - i_lo, 0, len(ptr) - 1)


def _rank_main(rank, world, port, out_dir, kind, arg):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    part = {"trlwe_targets": _part_trlwe_targets, "lwe_targets": _part_lwe_targets,
            "lwe_individuals": _part_lwe_individuals}[kind](world, rank, arg)
    parts = [None] * world if rank == 0 else None
    dist.gather_object(part, parts, dst=0)
    dist.barrier()
    dist.destroy_process_group()
    if rank == 0:
        np.save(os.path.join(out_dir, "merged.npy"),
                np.concatenate(parts, axis=1) if kind == "lwe_individuals" else np.concatenate(parts, axis=0))


def _run(tmp_path, kind, arg, world=2):
    import torch.multiprocessing as mp
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path), kind, arg), nprocs=world,
                       start_method="spawn")
    return np.load(tmp_path / "merged.npy")


@pytest.mark.parametrize("regions", [1, 10])
def test_trlwe_split_by_targets_equals_one_rank(tmp_path, regions):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    merged = _run(tmp_path, "trlwe_targets", regions)
    np.testing.assert_array_equal(merged, _trlwe_whole(regions))


def test_lwe_split_by_targets_equals_one_rank(tmp_path):
    import pyoracle
    merged = _run(tmp_path, "lwe_targets", 3)
    ptr, feat, coef, rows = _lwe_inputs(3)
    np.testing.assert_array_equal(merged, pyoracle.lwe_score(ptr, feat, coef, rows, 3, 0, len(ptr) - 1))


def test_lwe_split_by_individuals_equals_one_rank(tmp_path):
    import pyoracle
    merged = _run(tmp_path, "lwe_individuals", 5)
    ptr, feat, coef, rows = _lwe_inputs(5)
    whole = pyoracle.lwe_score(ptr, feat, coef, rows, 5, 0, len(ptr) - 1)
    np.testing.assert_array_equal(merged, whole[:, :5 * 1025])


def test_ranges_cover_everything_once():
    from idash2019_2_gb300 import shard
    for n, world in [(0, 2), (1, 3), (7, 2), (80882, 8), (5, 5)]:
        rs = shard.even_ranges(n, world)
        assert len(rs) == world and rs[0][0] == 0 and rs[-1][1] == n
        assert all(a[1] == b[0] for a, b in zip(rs, rs[1:]))
        assert max(h - l for l, h in rs) - min(h - l for l, h in rs) <= 1
    # whole blocks of 1,024 individuals
    assert [shard.block_shard(2000, 1024, 2, r) for r in range(2)] == [(0, 1), (1, 2)]
    assert [shard.block_shard(5000, 1024, 2, r) for r in range(2)] == [(0, 3), (3, 5)]
