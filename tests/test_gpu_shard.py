"""The split by targets through the GPU path (idash2019_2_gb300/shard.py):
each rank's part scored from only the input rows it reads, one part after
the other on this GPU (the parts are independent: no rank waits on
another), merged in rank order, equals the oracle's one-rank outputs."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

gpu = pytest.importorskip("idash2019_2_gb300.gpu")


@pytest.mark.parametrize("world", [2, 3])
def test_target_shards_merge_to_the_one_rank_outputs(oracle, world):
    from idash2019_2_gb300 import shard
    ctx = gpu.Context(0)
    try:
        w = gpu.synth_model(seed=12, n_tags=300, n_targets=1000, neighbours=5)
        rng = np.random.default_rng(12)
        rows = rng.integers(0, 2 ** 32, size=(900, 2048), dtype=np.uint64).astype(np.uint32).view(np.int32)
        m = gpu.TrlweModel(ctx, w.model, 900, 1000, 1, 1024)
        parts = [shard.score_target_shard(m, rows, 1000, world, r, 1000) for r in range(world)]
        m.free()
    finally:
        ctx.close()
    want, _ = oracle.trlwe_score(w.model.term_ptr, w.model.term_feat, w.model.term_coef, rows, 1000, 1, 1024)
    np.testing.assert_array_equal(shard.merge(parts), want)
