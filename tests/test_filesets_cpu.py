"""The synthetic file sets that bench.py's `files` section writes parse with
the oracle's readers of the reference's formats (params.bin, model/*.hr,
encrypted_data.bin), with the counts and neighbourhoods they claim."""
import os

import numpy as np

from idash2019_2_gb300 import filesets


def test_fileset_round_trip(tmp_path, oracle):
    info = filesets.write_cloud_inputs(str(tmp_path), seed=5, n_indiv=1000, n_tags=40, n_targets=25, neighbours=5)
    p = oracle.read_params(str(tmp_path / "params.bin"))
    assert (p["NUM_SAMPLES"], p["NUM_INPUT_POSITIONS"], p["NUM_OUTPUT_POSITIONS"]) == (1000, 40, 25)
    assert (p["NUM_INPUT_FEATURES"], p["NUM_OUTPUT_FEATURES"], p["NUM_REGIONS"]) == (121, 75, 1)
    model = oracle.read_model(p, str(tmp_path / "model"))
    assert len(model) == info["outputs"] == 75
    assert sum(len(t) for t in model.values()) == info["terms"]
    for terms in model.values():  # [(FeatBigIndex, coef)], "Constant" as 0xFFFFFFFF
        feats = [f for f, _ in terms if f != 0xFFFFFFFF]
        assert len(feats) == 15 and len(terms) == 16  # 5 neighbours x 3 genotypes + Constant
        tags = sorted({f // 3 for f in feats})
        assert len(tags) == 5 and tags[-1] - tags[0] <= 9  # the nearest tags are contiguous or nearly so
        assert all(-8192 <= c < 8192 and c != 0 for f, c in terms if f != 0xFFFFFFFF)
    rec = oracle.read_records(str(tmp_path / "encrypted_data.bin"))
    assert len(rec) == info["in_records"] == 120
    np.testing.assert_array_equal(rec["idx"], np.arange(120))
    assert (rec["tag"] == 42).all()
    assert os.path.getsize(tmp_path / "encrypted_data.bin") == 8 + 120 * 8208
