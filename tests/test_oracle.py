"""The oracle against the reference: the C restatement (oracle.c) must agree
bit for bit with the reference's own cloud_compute_score (eval/idash.cpp:763-848)
on the committed fixtures the reference produced, and decrypting the
reference's output must give the plaintext model scores (compute_score,
eval/idash.cpp:888-927) within the encryption noise."""
import hashlib
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, SMALL_CASES


def load_case(oracle, name):
    d = os.path.join(GOLDEN, name)
    params = oracle.read_params(os.path.join(d, "params.bin"))
    model = oracle.read_model(params, os.path.join(d, "model"))
    data = oracle.read_records(os.path.join(d, "encrypted_data.bin"))
    preds = oracle.read_records(os.path.join(d, "encrypted_prediction.bin"))
    return d, params, model, data, preds


def oracle_on_records(oracle, params, model, data, order=None):
    outs, ptr, feat, coef = oracle.model_csr(model, order)
    n_index = int(data["idx"].max()) + 1
    row_of_index = np.full(n_index, 0xFFFFFFFF, np.uint32)
    row_of_index[data["idx"]] = np.arange(len(data), dtype=np.uint32)
    rows = np.ascontiguousarray(data["coef"])
    out, var = oracle.trlwe_score(ptr, feat, coef, rows, params["NUM_SAMPLES"], params["NUM_REGIONS"],
                                  params["REGION_SIZE"], in_var=np.ascontiguousarray(data["var"]),
                                  row_of_index=row_of_index)
    return outs, out, var


@pytest.mark.parametrize("name", SMALL_CASES)
def test_oracle_matches_reference_fixture(oracle, name):
    d, params, model, data, preds = load_case(oracle, name)
    outs, out, var = oracle_on_records(oracle, params, model, data)
    assert len(preds) == len(outs) == params["NUM_OUTPUT_FEATURES"]
    by_idx = {int(r["idx"]): i for i, r in enumerate(preds)}
    for k, o in enumerate(outs):
        ref = preds[by_idx[int(o)]]
        assert ref["tag"] == 42
        np.testing.assert_array_equal(out[k], ref["coef"], err_msg=f"{name}: output {o}")
        if max((abs(c) for f, c in model[int(o)]), default=0) <= 46340:
            # coef^2 * 2^-50 sums are exact in double: any order gives the same bits
            assert var[k] == ref["var"], f"{name}: variance of output {o}"
        else:
            # huge coefficients: the double sum depends on the map's iteration
            # order, which this Python reader does not reproduce
            assert var[k] == pytest.approx(ref["var"], rel=1e-14)


@pytest.mark.parametrize("name", SMALL_CASES)
def test_reference_output_decrypts_to_plaintext_scores(oracle, name):
    """decrypt(cloud(encrypt(x))) ~ compute_score(x): the fixtures are real
    encryptions, and the slots the reference hides are zero."""
    d, params, model, data, preds = load_case(oracle, name)
    key = oracle.read_key(os.path.join(d, "keys.bin"))
    plain = oracle.plaintext_scores(params, model, os.path.join(d, "tags.txt"))
    ns, rs = params["NUM_SAMPLES"], params["REGION_SIZE"]
    for r in preds:
        o = int(r["idx"])
        ph = oracle.torus_to_double(oracle.phase(r["coef"], key))
        coefs = [c for f, c in model[o] if f != oracle.CONST]
        # noise sd 2^-25 * sqrt(sum w^2), 6 sigma, plus NaN one-hot truncation
        bound = 6 * 2.0 ** -25 * np.sqrt(1 + sum(float(c) ** 2 for c in coefs)) + \
            sum(abs(float(c)) for c in coefs) * 2.0 ** -32 + 1e-12
        if all(abs(c) <= 8192 for f, c in model[o]):
            # scores live on the torus: compare modulo 1
            diff = (ph[:ns] - plain[o] + 0.5) % 1.0 - 0.5
            assert np.max(np.abs(diff)) <= bound, f"{name}: output {o} off by {np.max(np.abs(diff))}"
        assert np.all(r["coef"][1024 + rs:] == 0), "hidden slots must be zero (eval/idash.cpp:839-841)"


@pytest.mark.parametrize("name", SMALL_CASES)
def test_decrypted_csv_matches_fixture(oracle, name):
    """The reference's own decrypt output (result_bypos.csv) is the phase of
    its prediction records (eval/idash.cpp:714-719, :455-465)."""
    d, params, model, data, preds = load_case(oracle, name)
    key = oracle.read_key(os.path.join(d, "keys.bin"))
    lines = open(os.path.join(d, "result_bypos.csv")).read().splitlines()[1:]
    by_idx = {int(r["idx"]): r for r in preds}
    for ln in lines[:50]:
        s, pos, *vals = ln.split(",")
        bidx = params["out"][int(pos)]
        for v in range(3):
            ph = oracle.torus_to_double(oracle.phase(by_idx[bidx[v]]["coef"], key))[int(s)]
            assert abs(np.float32(ph) - float(vals[v])) <= 1e-5 * max(1.0, abs(float(vals[v])))


def oracle_csv(oracle, d, params, preds, by_position=True):
    """The reference's CSV (write_decrypted_predictions, eval/idash.cpp:436-469)
    rebuilt from the oracle's decryption: sample-major lines, positions in
    params order, each float as printf("%.6g") (what an ostream prints)."""
    key = oracle.read_key(os.path.join(d, "keys.bin"))
    ns = params["NUM_SAMPLES"]
    scores = oracle.trlwe_decrypt(np.ascontiguousarray(preds["coef"]), key, ns)
    row = {int(r["idx"]): i for i, r in enumerate(preds)}
    out = ["Subject ID,target SNP,0,1,2"]
    for s in range(ns):
        for pos, name in params["out_names"]:
            b = params["out"][pos]
            vals = ",".join("%.6g" % float(scores[row[b[g]], s]) for g in range(3))
            out.append(f"{s},{pos if by_position else name},{vals}")
    return "\n".join(out) + "\n"


@pytest.mark.parametrize("name", SMALL_CASES)
def test_oracle_decrypt_reproduces_reference_csv(oracle, name):
    """The oracle's decryption (oracle_trlwe_decrypt) formatted as the
    reference formats it equals the reference decrypt's CSV byte for byte."""
    d, params, model, data, preds = load_case(oracle, name)
    assert oracle_csv(oracle, d, params, preds, True) == open(os.path.join(d, "result_bypos.csv")).read()
    assert oracle_csv(oracle, d, params, preds, False) == open(os.path.join(d, "result.csv")).read()


REF_BIN = os.path.join(ROOT, "oracle", "_ref", "cloud")


@pytest.mark.skipif(not os.path.exists(REF_BIN), reason="reference build (oracle/_ref) not present")
@pytest.mark.parametrize("name", ["rand_r1_i1000", "rand_r4_i250", "rand_r10_i100"])
def test_oracle_matches_reference_binary_medium(oracle, tmp_path, name):
    import gen_inputs
    meta = json.load(open(os.path.join(GOLDEN, "hashes.json")))[name]
    kw = {k: meta[k] for k in ("seed", "n_indiv", "n_tags", "n_targets", "neighbours")}
    gen_inputs.write_random_case(str(tmp_path), **kw)
    subprocess.run([REF_BIN, "model"], cwd=tmp_path, check=True, capture_output=True)
    raw = open(tmp_path / "encrypted_prediction.bin", "rb").read()
    assert hashlib.sha256(raw).hexdigest() == meta["sha256"]
    params = oracle.read_params(str(tmp_path / "params.bin"))
    model = oracle.read_model(params, str(tmp_path / "model"))
    data = oracle.read_records(str(tmp_path / "encrypted_data.bin"))
    preds = oracle.read_records(str(tmp_path / "encrypted_prediction.bin"))
    outs, out, var = oracle_on_records(oracle, params, model, data)
    by_idx = {int(r["idx"]): i for i, r in enumerate(preds)}
    sel = np.array([by_idx[int(o)] for o in outs])
    np.testing.assert_array_equal(out, np.ascontiguousarray(preds["coef"][sel]))
    np.testing.assert_array_equal(var, preds["var"][sel])
