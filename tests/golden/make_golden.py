"""Regenerates the golden fixtures from the reference's own pipeline.

Needs the reference sources (REF_DIR, else "reference" beside the repository) and builds
them with `make -C oracle ref` (the reference's eval/*.cpp compiled against
oracle/tfhe_compat).  Run from the repository root:

    python tests/golden/make_golden.py

Small cases (committed under tests/golden/<case>/) run the full reference
chain keygen -> encrypt -> cloud -> decrypt on seeded challenge-format
inputs; the reference's encrypted_prediction.bin is the golden output.
Medium cases (tests/golden/hashes.json) run the reference's cloud on seeded
random ciphertexts from gen_inputs.py and keep the SHA-256 of its output.
"""
from __future__ import annotations

import hashlib
import json
import os
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
import gen_inputs  # noqa: E402

REF_BIN = os.path.join(ROOT, "oracle", "_ref")

# name -> (n_indiv, n_tags, n_targets, neighbours, nan_rate, edits)
SMALL_CASES = {
    "ref_r10": (100, 30, 8, 5, 0.05, False),
    "ref_r1": (600, 8, 4, 5, 0.05, False),
    "ref_r3_edge": (300, 16, 6, [5, 2, 8, 1, 16, 3], 0.30, True),
}


def run(cmd, cwd, env=None):
    r = subprocess.run(cmd, cwd=cwd, env=env, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"{cmd} failed:\n{r.stdout}\n{r.stderr}")
    return r.stdout


def edit_models(d, tgt):
    """Edge cases the reference's loader and scorer accept:
    a constant-only model, a repeated feature line (later value wins,
    eval/parse_vw.cpp:24), and coefficients far outside [-8192, 8191]
    whose products wrap mod 2^32."""
    m = os.path.join(d, "model")
    with open(os.path.join(m, f"{tgt[0]}_0.hr"), "w") as f:
        f.write("Constant 1234\n")
    p = os.path.join(m, f"{tgt[1]}_1.hr")
    lines = open(p).read().splitlines()
    first = lines[0].split()[0]
    lines.append(f"{first} -4321")
    open(p, "w").write("\n".join(lines) + "\n")
    p = os.path.join(m, f"{tgt[2]}_2.hr")
    lines = open(p).read().splitlines()
    name0, name1 = lines[0].split()[0], lines[1].split()[0]
    lines[0] = f"{name0} 2000000000"
    lines[1] = f"{name1} -2147483647"
    lines[-1] = "Constant 99999"
    open(p, "w").write("\n".join(lines) + "\n")


def make_small(name, n_indiv, n_tags, n_targets, neighbours, nan_rate, edits, seed):
    out = os.path.join(HERE, name)
    with tempfile.TemporaryDirectory() as d:
        tag_pos, tgt, geno, models = gen_inputs.make_problem(seed, n_indiv, n_tags, n_targets, neighbours, nan_rate)
        gen_inputs.write_text_inputs(d, tag_pos, tgt, geno, models)
        if edits:
            edit_models(d, tgt)
        env = dict(os.environ, TFHE_COMPAT_SEED=str(seed))
        run([os.path.join(REF_BIN, "keygen"), "targets.txt", "tags.txt", "1"], d, env)
        run([os.path.join(REF_BIN, "encrypt"), "tags.txt"], d, env)
        run([os.path.join(REF_BIN, "cloud1"), "model"], d, env)
        run([os.path.join(REF_BIN, "decrypt"), "bypos"], d, env)
        run([os.path.join(REF_BIN, "decrypt")], d, env)
        if os.path.exists(out):
            shutil.rmtree(out)
        os.makedirs(out)
        for f in ["params.bin", "keys.bin", "encrypted_data.bin", "encrypted_prediction.bin", "result_bypos.csv",
                  "result.csv", "tags.txt", "targets.txt"]:
            shutil.copy(os.path.join(d, f), os.path.join(out, f))
        shutil.copytree(os.path.join(d, "model"), os.path.join(out, "model"))
    print(f"{name}: {sorted(os.listdir(out))}")


def add_named_csv(name):
    """The reference's decrypt without arguments (result.csv, target SNPs by
    name) on a committed case's keys and predictions."""
    out = os.path.join(HERE, name)
    with tempfile.TemporaryDirectory() as d:
        for f in ["keys.bin", "encrypted_prediction.bin"]:
            shutil.copy(os.path.join(out, f), os.path.join(d, f))
        run([os.path.join(REF_BIN, "decrypt")], d)
        shutil.copy(os.path.join(d, "result.csv"), os.path.join(out, "result.csv"))
    print(f"{name}: result.csv")


def make_hashed():
    hashes = {}
    for name, kw in gen_inputs.HASHED_CASES.items():
        with tempfile.TemporaryDirectory() as d:
            gen_inputs.write_random_case(d, **kw)
            run([os.path.join(REF_BIN, "cloud"), "model"], d)
            data = open(os.path.join(d, "encrypted_prediction.bin"), "rb").read()
            hashes[name] = {"sha256": hashlib.sha256(data).hexdigest(), "bytes": len(data), **kw}
            print(name, hashes[name]["sha256"], len(data))
    with open(os.path.join(HERE, "hashes.json"), "w") as f:
        json.dump(hashes, f, indent=1)


def main():
    ref = os.environ.get("REF_DIR") or os.path.join(os.path.dirname(ROOT), "reference")
    run(["make", "-s", "ref", f"REF_DIR={ref}"], os.path.join(ROOT, "oracle"))
    if "--named-csv" in sys.argv:  # only add result.csv to the committed cases
        for name in SMALL_CASES:
            add_named_csv(name)
        return
    for i, (name, args) in enumerate(SMALL_CASES.items()):
        make_small(name, *args, seed=100 + i)
    make_hashed()


if __name__ == "__main__":
    main()
