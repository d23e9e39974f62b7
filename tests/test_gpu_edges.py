"""Edge cases of the TRLWE-packed scoring (eval/idash.cpp:779-842) against
oracle B, bit for bit, through each kernel kind:

- outputs with no terms, or with the constant alone (eval/idash.cpp:805-810);
- extreme and zero coefficients, whose products wrap mod 2^32 as tLweAddMulTo's
  do (eval/idash.cpp:817);
- a feature named twice in one output;
- an output that reads every input feature;
- NUM_SAMPLES 0 and NUM_SAMPLES = REGION_SIZE, and the largest region count
  (REGION_SIZE 1: every feature of a row at its own rotation, :822-836);
- an empty model, which scores nothing and succeeds, as the reference's loop
  over an empty map does."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

gpu = pytest.importorskip("idash2019_2_gb300.gpu")

CONST = 0xFFFFFFFF
I32_MIN, I32_MAX = -2 ** 31, 2 ** 31 - 1
N_FEAT = 40


@pytest.fixture(scope="module")
def ctx():
    c = gpu.Context(0)
    yield c
    c.close()


def edge_model(seed: int) -> "gpu.CSRModel":
    rng = np.random.default_rng(seed)
    lists = [
        [],
        [(CONST, 5)],
        [(CONST, I32_MIN)],
        [(1, I32_MAX), (2, I32_MIN), (3, -1), (4, 0), (5, 1), (CONST, I32_MAX)],
        [(7, 3), (7, -2), (CONST, -3)],
        [(f, int(c)) for f, c in zip(range(N_FEAT), rng.integers(-8192, 8192, N_FEAT))],
    ]
    for _ in range(30):  # ordinary windows of 5 neighbouring features
        lo = int(rng.integers(0, N_FEAT - 5))
        lists.append([(lo + j, int(rng.integers(-8192, 8192))) for j in range(5)] +
                     [(CONST, int(rng.integers(-100, 100)))])
    lists.append([])  # and one more empty output at the end
    ptr = np.zeros(len(lists) + 1, np.uint64)
    ptr[1:] = np.cumsum([len(t) for t in lists])
    feat = np.array([f for t in lists for f, _ in t], np.uint32)
    coef = np.array([c for t in lists for _, c in t], np.int32)
    return gpu.CSRModel(ptr, feat, coef)


def rows_for(regions: int, seed: int) -> np.ndarray:
    n_rows = (N_FEAT + regions - 1) // regions
    rng = np.random.default_rng(seed)
    return rng.integers(0, 2 ** 32, size=(n_rows, 2048), dtype=np.uint64).astype(np.uint32).view(np.int32)


@pytest.mark.parametrize("regions,region_size,num_samples", [(1, 1024, 1000), (1, 1024, 0), (10, 102, 102),
                                                             (1024, 1, 1)])
@pytest.mark.parametrize("kernel", [1, 2, 3, 4])
def test_edge_models_vs_oracle(ctx, oracle, kernel, regions, region_size, num_samples):
    csr = edge_model(11 + regions)
    rows = rows_for(regions, 5 + kernel)
    ctx.set_option("kernel", kernel)
    try:
        m = gpu.TrlweModel(ctx, csr, rows.shape[0], num_samples, regions, region_size)
        got = m.score(rows)
        m.free()
    finally:
        ctx.set_option("kernel", 0)
    want, _ = oracle.trlwe_score(csr.term_ptr, csr.term_feat, csr.term_coef, rows, num_samples, regions,
                                 region_size)
    np.testing.assert_array_equal(got, want)
    # the outputs without terms hold zeros; the constant alone is bias * 2^18 on b[0, NUM_SAMPLES)
    assert not got[0].any() and not got[-1].any()
    assert (got[1, 1024:1024 + num_samples] == 5 << 18).all()
    assert not got[1, :1024].any() and not got[1, 1024 + num_samples:].any()


def test_empty_model_scores_nothing(ctx):
    csr = gpu.CSRModel(np.zeros(1, np.uint64), np.zeros(0, np.uint32), np.zeros(0, np.int32))
    m = gpu.TrlweModel(ctx, csr, 4, 1000, 1, 1024)
    assert m.score(rows_for(10, 1)[:4]).shape == (0, 2048)
    m.free()
