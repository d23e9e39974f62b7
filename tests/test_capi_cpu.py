"""CPU-only checks of the C ABI library: it loads, exports every function the
header declares, reports errors as statuses without a GPU, and its host-side
synthetic model generator follows the reference's conventions."""
import numpy as np
import pytest

_lib = pytest.importorskip("idash2019_2_gb300._lib")


@pytest.fixture(scope="module")
def lib():
    try:
        return _lib.load()
    except ImportError as e:
        pytest.skip(str(e))


def test_library_exports_every_declared_function(lib):
    declared = _lib.declared_functions()
    assert len(declared) >= 25
    for name in declared:
        assert hasattr(lib, name), f"libidash_gpu.so does not export {name}"
        assert name in _lib.PROTOTYPES, f"no ctypes prototype for {name}"
    assert lib.idash_abi_version() == 1


def test_status_strings(lib):
    """Every status the header declares has its own string."""
    strings = [lib.idash_status_string(code) for code in range(len(_lib.STATUS))]
    assert all(strings) and b"unknown status" not in strings
    assert len(set(strings)) == len(strings)


def test_open_without_device_is_a_status(lib):
    import ctypes as C
    h = C.c_void_p()
    code = lib.idash_open(C.byref(h), 999)
    assert code != 0
    assert not h.value
    assert lib.idash_last_error(None)


def test_synth_model_windows_are_nearest_tags():
    from idash2019_2_gb300 import gpu
    w = gpu.synth_model(seed=42, n_tags=200, n_targets=500, choices=[5, 10, 20, 30, 50])
    tags = w.tag_pos.astype(np.int64)
    assert np.all(np.diff(tags) > 0)
    assert np.all(np.diff(w.target_pos.astype(np.int64)) >= 0)
    assert set(np.unique(w.window_len)) <= {5, 10, 20, 30, 50}
    for t in range(0, 500, 37):
        s, k = int(w.window_start[t]), int(w.window_len[t])
        d = np.abs(tags - int(w.target_pos[t]))
        inside = d[s:s + k].max()
        outside = np.concatenate([d[:s], d[s + k:]])
        assert outside.size == 0 or inside <= outside.min()
    csr = w.model
    assert csr.n_out == 1500
    for o in range(0, csr.n_out, 101):
        f = csr.term_feat[csr.term_ptr[o]:csr.term_ptr[o + 1]]
        c = csr.term_coef[csr.term_ptr[o]:csr.term_ptr[o + 1]]
        assert f[-1] == 0xFFFFFFFF
        t = o // 3
        tags_used = set((f[:-1] // 3).tolist())
        assert tags_used <= set(range(int(w.window_start[t]), int(w.window_start[t] + w.window_len[t])))
        assert np.all(c[:-1] != 0) and np.all(c >= -8192) and np.all(c <= 8191)


def test_synth_model_is_deterministic():
    from idash2019_2_gb300 import gpu
    a = gpu.synth_model(seed=5, n_tags=50, n_targets=60, neighbours=5)
    b = gpu.synth_model(seed=5, n_tags=50, n_targets=60, neighbours=5)
    np.testing.assert_array_equal(a.model.term_coef, b.model.term_coef)
    np.testing.assert_array_equal(a.model.term_feat, b.model.term_feat)


def test_synth_model_rejects_bad_spec(lib):
    import ctypes as C
    spec = _lib.SynthSpec()
    spec.n_tags = 0
    m = _lib.SynthModel()
    assert lib.idash_synth_model(C.byref(spec), C.byref(m)) == 1


def _digest(words, index_base):
    """The serving digest restated in numpy (32-bit lanes): words at global
    indices index_base + i, taken by aligned quads Q = index // 4; a quad's
    hash starts at lo(Q) * 0x85EBCA77 + hi(Q) * 0xC2B2AE3D, takes
    h = h * 0x9E3779B1 + w for each of its words present in index order, and
    ends with h ^= h >> 15, h *= 0x2C1B3C6D, h ^= h >> 12; the digest is the
    sum of the quad hashes mod 2^64."""
    idx = np.uint64(index_base) + np.arange(words.size, dtype=np.uint64)
    quad = idx >> np.uint64(2)
    qs, first = np.unique(quad, return_index=True)
    lo = (qs & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    hi = (qs >> np.uint64(32)).astype(np.uint32)
    h = lo * np.uint32(0x85EBCA77) + hi * np.uint32(0xC2B2AE3D)
    ends = np.append(first[1:], words.size)
    for step in range(4):  # the quad's words in index order
        pos = first + step
        live = pos < ends
        h[live] = h[live] * np.uint32(0x9E3779B1) + words[pos[live]]
    h ^= h >> np.uint32(15)
    h *= np.uint32(0x2C1B3C6D)
    h ^= h >> np.uint32(12)
    return int(h.astype(np.uint64).sum(dtype=np.uint64))


@pytest.mark.parametrize("index_base,n", [(0, 1000), (1 << 20, 1000), ((1 << 34) - 6, 1000), (3 << 33, 999),
                                          (7, 13), (5, 2), (0, 1)])
def test_digest_host_restates_the_quad_hash(lib, index_base, n):
    """idash_digest_host (the host restatement the serving tests check the
    device digests against) is the sum mod 2^64 of the quad hashes, with
    partial quads at either end and where the quad index crosses 2^32; and
    the digest of a buffer is the sum of the digests of its pieces when they
    are cut at quad boundaries."""
    import ctypes as C
    words = np.random.default_rng(index_base % 1000 + n).integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
    with np.errstate(over="ignore"):
        want = _digest(words, index_base)
    P = C.POINTER(C.c_uint32)
    got = lib.idash_digest_host(words.ctypes.data_as(P), words.size, index_base)
    assert got == want
    cut = (4 - index_base % 4) % 4 + 4 * (n // 8)
    if 0 < cut < n:
        a, b = np.ascontiguousarray(words[:cut]), np.ascontiguousarray(words[cut:])
        parts = lib.idash_digest_host(a.ctypes.data_as(P), a.size, index_base) + \
            lib.idash_digest_host(b.ctypes.data_as(P), b.size, index_base + cut)
        assert parts % (1 << 64) == got


@pytest.mark.parametrize("spec", [dict(n_tags=200, n_targets=500, neighbours=5),
                                  dict(n_tags=300, n_targets=800, choices=[5, 10, 20, 30, 50]),
                                  dict(n_tags=7, n_targets=40, neighbours=10)])
def test_oracle_restates_the_synthetic_model(oracle, spec):
    """The benchmark's CPU reference arm builds its workload with the oracle's
    generator (no product import): it must be the product's model exactly."""
    from idash2019_2_gb300 import gpu
    choices = spec.get("choices")
    w = gpu.synth_model(seed=0x1DA52019, n_tags=spec["n_tags"], n_targets=spec["n_targets"],
                        neighbours=spec.get("neighbours", 5), choices=choices)
    ptr, feat, coef, ws, wl = oracle.synth_model(0x1DA52019, spec["n_tags"], spec["n_targets"],
                                                 neighbours=spec.get("neighbours", 5), choices=choices)
    np.testing.assert_array_equal(ptr, w.model.term_ptr)
    np.testing.assert_array_equal(feat, w.model.term_feat)
    np.testing.assert_array_equal(coef, w.model.term_coef)
    np.testing.assert_array_equal(ws, w.window_start)
    np.testing.assert_array_equal(wl, w.window_len)
