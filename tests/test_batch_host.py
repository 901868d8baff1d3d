"""Host side of the batched projection (no GPU): the work plan computed by
so3g_batch_work_offsets, and the tuner's JSON cache."""
import ctypes

import numpy as np
import pytest


@pytest.fixture(scope="module")
def lib():
    import so3g_gb300.build as b
    b.build()
    from so3g_gb300 import _abi
    return _abi.lib()


def _recs(sizes):
    from so3g_gb300 import _abi
    recs = (_abi.Obs * len(sizes))()
    for r, (nd, nt) in zip(recs, sizes):
        r.n_det = nd
        r.n_time = nt
    return recs


@pytest.mark.parametrize("piece", [256, 4096, 8192])
def test_work_offsets(lib, piece):
    from so3g_gb300 import _abi
    rng = np.random.default_rng(3)
    sizes = [(int(rng.integers(0, 2000)), int(rng.integers(0, 2_000_000))) for _ in range(16)]
    sizes[3] = (0, 1000)
    sizes[7] = (12, 0)
    recs = _recs(sizes)
    off = np.full(len(sizes) + 1, -7, dtype=np.int64)
    n = lib.so3g_batch_work_offsets(ctypes.cast(recs, ctypes.POINTER(_abi.Obs)), len(sizes),
                                    piece, off.ctypes.data)
    want = np.concatenate([[0], np.cumsum([nd * -(-nt // piece) for nd, nt in sizes])])
    assert n == want[-1]
    assert np.array_equal(off, want)


def test_work_offsets_bad_args(lib):
    from so3g_gb300 import _abi
    recs = _recs([(1, 1)])
    off = np.zeros(2, dtype=np.int64)
    p = ctypes.cast(recs, ctypes.POINTER(_abi.Obs))
    assert lib.so3g_batch_work_offsets(p, 1, 0, off.ctypes.data) == -1
    assert lib.so3g_batch_work_offsets(p, -1, 256, off.ctypes.data) == -1
    assert lib.so3g_batch_work_offsets(p, 1, 256, None) == -1
    assert lib.so3g_batch_work_offsets(p, 0, 256, off.ctypes.data) == 0


def test_tune_cache_roundtrip(tmp_path, monkeypatch):
    from so3g_gb300 import batch
    path = tmp_path / "sub" / "tune.json"
    monkeypatch.setenv("SO3G_GB300_TUNE_CACHE", str(path))
    assert batch._load_cache() == {}
    batch._store_cache("k1", {"piece": 4096, "blocks": 0})
    batch._store_cache("k2", {"piece": 8192, "blocks": 304})
    assert batch._load_cache() == {"k1": {"piece": 4096, "blocks": 0},
                                   "k2": {"piece": 8192, "blocks": 304}}
    path.write_text("not json")
    assert batch._load_cache() == {}
