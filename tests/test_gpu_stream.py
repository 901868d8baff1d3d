"""Host signals (to_map and from_map with numpy arrays or CPU tensors),
streamed through the device in chunks of detector rows or read and written
by the kernels in place: the results equal those of the same call with
device tensors, for pageable and pinned host memory, with chunk sizes that
do and do not divide the detector count."""
import ctypes

import numpy as np
import pytest

from so3g_gb300 import projeng, synth

pytestmark = pytest.mark.gpu
ARCMIN = np.pi / 180 / 60


@pytest.fixture
def small_chunks(monkeypatch):
    # 7 detectors' rows per chunk; every signal is streamed.
    monkeypatch.setattr(projeng, "STREAM_MIN_BYTES", 0)
    monkeypatch.setattr(projeng, "STREAM_CHUNK_BYTES", 7 * 4 * 20000)


def _setup(n_det=40, n_time=20000, weights=True):
    Q, dets, resp, gamma, sig = synth.workload(n_det, n_time, seed=31, radius_deg=0.7)
    p = synth.car_projectionist((300, 360), ARCMIN)
    q = synth.native(p, Q)
    w = np.random.default_rng(2).uniform(0.5, 1.5, n_det).astype(np.float32) if weights else None
    if weights:
        w[3] = 0.0
    return p.get_ProjEng("TQU"), q, dets, resp, sig, w


@pytest.mark.parametrize("policy", ["stream", "direct", "mapped", "auto"])
@pytest.mark.parametrize("host_kind", ["numpy", "torch", "pinned"])
def test_streamed_to_map_and_from_map(small_chunks, monkeypatch, host_kind, policy):
    import torch
    from so3g_gb300 import _abi
    monkeypatch.setenv("SO3G_GB300_HOST_SIGNAL", policy)
    streamed = []
    orig = projeng._stream_rows

    def spy(*a, **k):
        streamed.append(k.get("download", a[3] if len(a) > 3 else None))
        return orig(*a, **k)

    monkeypatch.setattr(projeng, "_stream_rows", spy)
    eng, q, dets, resp, sig, w = _setup()
    dq, dd, dr, ds, dw = (torch.from_numpy(x).cuda() for x in (q, dets, resp, sig, w))
    want_m = eng.to_map(None, dq, dd, dr, ds, dw, None).cpu().numpy()
    sig0 = np.random.default_rng(5).standard_normal(sig.shape).astype(np.float32)
    want_s = eng.from_map(torch.from_numpy(want_m).cuda(), dq, dd, dr,
                          torch.from_numpy(sig0.copy()).cuda()).cpu().numpy()

    def host(a):
        if host_kind == "numpy":
            return a.copy()
        t = torch.from_numpy(a.copy())
        return t.pin_memory() if host_kind == "pinned" else t

    m = np.zeros_like(want_m)
    h = host(sig)
    mode = projeng._host_mode(h if isinstance(h, torch.Tensor) else torch.from_numpy(h))
    eng.to_map(m, q, dets, resp, h, w, None)
    assert np.abs(m - want_m).max() <= 1e-12 * np.abs(want_m).max()
    s = host(sig0)
    ret = eng.from_map(want_m, q, dets, resp, s)
    got = np.asarray(s) if host_kind == "numpy" else s.numpy()
    assert np.array_equal(got.view(np.int32), want_s.view(np.int32))
    if host_kind == "numpy":
        assert all(np.shares_memory(r, s) for r in ret)
    else:
        assert ret is s
    # Which calls streamed (False: to_map, True: from_map).  Page-locked
    # memory is mapped under unified addressing; pageable memory is
    # reachable only where the device accesses it coherently.
    assert mode in ((_abi.HOST_MAPPED,) if host_kind == "pinned"
                    else (_abi.HOST_NONE, _abi.HOST_PAGEABLE))
    direct = {
        "stream": lambda writes: False,
        "direct": lambda writes: mode != _abi.HOST_NONE,
        "mapped": lambda writes: mode == _abi.HOST_MAPPED,
        "auto": lambda writes: mode == _abi.HOST_PAGEABLE and not writes,
    }[policy]
    assert streamed == [w for w in (False, True) if not direct(w)]


def test_host_access_modes():
    import torch
    from so3g_gb300 import _abi
    projeng._ensure_init()
    lib = _abi.lib()

    def mode(ptr):
        m = ctypes.c_int32(-1)
        assert lib.so3g_host_access(ptr, ctypes.byref(m)) == 0
        return m.value

    dev = torch.zeros(16, device="cuda")
    pinned = torch.zeros(16).pin_memory()
    pageable = np.zeros(1 << 20, np.float32)
    assert mode(None) == _abi.HOST_NONE
    assert mode(dev.data_ptr()) == _abi.HOST_NONE
    assert mode(pinned.data_ptr()) == _abi.HOST_MAPPED
    assert mode(pageable.ctypes.data) in (_abi.HOST_NONE, _abi.HOST_PAGEABLE)
    assert lib.so3g_host_access(None, None) == -1


def test_stream_threshold(monkeypatch):
    """Signals below the threshold, lists of rows and thread_intervals go
    through the device whole."""
    monkeypatch.setenv("SO3G_GB300_HOST_SIGNAL", "stream")
    eng, q, dets, resp, sig, w = _setup(n_det=8, n_time=5000)
    calls = []
    orig = projeng._stream_rows

    def spy(*a, **k):
        calls.append(1)
        return orig(*a, **k)

    monkeypatch.setattr(projeng, "_stream_rows", spy)
    eng.to_map(None, q, dets, resp, sig, None, None)
    assert not calls
    monkeypatch.setattr(projeng, "STREAM_MIN_BYTES", 0)
    m1 = eng.to_map(None, q, dets, resp, sig, None, None)
    assert len(calls) == 1
    m2 = eng.to_map(None, q, dets, resp, list(sig), None, None)
    assert len(calls) == 1
    assert np.abs(m1 - m2).max() <= 1e-12 * np.abs(m1).max()


@pytest.mark.parametrize("policy", ["stream", "direct"])
def test_from_map_new_host_signal(small_chunks, monkeypatch, policy):
    """from_map with signal=None and host pointing: a new host signal,
    filled chunk by chunk (or in place), equal to the device result."""
    import torch
    monkeypatch.setenv("SO3G_GB300_HOST_SIGNAL", policy)
    eng, q, dets, resp, sig, w = _setup()
    dq, dd, dr = (torch.from_numpy(x).cuda() for x in (q, dets, resp))
    m = eng.to_map(None, q, dets, resp, sig, None, None)
    want = eng.from_map(torch.from_numpy(m).cuda(), dq, dd, dr, None).cpu().numpy()
    for _ in range(2):
        got = eng.from_map(m, q, dets, resp, None)
        assert isinstance(got, list) and len(got) == len(dets)
        assert all(isinstance(r, np.ndarray) and r.shape == (q.shape[0],) for r in got)
        assert np.array_equal(np.stack(got).view(np.int32), want.view(np.int32))
