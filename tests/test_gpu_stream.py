"""Host signals streamed through the device in chunks of detector rows
(to_map and from_map with numpy arrays or CPU tensors): the results equal
those of the same call with device tensors, for pageable and pinned host
memory, with chunk sizes that do and do not divide the detector count."""
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


@pytest.mark.parametrize("host_kind", ["numpy", "torch", "pinned"])
def test_streamed_to_map_and_from_map(small_chunks, host_kind):
    import torch
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
    eng.to_map(m, q, dets, resp, host(sig), w, None)
    assert np.abs(m - want_m).max() <= 1e-12 * np.abs(want_m).max()
    s = host(sig0)
    ret = eng.from_map(want_m, q, dets, resp, s)
    got = np.asarray(s) if host_kind == "numpy" else s.numpy()
    assert np.array_equal(got.view(np.int32), want_s.view(np.int32))
    if host_kind == "numpy":
        assert all(np.shares_memory(r, s) for r in ret)
    else:
        assert ret is s


def test_stream_threshold(monkeypatch):
    """Signals below the threshold, lists of rows and thread_intervals go
    through the device whole."""
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
