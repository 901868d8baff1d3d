"""Batched projection: many observations of uneven size into one map by
one persistent launch (so3g_proj_to_map_batch / to_weight_map_batch),
against the oracle's per-observation to_map calls and against one GPU
to_map call per observation; CUDA-graph replay; the autotuner and its
cache; empty observations, detector weights, missing tiles and bad
plans."""
import json

import numpy as np
import pytest

from so3g_gb300 import _abi
from so3g_gb300.batch import Observation, ObservationBatch
from helpers import Case, native_inputs, oracle_map, stack_map

pytestmark = pytest.mark.gpu

SIZES = [(7, 3000), (3, 12000), (0, 500), (11, 800), (5, 0), (2, 7001)]


def _observations(coord, seed=30, sizes=SIZES, weights=True):
    rng = np.random.default_rng(seed)
    obs = []
    for i, (nd, nt) in enumerate(sizes):
        if nd == 0 or nt == 0:
            bore = np.zeros((nt, 4))
            bore[:, 0] = 1
            dets = np.zeros((nd, 4))
            dets[:, 0] = 1
            resp = np.ones((nd, 2), np.float32)
        else:
            bore, dets, resp = native_inputs(coord, nd, nt, seed + i)
        sig = rng.standard_normal((nd, nt)).astype(np.float32)
        w = None
        if weights and i % 2 == 0:
            w = rng.uniform(0.5, 2.0, nd).astype(np.float32)
            if nd > 2:
                w[1] = 0.0
        obs.append(Observation(bore, dets, resp, sig, w))
    return obs


def _case(orc, coord, tiled=False, bilinear=False, hp=None, active=None):
    return Case(orc, coord=coord, ncomp=3, tiled=tiled, bilinear=bilinear, n_det=4,
                n_time=3000, seed=30, hp=hp, active=active)


def _sequential(eng, obs, lead, blank, weight):
    m = blank(lead)
    for ob in obs:
        if ob.dets.shape[0] == 0 or ob.boresight.shape[0] == 0:
            continue
        if weight:
            eng.to_weight_map(m, ob.boresight, ob.dets, ob.response, ob.det_weights, None)
        else:
            eng.to_map(m, ob.boresight, ob.dets, ob.response, ob.signal, ob.det_weights, None)
    return m


CASES = [
    ("CAR", False, False, None),
    ("CAR", True, False, None),
    ("ZEA", False, True, None),
    ("TAN", True, True, None),
    ("CAR", False, False, (64, False, None)),
    ("CAR", True, False, (64, True, 4)),
]


@pytest.mark.parametrize("coord,tiled,bilinear,hp", CASES)
@pytest.mark.parametrize("piece", [256, 2048])
def test_batch_matches_oracle(orc, gpulib, coord, tiled, bilinear, hp, piece):
    c = _case(orc, coord, tiled, bilinear, hp)
    obs = _observations(coord)
    b = ObservationBatch(c.eng, obs)
    assert b.n_samples == sum(nd * nt for nd, nt in SIZES)
    for weight in (False, True):
        lead = (3, 3) if weight else (3,)
        want = c.blank(lead)
        flat, offs = oracle_map(want)
        for ob in obs:
            if ob.dets.shape[0] == 0 or ob.boresight.shape[0] == 0:
                continue
            if weight:
                orc.to_weight_map(c.pz, ob.boresight, ob.dets, ob.response, ob.det_weights,
                                  flat, offs)
            else:
                orc.to_map(c.pz, ob.boresight, ob.dets, ob.response, ob.signal,
                           ob.det_weights, flat, offs)
        m = c.blank(lead)
        got = (b.to_weight_map(m, piece=piece) if weight else b.to_map(m, piece=piece))
        assert got is m
        scale = max(np.abs(flat).max(), 1.0)
        # Certified bilinear weights are within one float32 ulp.
        rtol = 1e-6 if bilinear else 1e-12
        assert np.abs(stack_map(m) - flat).max() <= rtol * scale
        seq = _sequential(c.eng, obs, lead, c.blank, weight)
        assert np.abs(stack_map(seq) - stack_map(m)).max() <= 1e-12 * scale


@pytest.mark.parametrize("blocks", [1, 3, 0, 4096, -1, -2])
def test_batch_grid_sizes(orc, gpulib, blocks):
    """Any grid size covers every work item exactly once."""
    c = _case(orc, "CAR")
    obs = _observations("CAR")
    b = ObservationBatch(c.eng, obs)
    ref = b.to_weight_map(c.blank((3, 3)), piece=512, blocks=0)
    got = b.to_weight_map(c.blank((3, 3)), piece=512, blocks=blocks)
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()


def test_batch_device_tensors_and_graph(orc, gpulib):
    import torch
    c = _case(orc, "CAR")
    obs = _observations("CAR")
    dobs = [Observation(*(None if a is None else torch.from_numpy(np.ascontiguousarray(a)).cuda()
                          for a in (o.boresight, o.dets, o.response, o.signal, o.det_weights)))
            for o in obs]
    b = ObservationBatch(c.eng, dobs)
    m1 = b.to_map(None)
    w1 = b.to_weight_map(None)
    assert m1.is_cuda and w1.is_cuda
    want = _sequential(c.eng, obs, (3,), c.blank, False)
    scale = np.abs(want).max()
    assert np.abs(m1.cpu().numpy() - want).max() <= 1e-12 * scale
    m = torch.zeros_like(m1)
    w = torch.zeros_like(w1)
    g = b.graph(m, w)
    assert g.launches == 2
    # The per-observation strategy in a graph gives the same sums.
    m2 = torch.zeros_like(m1)
    w2 = torch.zeros_like(w1)
    g2 = b.graph(m2, w2, map_shape=(8192, -2), weight_shape=(8192, -2))
    g2.replay()
    torch.cuda.synchronize()
    assert float((m2 - m1).abs().max()) <= 1e-12 * scale
    assert float((w2 - w1).abs().max()) <= 1e-12 * float(w1.abs().max())
    for _ in range(3):
        g.replay()
    torch.cuda.synchronize()
    g.check()
    assert float((m - 3 * m1).abs().max()) <= 1e-11 * scale
    assert float((w - 3 * w1).abs().max()) <= 1e-11 * float(w1.abs().max())


def test_graph_needs_device_maps(orc, gpulib):
    c = _case(orc, "CAR")
    b = ObservationBatch(c.eng, _observations("CAR"))
    with pytest.raises(TypeError):
        b.graph(c.blank((3,)))


def test_tuner_and_cache(orc, gpulib, tmp_path, monkeypatch):
    cache = tmp_path / "tune.json"
    monkeypatch.setenv("SO3G_GB300_TUNE_CACHE", str(cache))
    c = _case(orc, "CAR")
    obs = _observations("CAR")
    b = ObservationBatch(c.eng, obs)
    assert b.tuned() is None
    piece, blocks = b.tune(pieces=(256, 1024), blocks_per_sm=(0, 2), reps=1)
    assert (piece, blocks) in [(r["piece"], r["blocks"]) for r in b.tune_log]
    assert len(b.tune_log) == 5
    assert b.tuned() == (piece, blocks)
    d = json.loads(cache.read_text())
    assert len(d) == 1
    # Tuning writes nothing into the caller's maps; the tuned shape is used
    # by default and gives the same map.
    m = b.to_map(c.blank((3,)))
    want = _sequential(c.eng, obs, (3,), c.blank, False)
    assert np.abs(m - want).max() <= 1e-12 * np.abs(want).max()
    assert b.tuned(weight=True) is None


def test_missing_tile_raises(orc, gpulib):
    c = _case(orc, "CAR", tiled=True)
    obs = _observations("CAR")
    b = ObservationBatch(c.eng, obs)
    m = c.blank((3,), populate=[0, 1])
    with pytest.raises(RuntimeError, match="non-instantiated tile"):
        b.to_map(m)


def test_bad_arguments(orc, gpulib):
    c = _case(orc, "CAR")
    obs = _observations("CAR")
    b = ObservationBatch(c.eng, obs)
    with pytest.raises(ValueError, match="multiple of 256"):
        b.to_map(c.blank((3,)), piece=1000)
    nosig = [Observation(o.boresight, o.dets, o.response) for o in obs]
    b2 = ObservationBatch(c.eng, nosig)
    with pytest.raises(ValueError, match="signal"):
        b2.to_map(c.blank((3,)))
    w = b2.to_weight_map(c.blank((3, 3)))
    assert np.abs(w).max() > 0
    bad = obs[0]
    with pytest.raises(RuntimeError, match="incompatible shape"):
        ObservationBatch(c.eng, [Observation(bad.boresight, bad.dets, bad.response,
                                             bad.signal[:, :-1])])
    with pytest.raises(ValueError, match="float32"):
        ObservationBatch(c.eng, [Observation(bad.boresight, bad.dets, bad.response,
                                             bad.signal.astype(np.float64))])
    e = ObservationBatch(c.eng, [])
    m = c.blank((3,))
    e.to_map(m)
    assert not m.any()
