"""The differentiable from_map: its backward is the hand-written to_map
adjoint.  Checks the adjoint dot-product identity <P m, d> = <m, P^T d>,
central finite differences on random pixels, and that the gradient equals
to_map of the incoming signal gradient (ZEA bilinear, SpinTQU, as the
differentiable-from_map workload; and CAR nearest)."""
import numpy as np
import pytest

from so3g_gb300 import synth, autograd
from so3g_gb300.proj import SimpleWCS, Projectionist

pytestmark = pytest.mark.gpu
ARCMIN = np.pi / 180 / 60


def _setup(proj, interpol, n_det=16, n_time=20000, shape=(200, 240)):
    import torch
    Q, dets, resp, gamma, _ = synth.workload(n_det, n_time, seed=21, radius_deg=0.5,
                                             throw=2.)
    ny, nx = shape
    r = 2 * ARCMIN * 180 / np.pi
    w = SimpleWCS(proj, (-180., 50.), (-r, r), (nx / 2 + 0.5, ny / 2 + 0.5))
    p = Projectionist.for_geom((ny, nx), w, interpol=interpol)
    q = synth.native(p, Q)
    eng = p.get_ProjEng("TQU")
    t = [torch.from_numpy(x).cuda() for x in (q, dets, resp)]
    rng = np.random.default_rng(4)
    m = torch.from_numpy(rng.standard_normal((3, ny, nx))).cuda()
    d = torch.from_numpy(rng.standard_normal((n_det, n_time)).astype(np.float32)).cuda()
    return eng, t, m, d


@pytest.mark.parametrize("proj,interpol", [("ZEA", "bilinear"), ("CAR", "nearest")])
def test_adjoint_identity(proj, interpol):
    import torch
    eng, (q, dets, resp), m, d = _setup(proj, interpol)
    Pm = autograd.from_map(eng, m, q, dets, resp)
    PTd = torch.zeros_like(m)
    eng.to_map(PTd, q, dets, resp, d, None, None)
    lhs = float((Pm.double() * d.double()).sum())
    rhs = float((m * PTd).sum())
    scale = float((Pm.double().abs() * d.double().abs()).sum())
    assert abs(lhs - rhs) <= 1e-6 * scale


@pytest.mark.parametrize("proj,interpol", [("ZEA", "bilinear"), ("CAR", "nearest")])
def test_backward_is_to_map(proj, interpol):
    import torch
    eng, (q, dets, resp), m, d = _setup(proj, interpol)
    mm = m.clone().requires_grad_(True)
    sig = autograd.from_map(eng, mm, q, dets, resp)
    (sig * d).sum().backward()
    want = torch.zeros_like(m)
    eng.to_map(want, q, dets, resp, d, None, None)
    g = mm.grad
    assert torch.allclose(g, want, rtol=1e-12, atol=1e-12 * float(want.abs().max()))


def test_finite_differences():
    """Central differences of L(m) = <d, P m> on 1000 random pixels
    against the autograd gradient.  L is linear in m, so the difference
    quotient equals the gradient up to float32 rounding of P m."""
    import torch
    eng, (q, dets, resp), m, d = _setup("ZEA", "bilinear", n_det=8, n_time=10000,
                                          shape=(120, 150))
    mm = m.clone().requires_grad_(True)
    (autograd.from_map(eng, mm, q, dets, resp).double() * d.double()).sum().backward()
    grad = mm.grad.cpu().numpy()
    rng = np.random.default_rng(8)
    flat = rng.choice(m.numel(), 1000, replace=False)
    h = 1.0
    errs = []
    mp = m.clone()
    dd = d.double()
    for one in zip(*np.unravel_index(flat, m.shape)):
        mp[one] += h
        lp = float((autograd.from_map(eng, mp, q, dets, resp).double() * dd).sum())
        mp[one] -= 2 * h
        lm = float((autograd.from_map(eng, mp, q, dets, resp).double() * dd).sum())
        mp[one] += h
        errs.append(((lp - lm) / (2 * h), grad[one]))
    fd, g = np.array(errs).T
    assert np.any(g != 0)
    assert np.all(np.abs(fd - g) <= 1e-3 * np.maximum(1.0, np.abs(g)))


def test_backward_uses_the_forward_pointing_mode():
    """The pointing mode is pinned at forward: a caller that switches
    eng.pointing before backward still gets to_map in the forward's mode
    (mixed here), and its own setting back afterwards."""
    import torch
    from so3g_gb300 import _abi
    eng, (q, dets, resp), m, d = _setup("CAR", "nearest")
    eng.pointing = _abi.POINTING_MIXED
    mm = m.clone().requires_grad_(True)
    sig = autograd.from_map(eng, mm, q, dets, resp)
    eng.pointing = _abi.POINTING_EXACT
    (sig * d).sum().backward()
    assert eng.pointing == _abi.POINTING_EXACT
    eng.pointing = _abi.POINTING_MIXED
    want = torch.zeros_like(m)
    eng.to_map(want, q, dets, resp, d, None, None)
    eng.pointing = _abi.POINTING_EXACT
    exact = torch.zeros_like(m)
    eng.to_map(exact, q, dets, resp, d, None, None)
    scale = float(want.abs().max())
    assert float((mm.grad - want).abs().max()) <= 1e-12 * scale
    # The two modes' maps differ (float32 spin factors), so the check above
    # does tell them apart.
    assert float((exact - want).abs().max()) > 1e-12 * scale


def _setup_tiled(n_det=16, n_time=20000, shape=(200, 240)):
    """A tiled CAR engine whose active tiles are the ones the scan hits
    (the others absent), its inputs, random tiles and a signal."""
    import torch
    Q, dets, resp, gamma, _ = synth.workload(n_det, n_time, seed=23, radius_deg=0.5,
                                             throw=2.)
    ny, nx = shape
    r = 2 * ARCMIN * 180 / np.pi
    w = SimpleWCS("CAR", (-180., 50.), (-r, r), (nx / 2 + 0.5, ny / 2 + 0.5))
    p = Projectionist.for_tiled((ny, nx), w, (64, 96))
    q = synth.native(p, Q)
    eng = p.get_ProjEng("TQU")
    t = [torch.from_numpy(x).cuda() for x in (q, dets, resp)]
    rng = np.random.default_rng(6)
    d = torch.from_numpy(rng.standard_normal((n_det, n_time)).astype(np.float32)).cuda()
    shapes = [(3,) + tuple(eng._tile_pix_shape(i)) for i in range(eng._n_tile())]
    hits = eng.to_map([torch.zeros(sh, dtype=torch.float64, device="cuda") for sh in shapes],
                      t[0], t[1], t[2], torch.ones_like(d), None, None)
    active = [i for i, h in enumerate(hits) if float(h.abs().sum()) > 0]
    assert 0 < len(active) < len(shapes)
    p = Projectionist.for_tiled((ny, nx), w, (64, 96), active_tiles=active)
    eng = p.get_ProjEng("TQU")
    tiles = [torch.from_numpy(rng.standard_normal(sh)).cuda() if i in active else None
             for i, sh in enumerate(shapes)]
    return eng, t, tiles, d


def test_tiled_backward_is_to_map_and_adjoint():
    """A tiled map (a list of tiles, those the scan never hits absent): the
    gradient of each present tile is to_map's tile, <P m, d> = <m, P^T d>,
    and the absent tiles get no gradient."""
    import torch
    eng, (q, dets, resp), tiles, d = _setup_tiled()
    leaves = [None if t is None else t.clone().requires_grad_(True) for t in tiles]
    sig = autograd.from_map(eng, leaves, q, dets, resp)
    (sig * d).sum().backward()
    want = eng.to_map([None if t is None else torch.zeros_like(t) for t in tiles], q, dets,
                      resp, d, None, None)
    lhs = float((sig.detach().double() * d.double()).sum())
    rhs = 0.
    for leaf, w in zip(leaves, want):
        if leaf is None:
            assert w is None
            continue
        assert torch.allclose(leaf.grad, w, rtol=1e-12,
                              atol=1e-12 * float(w.abs().max()) + 1e-300)
        rhs += float((leaf.detach() * w).sum())
    scale = float((sig.detach().double().abs() * d.double().abs()).sum())
    assert abs(lhs - rhs) <= 1e-6 * scale
