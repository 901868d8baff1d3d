"""Differentiable from_map.

from_map is the linear operator P: map -> signal (the pointing matrix
applied to a map); to_map is its transpose P^T: signal -> map.  FromMap
wraps from_map as a torch.autograd.Function whose hand-written backward is
to_map applied to the incoming signal gradient, so that

    <P m, d> = <m, P^T d>

and gradients of any loss of the projected signal flow back to the map.
Both directions run the CUDA kernels of this package on the current
stream.  Maps are CUDA float64 tensors of shape (n_comp, ...), or for a
tiled engine lists of such tiles (None for an absent tile; a gradient is
returned for each present one); the signal is float32 (n_det, n_time).  The engine's pointing mode is read once,
in forward, and backward runs to_map in that same mode, so that the pair
stays an adjoint pair even if the caller changes ``eng.pointing`` between
the two.
"""
import contextlib

import torch

from .projeng import DEFAULT_POINTING


@contextlib.contextmanager
def _pointing(eng, mode):
    """Runs the block with ``eng.pointing = mode``, then restores it."""
    had = "pointing" in vars(eng)
    old = getattr(eng, "pointing", None)
    eng.pointing = mode
    try:
        yield
    finally:
        if had:
            eng.pointing = old
        else:
            del eng.pointing


class FromMap(torch.autograd.Function):
    """signal = P(map) for a fixed pointing (engine, boresight, detectors,
    responses); backward: grad_map = P^T(grad_signal) via to_map."""

    @staticmethod
    def forward(ctx, map, eng, boresight, dets, response):
        if not (isinstance(map, torch.Tensor) and map.is_cuda and map.dtype == torch.float64):
            raise TypeError("FromMap needs a CUDA float64 map tensor")
        if getattr(eng, "_tiled", False):
            raise TypeError("FromMap takes untiled maps; tiled maps go through FromMapTiled")
        ctx.eng = eng
        ctx.mode = getattr(eng, "pointing", DEFAULT_POINTING)
        ctx.save_for_backward(boresight, dets, response)
        ctx.map_shape = tuple(map.shape)
        with torch.no_grad():
            sig = eng.from_map(map.detach().contiguous(), boresight, dets, response, None)
        return sig

    @staticmethod
    def backward(ctx, grad_sig):
        boresight, dets, response = ctx.saved_tensors
        g = grad_sig.detach().to(torch.float32).contiguous()
        gmap = torch.zeros(ctx.map_shape, dtype=torch.float64, device=g.device)
        with _pointing(ctx.eng, ctx.mode):
            ctx.eng.to_map(gmap, boresight, dets, response, g, None, None)
        return gmap, None, None, None, None


class FromMapTiled(torch.autograd.Function):
    """FromMap for a tiled engine: the present tiles are the function's
    tensor inputs (autograd tracks only direct tensor arguments), `present`
    their tile numbers; backward returns to_map's tiles as their
    gradients."""

    @staticmethod
    def forward(ctx, eng, boresight, dets, response, present, n_tile, *tiles):
        for t in tiles:
            if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.float64):
                raise TypeError("FromMap needs CUDA float64 tile tensors")
        ctx.eng = eng
        ctx.mode = getattr(eng, "pointing", DEFAULT_POINTING)
        ctx.present = present
        ctx.n_tile = n_tile
        ctx.shapes = [tuple(t.shape) for t in tiles]
        ctx.save_for_backward(boresight, dets, response)
        full = [None] * n_tile
        for i, t in zip(present, tiles):
            full[i] = t.detach().contiguous()
        with torch.no_grad():
            sig = eng.from_map(full, boresight, dets, response, None)
        return sig

    @staticmethod
    def backward(ctx, grad_sig):
        boresight, dets, response = ctx.saved_tensors
        g = grad_sig.detach().to(torch.float32).contiguous()
        grads = [torch.zeros(sh, dtype=torch.float64, device=g.device) for sh in ctx.shapes]
        full = [None] * ctx.n_tile
        for i, t in zip(ctx.present, grads):
            full[i] = t
        with _pointing(ctx.eng, ctx.mode):
            ctx.eng.to_map(full, boresight, dets, response, g, None, None)
        return (None, None, None, None, None, None) + tuple(grads)


def from_map(eng, map, boresight, dets, response):
    """Differentiable ``eng.from_map(map, boresight, dets, response)``: the
    inputs other than the map are CUDA tensors (boresight (n_time, 4) and
    dets (n_det, 4) float64, response (n_det, 2) float32).  A tiled
    engine's map is a list of tiles (None: absent); its present tiles get
    gradients."""
    if isinstance(map, (list, tuple)):
        present = tuple(i for i, t in enumerate(map) if t is not None)
        return FromMapTiled.apply(eng, boresight, dets, response, present, len(map),
                                  *[map[i] for i in present])
    return FromMap.apply(map, eng, boresight, dets, response)
