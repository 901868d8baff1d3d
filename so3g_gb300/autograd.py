"""Differentiable from_map.

from_map is the linear operator P: map -> signal (the pointing matrix
applied to a map); to_map is its transpose P^T: signal -> map.  FromMap
wraps from_map as a torch.autograd.Function whose hand-written backward is
to_map applied to the incoming signal gradient, so that

    <P m, d> = <m, P^T d>

and gradients of any loss of the projected signal flow back to the map.
Both directions run the CUDA kernels of this package on the current
stream.  Maps are untiled CUDA float64 tensors of shape (n_comp, ...); the
signal is float32 (n_det, n_time).
"""
import torch


class FromMap(torch.autograd.Function):
    """signal = P(map) for a fixed pointing (engine, boresight, detectors,
    responses); backward: grad_map = P^T(grad_signal) via to_map."""

    @staticmethod
    def forward(ctx, map, eng, boresight, dets, response):
        if not (isinstance(map, torch.Tensor) and map.is_cuda and map.dtype == torch.float64):
            raise TypeError("FromMap needs a CUDA float64 map tensor")
        if getattr(eng, "_tiled", False):
            raise TypeError("FromMap supports untiled maps only")
        ctx.eng = eng
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
        ctx.eng.to_map(gmap, boresight, dets, response, g, None, None)
        return gmap, None, None, None, None


def from_map(eng, map, boresight, dets, response):
    """Differentiable ``eng.from_map(map, boresight, dets, response)``: the
    inputs other than the map are CUDA tensors (boresight (n_time, 4) and
    dets (n_det, 4) float64, response (n_det, 2) float32)."""
    return FromMap.apply(map, eng, boresight, dets, response)
