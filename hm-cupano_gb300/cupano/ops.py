"""``cupano.ops.compute_laplacian`` over this library's Laplacian kernel.

The reference's function (cupano/ops.py:586-600) forms one Laplacian level from two Gaussian
levels with its Triton kernel or a torch fallback; here it runs the kernel the stitchers' pyramid
dump uses (hmp_laplacian_rgba): high minus the alpha-aware bilinear upsample of low, high's alpha.
Tensors on the CPU are copied to the current CUDA device and the result back (there is no CPU
implementation); RGBA (4-channel) levels only.
"""
from __future__ import annotations

import ctypes as C

from hmpano import _lib
from hmpano.pano import _check_backend

__all__ = ["compute_laplacian"]


def compute_laplacian(high, low, *, out=None, backend: str = "auto"):
    """Laplacian of `high` ([B,] H, W, 4) against the next level `low` ([B,] h, w, 4)."""
    import torch

    _check_backend(backend)
    squeeze = high.dim() == 3
    hi = high.unsqueeze(0) if squeeze else high
    lo = low.unsqueeze(0) if low.dim() == 3 else low
    if hi.dim() != 4 or lo.dim() != 4 or hi.shape[-1] != 4 or lo.shape[-1] != 4 or hi.shape[0] != lo.shape[0]:
        raise ValueError("compute_laplacian takes RGBA levels [batch, h, w, 4] of one batch size")
    dev = hi.device if hi.is_cuda else torch.device("cuda", torch.cuda.current_device())
    h = hi.to(device=dev, dtype=torch.float32).contiguous()
    lw = lo.to(device=dev, dtype=torch.float32).contiguous()
    res = torch.empty_like(h)
    s = _lib.lib().hmp_laplacian_rgba(C.c_void_p(h.data_ptr()), h.shape[2], h.shape[1], C.c_void_p(lw.data_ptr()),
                                      lw.shape[2], lw.shape[1], C.c_void_p(res.data_ptr()), h.shape[0],
                                      C.c_void_p(torch.cuda.current_stream(dev).cuda_stream))
    if s.code:
        raise ValueError(s.message.decode(errors="replace"))
    res = res.to(high.device)
    if squeeze:
        res = res[0]
    if out is not None:
        out.copy_(res)
        return out
    return res
