"""Differentiable direct + one-bounce sink field (torch.autograd.Function).

    E = sink_field(a, x, y, pol, snk_n, scat, scat_n, beta=..., grid=...)

E (complex64 [M,3]) is the sink field of elements at x (float32 [N,3]) excited
by a_n * pol_n (a complex [N], pol complex [N,3] or [3]), with the one-bounce
path through scatter points (scat, scat_n; omit them for the direct path),
composed as the reference does (lyceanem/models/frequency_domain.py:195-264,
:847-849).  Backward returns d/da (complex, torch convention), d/dx and d/dy
(element and sink positions) from the hand-written adjoint kernels of
liblyem_gpu.so (lyem_adjoint); visibility is held at the forward pass's masks
and phases are recomputed, so nothing of size N x M is stored.
"""
import ctypes

import torch

from . import propagation as P
from ._native import check, lib


def _p(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


class SinkField(torch.autograd.Function):
    @staticmethod
    def forward(ctx, a, x, y, pol, snk_n, scat, scat_n, grid, tris, beta, alpha, self_to_self):
        dev = x.device
        a = a.to(torch.complex64).contiguous()
        x = x.to(torch.float32).contiguous()
        y = y.to(torch.float32).contiguous()
        N, M = x.shape[0], y.shape[0]
        pol = P._cvec(pol, N)
        snk_n = P._points(snk_n)
        E_src = (pol * a.reshape(-1, 1)).contiguous()
        kw = dict(beta=beta, alpha=alpha, grid=grid, tris=tris, self_to_self=self_to_self, want_mask=True)
        o_snk = P.direction_order(y, grid.centre) if grid is not None else None
        ts = P.source_schedule(x, grid)  # the transposed schedule for a compact element set
        r0 = P.pair_stage(x, E_src, y, snk_n, snk_order=o_snk, traversal=ts, **kw)
        E = r0.sink
        have_scat = scat is not None and scat.shape[0] > 0
        if have_scat:
            scat = P._points(scat)
            scat_n = P._points(scat_n)
            order = P.spatial_order(scat)
            r1 = P.pair_stage(x, E_src, scat, scat_n, snk_order=order, traversal=ts, **kw)
            w = r1.sink
            r2 = P.pair_stage(scat, w, y, snk_n, src_W=w, sink_out=E, accumulate=True, src_order=order,
                              snk_order=o_snk, **kw)
            masks = (r0.mask_bits, r1.mask_bits, r2.mask_bits)
        else:
            scat = scat_n = w = None
            masks = (r0.mask_bits, None, None)
        ctx.save_for_backward(a, x, y, pol, snk_n)
        ctx.extra = (scat, scat_n, w, masks, float(beta), float(alpha))
        del dev
        return E

    @staticmethod
    def backward(ctx, gE):
        a, x, y, pol, snk_n = ctx.saved_tensors
        scat, scat_n, w, masks, beta, alpha = ctx.extra
        N, M = x.shape[0], y.shape[0]
        Pn = 0 if scat is None else scat.shape[0]
        dev = x.device
        gE = gE.to(torch.complex64).contiguous()
        ga = torch.empty(N, dtype=torch.complex64, device=dev)
        gx = torch.empty((N, 3), dtype=torch.float32, device=dev)
        gy = torch.empty((M, 3), dtype=torch.float32, device=dev) if ctx.needs_input_grad[2] else None
        z = torch.empty((max(Pn, 1), 3), dtype=torch.complex64, device=dev)
        ws = P._ws(lib.lyem_adjoint_workspace(N, Pn, M), dev)
        r = torch.view_as_real
        st = lib.lyem_adjoint(_p(x), _p(r(pol)), _p(r(a)), N, _p(scat), _p(scat_n),
                              _p(None if w is None else r(w)), Pn, _p(y), _p(snk_n), _p(r(gE)), M, _p(masks[0]),
                              _p(masks[1]), _p(masks[2]), alpha, beta, _p(r(ga)), _p(gx), _p(gy), _p(r(z)), _p(ws),
                              ws.numel(), P._stream())
        check(st, "adjoint")
        return (ga if ctx.needs_input_grad[0] else None, gx if ctx.needs_input_grad[1] else None, gy,
                None, None, None, None, None, None, None, None, None)


def sink_field(a, x, y, pol, snk_n, scat=None, scat_n=None, *, beta, alpha=0.0, grid=None, tris=None,
               self_to_self=False):
    """Differentiable sink field (complex64 [M,3]); see the module docstring."""
    return SinkField.apply(a, x, y, pol, snk_n, scat, scat_n, grid, tris, beta, alpha, self_to_self)
