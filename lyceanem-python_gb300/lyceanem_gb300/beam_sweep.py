"""Beam sweeps over a formed propagation network (torch-level API).

The reference evaluates each excitation by re-running the whole model
(lyceanem/models/frequency_domain.py:858-921, multiE); here the network G of a
scene is formed once on the device (pair stage with unit excitations) and the
sink fields of K excitation vectors are three complex GEMMs:
    E[m, k, c] = sum_n G[n, m, c] W[k, n].
Modes: "fp32" (cublasCgemm, the comparison path), "bf16x3g" and "fp16x3g"
(this package's tcgen05 kernel: every real operand split into hi + lo halves,
each complex product formed from three real products, Gauss's Gr Wr, Gi Wi,
(Gr + Gi)(Wr + Wi), 6 instead of 8 M N K flops per component, each real product
accumulated in FP32 as hi*hi + lo*hi + hi*lo; FP16 operands are scaled by powers
of two so that no half overflows).
"""
import ctypes

import torch

from . import propagation as P
from ._native import check, lib

MODES = {"fp32": 0, "bf16x3g": 3, "fp16x3g": 4}


def set_multicast(on):
    """True: the tensor-core kernel in clusters of two CTAs sharing each weight tile by multicast; False
    (default): single CTAs.  Results are the same."""
    check(lib.lyem_sweep_set_multicast(int(bool(on))), "sweep_set_multicast")


def set_k_tile(k_tile):
    """Sources per pipeline stage of the tensor-core kernel: 32 (default) or 64."""
    check(lib.lyem_sweep_set_k_tile(int(k_tile)), "sweep_set_k_tile")


def _p(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def form_network(src, pol, snk, snk_n, *, beta, alpha=0.0, grid=None, tris=None, weights=None, self_to_self=True):
    """Propagation network complex64 [N, M, 3] for unit element excitations pol (complex [3] or [N,3]),
    optionally scaled per element by `weights` (e.g. element areas).  self_to_self=True tests every pair;
    False reproduces the reference engine's untested pair n == m."""
    src = P._points(src)
    E = P._cvec(pol, src.shape[0])
    if weights is not None:
        E = E * P._dev(weights, torch.complex64).reshape(-1, 1)
    return P.pair_stage(src, E, snk, snk_n, beta=beta, alpha=alpha, grid=grid, tris=tris, want_pairs=True,
                        self_to_self=self_to_self).pairs


class BeamSweep:
    """A network prepared as the GEMM operand of one mode; run(W) evaluates K excitations at once."""

    def __init__(self, network, mode="bf16x3g"):
        net = network.contiguous()
        assert net.dtype == torch.complex64 and net.dim() == 3 and net.shape[2] == 3
        self.mode = MODES[mode]
        self.n_src, self.n_snk = net.shape[0], net.shape[1]
        self.ld = (self.n_snk + 7) // 8 * 8
        nbytes = lib.lyem_sweep_network_bytes(self.n_src, self.ld, self.mode)
        self.operand = torch.empty(max(nbytes, 16), dtype=torch.uint8, device=net.device)
        self._wbuf = None
        self._ws = None
        self.refresh(net)

    def refresh(self, network):
        """Rewrites the operand from a network of the same shape (no allocation)."""
        net = network.contiguous()
        assert net.dtype == torch.complex64 and tuple(net.shape) == (self.n_src, self.n_snk, 3)
        check(lib.lyem_sweep_prepare_network(_p(torch.view_as_real(net)), self.n_src, self.n_snk, self.mode, self.ld,
                                             _p(self.operand), P._stream()), "sweep_prepare_network")
        return self

    def run(self, W, out=None):
        """Sink fields for excitations W complex [K, N]: returns complex64 [3, K, ld] (use .fields())."""
        W = P._dev(W, torch.complex64).reshape(-1, self.n_src).contiguous()
        K = W.shape[0]
        B = None
        if self.mode != 0:
            nb = lib.lyem_sweep_weights_bytes(self.n_src, K, self.mode)
            if self._wbuf is None or self._wbuf.numel() < nb:
                self._wbuf = torch.empty(nb, dtype=torch.uint8, device=W.device)
            B = self._wbuf
            check(lib.lyem_sweep_prepare_weights(_p(torch.view_as_real(W)), self.n_src, K, self.mode, _p(B),
                                                 P._stream()), "sweep_prepare_weights")
        if out is None:
            out = torch.empty((3, K, self.ld), dtype=torch.complex64, device=W.device)
        nws = lib.lyem_sweep_workspace_bytes(self.ld, K, self.mode)
        if nws and (self._ws is None or self._ws.numel() < nws):
            self._ws = torch.empty(nws, dtype=torch.uint8, device=W.device)
        ws = self._ws if nws else None
        check(lib.lyem_sweep_run_ws(_p(self.operand), self.n_src, self.n_snk, self.ld, _p(torch.view_as_real(W)),
                                    _p(B), K, self.mode, _p(torch.view_as_real(out)), self.ld, _p(ws),
                                    0 if ws is None else ws.numel(), P._stream()), "sweep_run")
        return out

    def fields(self, out):
        """View of run()'s output as E[m, k, c] (complex64 [M, K, 3], strided)."""
        return out[:, :, :self.n_snk].permute(2, 1, 0)
