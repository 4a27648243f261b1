"""Differentiable forward model behind torch.autograd: white noise and P(k)
knot amplitudes -> (2)LPT particles -> CIC -> binned P(k) -> chi^2 against a
target spectrum, with the hand-written CUDA adjoint (exh_diff_forward /
exh_diff_backward of the C ABI) as the backward pass.

The halo finder is not part of this model: it stays discrete and exact.
"""
import ctypes as C

import numpy as np
import torch

from . import _capi


def knots_from_spectrum(k, P, n_knots, k_lo, k_hi):
    """n_knots log-spaced knots in [k_lo, k_hi] with amplitudes interpolated
    (log-log) from a tabulated spectrum."""
    kk = np.geomspace(k_lo, k_hi, n_knots)
    PP = np.exp(np.interp(np.log(kk), np.log(np.asarray(k, dtype=np.float64)), np.log(np.asarray(P, dtype=np.float64))))
    return kk.astype(np.float32), PP.astype(np.float32)


class _Model:
    def __init__(self, nd, L, knot_k, Nk, k_min=None, k_max=None, Om0=0.31, z=0.0, do_2lpt=True):
        self.prm = _capi.DiffParams()
        self.prm.nd = int(nd)
        self.prm.L = float(L)
        self.prm.Om0 = float(Om0)
        self.prm.redshift = float(z)
        self.prm.do_2lpt = int(bool(do_2lpt))
        self.knot_k = np.ascontiguousarray(knot_k, dtype=np.float32)
        self.prm.n_knots = self.knot_k.size
        self.prm.Nk = int(Nk)
        self.prm.k_min = float(np.float32(2 * np.pi / L) if k_min is None else k_min)
        self.prm.k_max = float(np.float32(np.pi * nd / L) if k_max is None else k_max)

    def forward(self, noise, knot_P, target, var=None):
        L_ = _capi.load()
        kP = np.ascontiguousarray(knot_P, dtype=np.float32)
        T = np.ascontiguousarray(target, dtype=np.float32)
        v = None if var is None else np.ascontiguousarray(var, dtype=np.float32)
        loss = C.c_double(0.0)
        Nk = self.prm.Nk
        P = np.zeros(Nk, dtype=np.float32)
        kb = np.zeros(Nk, dtype=np.float32)
        cnt = np.zeros(Nk, dtype=np.int64)
        # the adjoint must run on the context that holds this forward's
        # intermediates, whichever thread calls it (autograd runs backward
        # on its own thread)
        self.ctx = _capi.context()
        _capi.check(L_.exh_diff_forward(self.ctx, C.byref(self.prm), _capi.ptr(noise), _capi.ptr(self.knot_k),
                                        _capi.ptr(kP), _capi.ptr(T), _capi.ptr(v), C.byref(loss), _capi.ptr(P),
                                        _capi.ptr(kb), _capi.ptr(cnt), None))
        return loss.value, P, kb, cnt

    def backward(self, grad_loss, grad_noise):
        gk = np.zeros(self.prm.n_knots, dtype=np.float64)
        if getattr(self, "ctx", None) is None:
            raise RuntimeError("backward before forward")
        _capi.check(_capi.load().exh_diff_backward(self.ctx, float(grad_loss), _capi.ptr(grad_noise),
                                                   _capi.ptr(gk), None))
        return gk


class PkChi2(torch.autograd.Function):
    """loss = PkChi2.apply(noise, knot_P, model, target[, var]).

    noise: CUDA float32 tensor (nd, nd, nd); knot_P: float tensor of knot
    amplitudes (any device); model: a _Model (see pk_chi2_model).  The
    backward of one forward must run before the next forward on the same
    thread (the adjoint reads the intermediates the forward keeps)."""

    @staticmethod
    def forward(ctx, noise, knot_P, model, target, var=None):
        if not noise.is_cuda or noise.dtype != torch.float32 or not noise.is_contiguous():
            raise ValueError("noise must be a contiguous CUDA float32 tensor")
        torch.cuda.synchronize(noise.device)
        loss, P, kb, cnt = model.forward(noise, knot_P.detach().cpu().numpy(), target, var)
        ctx.model = model
        ctx.noise_shape = noise.shape
        ctx.knot_device, ctx.knot_dtype = knot_P.device, knot_P.dtype
        ctx.P = P
        return torch.tensor(loss, dtype=torch.float64, device=noise.device)

    @staticmethod
    def backward(ctx, g):
        gn = torch.empty(ctx.noise_shape, dtype=torch.float32, device=g.device)
        gk = ctx.model.backward(float(g), gn)
        torch.cuda.synchronize(g.device)
        return gn, torch.as_tensor(gk, dtype=ctx.knot_dtype, device=ctx.knot_device), None, None, None


def pk_chi2_model(nd, L, knot_k, Nk=64, k_min=None, k_max=None, Om0=0.31, z=0.0, do_2lpt=True):
    return _Model(nd, L, knot_k, Nk, k_min, k_max, Om0, z, do_2lpt)


def pk_chi2(noise, knot_P, model, target, var=None):
    return PkChi2.apply(noise, knot_P, model, target, var)
