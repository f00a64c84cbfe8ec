"""Differentiable guest-framework energy of guest snapshots.

`GuestFrameworkEnergy` wraps the library's hand-written adjoint kernels
(`fmc_adjoint_eval`) as a torch.autograd.Function: the forward pass returns
E (kcal/mol) of one snapshot, the backward pass scales the analytic
dE/d(guest site coordinates) and dE/d(eps_t, sigma_t, lambda_t) of every
framework atom type by the incoming gradient.  E is the real-space erfc
Coulomb and 12-6 Lennard-Jones interaction of the guest sites with the
framework atoms within the cutoff plus the guest-framework cross term of
the reciprocal Ewald sum; framework type t carries (eps_t, sigma_t,
lambda_t), mixed with the guest sites by Lorentz-Berthelot, lambda_t
scaling the type-t charges.

`uptake_sensitivity` is the reweighting estimator of the derivative of the
mean guest count with respect to a force-field parameter, from snapshots of
a grand-canonical chain: d<N>/dtheta = -beta (<N dE/dtheta> - <N> <dE/dtheta>).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L


class Adjoint:
    """Adjoint kernels bound to one system (framework, guest type, k-vectors)."""

    def __init__(self, system):
        h = C.c_void_p()
        L.check(L.load().fmc_adjoint_create(system._h, C.byref(h)))
        self._h = h
        nt, ns = C.c_int(), C.c_int()
        L.check(L.load().fmc_adjoint_info(self._h, C.byref(nt), C.byref(ns), None))
        self.ntype, self.nsite = nt.value, ns.value

    def base_params(self) -> np.ndarray:
        """The FIELD's (eps_t, sigma_t, 1.0) per framework type, shape (ntype, 3)."""
        out = np.zeros(3 * self.ntype)
        L.check(L.load().fmc_adjoint_info(self._h, None, None, out.ctypes.data_as(L.dp)))
        return out.reshape(self.ntype, 3)

    def evaluate(self, xyz, params):
        """E, dE/dxyz and dE/dparams of one snapshot.  xyz: CUDA float64
        tensor (nmol, nsite, 3); params: (ntype, 3)."""
        import torch
        if not (xyz.is_cuda and xyz.dtype == torch.float64):
            raise TypeError("xyz must be a CUDA float64 tensor")
        x = xyz.contiguous()
        nmol = x.shape[0]
        if x.shape[1:] != (self.nsite, 3):
            raise ValueError("xyz must have shape (nmol, %d, 3)" % self.nsite)
        p = np.ascontiguousarray(np.asarray(params.detach().cpu() if hasattr(params, "detach") else params,
                                            dtype=np.float64).reshape(-1))
        if p.size != 3 * self.ntype:
            raise ValueError("params must have shape (%d, 3)" % self.ntype)
        gx = torch.empty_like(x)
        gp = np.zeros(3 * self.ntype)
        e = C.c_double()
        torch.cuda.synchronize(x.device)
        L.check(L.load().fmc_adjoint_eval(self._h, nmol, C.c_void_p(x.data_ptr()), p.ctypes.data_as(L.dp),
                                          C.byref(e), C.c_void_p(gx.data_ptr()), gp.ctypes.data_as(L.dp)))
        return e.value, gx, gp.reshape(self.ntype, 3)

    def evaluate_batch(self, xyz, nmol, params, precision: str = "fp32"):
        """The sampled energy of a batch of snapshots and its adjoint
        (fmc_adjoint_eval_batch): xyz a CUDA float64 tensor (sum(nmol),
        nsite, 3) holding every snapshot's molecules one after the other,
        nmol the molecule count of each snapshot.  Returns energies (S,)
        numpy, dE/dxyz as a CUDA float32 tensor shaped like xyz, and
        dE/dparams (S, ntype, 3) numpy."""
        import torch
        if not (xyz.is_cuda and xyz.dtype == torch.float64):
            raise TypeError("xyz must be a CUDA float64 tensor")
        x = xyz.contiguous()
        nm = np.ascontiguousarray(np.asarray(nmol, dtype=np.int32).reshape(-1))
        if x.shape[1:] != (self.nsite, 3) or x.shape[0] != int(nm.sum()):
            raise ValueError("xyz must have shape (sum(nmol), %d, 3)" % self.nsite)
        p = np.ascontiguousarray(np.asarray(params.detach().cpu() if hasattr(params, "detach") else params,
                                            dtype=np.float64).reshape(-1))
        if p.size != 3 * self.ntype:
            raise ValueError("params must have shape (%d, 3)" % self.ntype)
        prec = L.FMC_PREC_FP32 if precision == "fp32" else L.FMC_PREC_FP64
        gx = torch.empty(x.shape, dtype=torch.float32, device=x.device)
        xp = C.c_void_p(x.data_ptr()) if x.numel() else None
        gxp = C.c_void_p(gx.data_ptr()) if gx.numel() else None
        e = np.zeros(max(1, nm.size))
        gp = np.zeros(max(1, nm.size) * 3 * self.ntype)
        torch.cuda.synchronize(x.device)
        L.check(L.load().fmc_adjoint_eval_batch(
            self._h, int(nm.size), nm.ctypes.data_as(L.ip), xp, p.ctypes.data_as(L.dp), prec,
            e.ctypes.data_as(L.dp), gxp, gp.ctypes.data_as(L.dp)))
        return e[:nm.size], gx, gp[:nm.size * 3 * self.ntype].reshape(nm.size, self.ntype, 3)

    def close(self) -> None:
        if self._h:
            L.load().fmc_adjoint_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _function():
    import torch

    class GuestFrameworkEnergy(torch.autograd.Function):
        """E(xyz, params) of one snapshot with the adjoint as its backward."""

        @staticmethod
        def forward(ctx, adj, xyz, params):
            e, gx, gp = adj.evaluate(xyz, params)
            ctx.save_for_backward(gx, torch.as_tensor(gp, dtype=params.dtype, device=params.device))
            return torch.tensor(e, dtype=torch.float64, device=params.device)

        @staticmethod
        def backward(ctx, grad):
            gx, gp = ctx.saved_tensors
            return None, grad.to(gx.device) * gx, grad.to(gp.device) * gp

    return GuestFrameworkEnergy


def guest_framework_energy(adj: Adjoint, xyz, params):
    """Differentiable E (kcal/mol): torch autograd through the adjoint."""
    return _function().apply(adj, xyz, params)


def _batch_function():
    import torch

    class SampledEnergy(torch.autograd.Function):
        """E_q(xyz, params) of a batch of snapshots (the chains' sampled
        energy) with the batched adjoint as its backward."""

        @staticmethod
        def forward(ctx, adj, xyz, nmol, params, precision):
            e, gx, gp = adj.evaluate_batch(xyz, nmol, params, precision)
            ctx.save_for_backward(gx, torch.as_tensor(gp, dtype=params.dtype, device=params.device))
            ctx.snap = torch.as_tensor(np.repeat(np.arange(len(e)), np.asarray(nmol)), device=xyz.device)
            return torch.as_tensor(e, dtype=torch.float64, device=params.device)

        @staticmethod
        def backward(ctx, grad):
            gx, gp = ctx.saved_tensors
            gm = grad.to(gx.device, torch.float64)[ctx.snap].view(-1, 1, 1)
            gxyz = gm * gx.to(torch.float64)
            gpar = (grad.to(gp.device).view(-1, 1, 1) * gp).sum(dim=0)
            return None, gxyz, None, gpar, None

    return SampledEnergy


def sampled_energy(adj: Adjoint, xyz, nmol, params, precision: str = "fp32"):
    """Differentiable energies (kcal/mol) of a batch of snapshots."""
    return _batch_function().apply(adj, xyz, nmol, params, precision)


def uptake_sensitivity(n, de_dtheta, beta: float):
    """d<N>/dtheta from snapshots by reweighting: n (S,) guest counts,
    de_dtheta (S, P) derivatives of each snapshot's energy; returns (P,)."""
    n = np.asarray(n, dtype=np.float64)
    g = np.asarray(de_dtheta, dtype=np.float64).reshape(len(n), -1)
    return -beta * ((n[:, None] * g).mean(axis=0) - n.mean() * g.mean(axis=0))
