"""Distillation-profile objective and its gradient through the library's
hand-written adjoint kernels.

Every elemental Phi(p, t) is replaced by diag(f) Phi(p, t) diag(f) for a real
per-eigenvector profile f.  The correlators are differentiated in reverse mode
by the library (include/ctr.h: ctr_rho_profile_vjp, ctr_pipi_profile_vjp):
torch.autograd.Function wrappers hand the output gradients to those kernels as
complex weights, so a torch objective built on the correlators gets df from the
CUDA adjoint.  The wrappers exist for checks and for driving the objective; all
contraction work runs in libctr.so.

Objective (the profile benchmark):
    L(f) = sum_{t=t0..t1} [log|C_rho(t)| - log|C_rho(t+1)|]^2 + sum_d Re C_pipi,d(dt_pipi)
with C_rho(t) the zero-momentum rho correlator (gamma_i x Phi at both ends,
averaged over the 3 polarisations) and C_pipi,d the isospin-weighted pi pi
diagrams (square, double triangle, star, fish, horizontal double triangle), both
averaged over source times.  The magnitudes |C| make the logarithms real for
complex synthetic correlators.
"""

import numpy as np
import torch

from . import api


def _cplx(g):
    return torch.complex(g[..., 0], -g[..., 1])


class RhoProfile(torch.autograd.Function):
    """f -> rho correlators [Nt, Nt, 48, 2] (real view) on the entries of `mask`."""

    @staticmethod
    def forward(ctx, f, prop, mom5, mask, engine):
        w = mask.to(torch.complex128).contiguous()
        corr, _ = api.rho_profile_vjp(prop, mom5, f.detach().contiguous(), w, corr=True, grad=False, engine=engine)
        ctx.save_for_backward(f)
        ctx.data = (prop, mom5, mask, engine)
        return torch.stack([corr.real, corr.imag], dim=-1)

    @staticmethod
    def backward(ctx, g):
        (f,) = ctx.saved_tensors
        prop, mom5, mask, engine = ctx.data
        w = (_cplx(g) * mask).contiguous()
        _, grad = api.rho_profile_vjp(prop, mom5, f.detach().contiguous(), w, corr=False, grad=True, engine=engine)
        return grad, None, None, None, None


class PipiProfile(torch.autograd.Function):
    """f -> pi pi correlators [Nt, Nt, 5, 2] (real view) on the pairs of `mask`."""

    @staticmethod
    def forward(ctx, f, prop, p1, p2, p3, p4, mask, isospin, engine):
        w = mask.to(torch.complex128).contiguous()
        corr, _ = api.pipi_profile_vjp(prop, p1, p2, p3, p4, f.detach().contiguous(), w, isospin, corr=True,
                                       grad=False, engine=engine)
        ctx.save_for_backward(f)
        ctx.data = (prop, p1, p2, p3, p4, mask, isospin, engine)
        return torch.stack([corr.real, corr.imag], dim=-1)

    @staticmethod
    def backward(ctx, g):
        (f,) = ctx.saved_tensors
        prop, p1, p2, p3, p4, mask, isospin, engine = ctx.data
        w = (_cplx(g) * mask).contiguous()
        _, grad = api.pipi_profile_vjp(prop, p1, p2, p3, p4, f.detach().contiguous(), w, isospin, corr=False,
                                       grad=True, engine=engine)
        return grad, None, None, None, None, None, None, None, None


def dt_mask(nt, dts, nout, outputs, device):
    """mask[tf][ti][o] = ((tf - ti) mod Nt in dts) and o in outputs."""
    m = torch.zeros((nt, nt, nout), dtype=torch.bool, device=device)
    ti = torch.arange(nt, device=device)
    for dt in dts:
        for o in outputs:
            m[(ti + dt) % nt, ti, o] = True
    return m


def source_average(corr_real, dt):
    """1/Nt sum_ti corr[(ti + dt) % Nt][ti] (dumpData, lib/contract.cpp:621-631) on the real view."""
    nt = corr_real.shape[0]
    ti = torch.arange(nt, device=corr_real.device)
    return corr_real[(ti + dt) % nt, ti].mean(dim=0)


def default_profile(nev, seed=7, width=0.3):
    """f_k = exp(-lambda_k / width) for sorted lambda_k uniform in [0, 1]."""
    lam = np.sort(np.random.default_rng(seed).uniform(0.0, 1.0, nev))
    return np.exp(-lam / width)


def objective(f, prop, mom5, pipi, rho_ts=(2, 8), pipi_dt=4, isospin=0, engine="fp64"):
    """L(f) as a torch scalar (differentiable in f through the CUDA adjoint).

    prop: full perambulator [Nt, Nt, 4, 4, N, N]; mom5: rho elementals at zero
    momentum [Nt, 5, N, N]; pipi: (P1, P2, P3, P4) [Nt, N, N] each; engine: where
    the chain products run ("fp64" or "split")."""
    nt = prop.shape[0]
    t0, t1 = rho_ts
    rmask = dt_mask(nt, range(t0, t1 + 2), 48, (0, 1, 2), prop.device)
    rho = RhoProfile.apply(f, prop, mom5, rmask, engine)
    logc = []
    for t in range(t0, t1 + 2):
        c = source_average(rho, t)[0:3].mean(dim=0)  # polarisation average of ico = 0
        logc.append(0.5 * torch.log(c[0] ** 2 + c[1] ** 2))
    loss = sum((logc[i] - logc[i + 1]) ** 2 for i in range(len(logc) - 1))
    pmask = dt_mask(nt, (pipi_dt,), 5, range(5), prop.device)
    pp = PipiProfile.apply(f, prop, *pipi, pmask, isospin, engine)
    return loss + source_average(pp, pipi_dt)[:, 0].sum()
