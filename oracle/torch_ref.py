"""Plain-PyTorch FP64 restatement of the rho and pi pi correlators as functions
of the distillation profile f (test infrastructure: the reference gradient of
the profile adjoint, obtained with torch.autograd on the CPU).

The chains are the reference's, row by row, batched over spin rows with
gathered blocks:
  rho  (lib/calculate_rho_core.h):  coef * sum (tau_{s3s4} Phi'_lp(ti)) (.) conj(Phi'_rp(tf) tau_{s1s2})
  pi pi square / double triangle / horizontal double triangle / star / fish
       (lib/calculate_pipi_*_core.h, weights lib/contract_kernels_pipi.cu:288-303, :463-478)
with Phi' = diag(f) Phi diag(f).  Inputs are torch complex128 CPU tensors; f is
a float64 tensor (requires_grad for the reference gradient).
"""

import torch

from . import tables as T

_TABLES = {}


def _tab():
    if not _TABLES:
        s, lr, c = T.rho_tables()
        _TABLES["rho"] = (torch.from_numpy(s.astype("int64")), torch.from_numpy(lr.astype("int64")),
                          torch.complex(torch.from_numpy(c[:, 0]), torch.from_numpy(c[:, 1])))
        p = T.pipi_tables()
        for k, name in (("sq", "square"), ("dt", "doubleTriangle"), ("dth", "doubleTriangle_hor")):
            cf = p["coef_pipi_" + name]
            _TABLES[k] = (torch.from_numpy(p["spinIndices_pipi_" + name].astype("int64")),
                          torch.complex(torch.from_numpy(cf[:, 0]), torch.from_numpy(cf[:, 1])))
    return _TABLES


def profiled(f, phi):
    fc = f.to(torch.complex128)
    return fc[:, None] * phi * fc[None, :]


def _had(x, y):
    """sum over the last two axes of x (.) conj(y) = Tr[x y^dagger]."""
    return (x * y.conj()).sum(dim=(-2, -1))


def rho_pair(prop, mom5p, tf, ti, outputs):
    """corr[o] for o in outputs (o = ico*3 + dir) of one (t_sink, t_src) pair; mom5p profiled [Nt, 5, N, N]."""
    spin, lprp, coef = _tab()["rho"]
    rows = torch.cat([torch.arange(o * 16, o * 16 + 16) for o in outputs])
    s = spin[rows]
    blk = prop[tf, ti]
    t1 = blk[s[:, 2], s[:, 3]] @ mom5p[ti, lprp[rows, 0]]
    t2 = mom5p[tf, lprp[rows, 1]] @ blk[s[:, 0], s[:, 1]]
    v = coef[rows] * _had(t1, t2)
    return v.reshape(len(outputs), 16).sum(dim=1)


def pipi_pair(prop, P, tf, ti, isospin):
    """corr[5] (square, double triangle, star, fish, horizontal double triangle) of one pair;
    P = (P1, P2, P3, P4) profiled [Nt, N, N] each."""
    P1, P2, P3, P4 = P
    tab = _tab()
    row, dtf, dti = prop[tf, ti], prop[tf, tf], prop[ti, ti]
    s, c = tab["sq"]
    m = P3[tf] @ dtf[s[:, 2], s[:, 3]] @ P4[tf] @ row[s[:, 4], s[:, 5]] @ P2[ti] @ dti[s[:, 0], s[:, 1]] @ P1[ti]
    sq = (c * _had(m, row[s[:, 2], s[:, 1]])).sum()
    s, c = tab["dt"]
    m = P3[tf] @ dtf[s[:, 4], s[:, 5]] @ P4[tf] @ row[s[:, 0], s[:, 1]] @ P1[ti] @ dti[s[:, 2], s[:, 3]] @ P2[ti]
    dt = (c * _had(m, row[s[:, 4], s[:, 3]])).sum()
    s, c = tab["dth"]
    m = (P3[tf] @ row[s[:, 0], s[:, 1]] @ P1[ti] @ row[s[:, 2], s[:, 1]].conj().transpose(-1, -2) @ P4[tf]
         @ row[s[:, 2], s[:, 3]] @ P2[ti])
    dth = (c * _had(m, row[s[:, 0], s[:, 3]])).sum()
    idx = torch.arange(16)
    tb = row[idx // 4, idx % 4]

    def twin(pa, pb):
        return _had(pa[tf] @ tb @ pb[ti], tb).sum()

    star = twin(P4, P1) * twin(P3, P2)
    fish = twin(P3, P1) * twin(P4, P2)
    if isospin == 1:
        return torch.stack([-2.0 * sq, 2.0 * dt, -star, fish, torch.zeros_like(sq)])
    return torch.stack([-sq / 3.0, -dt / 3.0, star, fish, -5.0 / 3.0 * dth])


def objective(f, prop, mom5, pipi, rho_ts=(2, 8), pipi_dt=4, isospin=0):
    """The profile objective of contractions_code_scattering_gb300.adjoint.objective, in plain torch."""
    nt = prop.shape[0]
    mom5p = profiled(f, mom5)
    P = tuple(profiled(f, p) for p in pipi)
    t0, t1 = rho_ts
    logc = []
    for t in range(t0, t1 + 2):
        c = sum(rho_pair(prop, mom5p, (ti + t) % nt, ti, (0, 1, 2)).mean() for ti in range(nt)) / nt
        logc.append(torch.log(c.abs()))
    loss = sum((logc[i] - logc[i + 1]) ** 2 for i in range(len(logc) - 1))
    pp = sum(pipi_pair(prop, P, (ti + pipi_dt) % nt, ti, isospin) for ti in range(nt)) / nt
    return loss + pp.real.sum()
