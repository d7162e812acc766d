"""numpy restatement of the reference drivers' elemental construction (test
infrastructure: the checker of ctr_elementals, never the product path).

tests/compute_rho.cpp builds, per momentum p and time slice t (the same loops
in tests/compute_{rhopi,pipi_I0,pipi_I1,sigma,sigmapi}.cpp):
  :116-130  plain      matp(r,c)   = <v_r| e^{-ip.x} |v_c>
  :132-163  smeared    matps(r,c)  = sum_j <D_j v_r| e^{-ip.x} |D_j v_c>
  :165-201  commutator matpc_j(r,c) = <v_r| e^{-ip.x} |D_j v_c> - <D_j v_r| e^{-ip.x} |v_c>
  :204-223  tmpMom[op][t][r][c] = (matp, matps, matpc_x, matpc_y, matpc_z)
with <a|b> = sum over sites and colours of conj(a) b (cscalar_product) and the
phase exp(-i 2 pi (x p_x/nx + y p_y/ny + z p_z/nz)) (:122).  The covariant
derivative (lapmult::covderiv) belongs to the gwu-qcd library, which the
reference does not ship; this restatement uses the symmetric lattice derivative
D_j v(x) = U_j(x) v(x + j) - U_j(x - j)^dagger v(x - j) (periodic), the
definition ctr_elementals states, so parity of ops 1-4 with the reference's own
library is unpinned.
"""

import numpy as np


def covderiv(v, U, j):
    """D_j v for v [nev, nz, ny, nx, 3] and U [nz, ny, nx, 3, 3, 3] of one slice."""
    vax = {0: 3, 1: 2, 2: 1}[j]  # x, y, z axes of v
    uax = vax - 1  # the same axes of U
    Uj = U[:, :, :, j]
    vp = np.roll(v, -1, axis=vax)  # v(x + j)
    vm = np.roll(v, 1, axis=vax)  # v(x - j)
    Ub = np.roll(Uj, 1, axis=uax)  # U_j(x - j)
    return np.einsum("zyxab,czyxb->czyxa", Uj, vp) - np.einsum("zyxba,czyxb->czyxa", Ub.conj(), vm)


def phase(moms_p, nx, ny, nz):
    px, py, pz = moms_p
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    return np.exp(-2j * np.pi * (x * px / nx + y * py / ny + z * pz / nz))


def elementals(evec, moms, links=None):
    """[nmom, nops, nt, nev, nev] with nops = 5 when links are given, else 1."""
    nt, nev, nz, ny, nx, _ = evec.shape
    nops = 5 if links is not None else 1
    out = np.zeros((len(moms), nops, nt, nev, nev), np.complex128)
    for t in range(nt):
        v = evec[t]
        d = [covderiv(v, links[t], j) for j in range(3)] if links is not None else None
        for p, mp in enumerate(moms):
            ph = phase(mp, nx, ny, nz)

            def prod(a, b):
                return np.einsum("rzyxa,zyx,czyxa->rc", a.conj(), ph, b, optimize=True)

            out[p, 0, t] = prod(v, v)
            if d is not None:
                out[p, 1, t] = sum(prod(d[j], d[j]) for j in range(3))
                for j in range(3):
                    out[p, 2 + j, t] = prod(v, d[j]) - prod(d[j], v)
    return out
