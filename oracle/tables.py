"""Spin-index / coefficient tables of the distillation diagrams (test infrastructure).

This module is part of the ORACLE: it is imported only by ``tests/``, by
``__graft_entry__.smoke()`` and by the CPU-baseline leg of ``bench.py``, always as
the checker.  The product library generates its own tables in C++
(``contractions_code_scattering_gb300/csrc/tables.cpp``); the tests compare the
two and pin both against digests of the reference's shipped headers.

It restates the table generators of the reference,
``devTools/comb_rho.cpp``, ``devTools/comb_rhopi.cpp``, ``devTools/comb_pipi.cpp``,
``devTools/comb_sigma.cpp`` and ``devTools/comb_sigmapi.cpp``: loop order, the
non-zero filter ``abs(coef) != 0`` and the coefficient formulas are the same.
Those generators take their gamma matrices from the (un-vendored) gwu-qcd
library.  The basis that reproduces the shipped ``include/constants_*.h``
exactly, signed zeros included, is the DeGrand-Rossi chiral basis with all four
gamma_mu negated; gamma_5 = g1 g2 g3 g4 = diag(1, 1, -1, -1).  Complex products are
evaluated left to right with the textbook formula, which is what fixes the sign
of zero in the printed coefficients.
"""

from itertools import product

import numpy as np

_Z = (0.0, 0.0)


def _cmul(a, b):
    return (a[0] * b[0] - a[1] * b[1], a[0] * b[1] + a[1] * b[0])


def _cneg(a):
    return (-a[0], -a[1])


def _cscale(s, a):
    return (s * a[0], s * a[1])


def _mat(entries):
    m = [[_Z] * 4 for _ in range(4)]
    for (r, c), v in entries.items():
        m[r][c] = v
    return m


def _mm(a, b):
    out = [[_Z] * 4 for _ in range(4)]
    for i in range(4):
        for j in range(4):
            acc = (0.0, 0.0)
            for k in range(4):
                p = _cmul(a[i][k], b[k][j])
                acc = (acc[0] + p[0], acc[1] + p[1])
            out[i][j] = acc
    return out


# gamma matrices (negated DeGrand-Rossi), entries as (re, im)
G1 = _mat({(0, 3): (0.0, -1.0), (1, 2): (0.0, -1.0), (2, 1): (0.0, 1.0), (3, 0): (0.0, 1.0)})
G2 = _mat({(0, 3): (1.0, 0.0), (1, 2): (-1.0, 0.0), (2, 1): (-1.0, 0.0), (3, 0): (1.0, 0.0)})
G3 = _mat({(0, 2): (0.0, -1.0), (1, 3): (0.0, 1.0), (2, 0): (0.0, 1.0), (3, 1): (0.0, -1.0)})
G4 = _mat({(0, 2): (-1.0, 0.0), (1, 3): (-1.0, 0.0), (2, 0): (-1.0, 0.0), (3, 1): (-1.0, 0.0)})
G5 = _mm(_mm(_mm(G1, G2), G3), G4)
_GI = [G1, G2, G3]


def gamma_matrices():
    """Return (g1, g2, g3, g4, g5) as 4x4 complex numpy arrays."""
    return tuple(np.array([[complex(*e) for e in row] for row in g]) for g in (G1, G2, G3, G4, G5))


def _rhoj(j, i, r, c, dag=False):
    # devTools/comb_rho.cpp:19-49 (same function in comb_rhopi.cpp)
    if j == 1 or j == 3:
        return _cneg(_GI[i][r][c]) if dag else _GI[i][r][c]
    if j == 2:
        return _mm(G4, _GI[i])[r][c]
    if j == 4:
        res = _mm(G4, G4)
        return _cscale(-0.5, res[r][c]) if dag else _cscale(0.5, res[r][c])
    raise ValueError(j)


def _nz(c):
    return (c[0] * c[0] + c[1] * c[1]) != 0.0


def _lp_rp(l, k, i):
    # devTools/comb_rho.cpp:52-74: op index of the source (lp) and sink (rp) ends
    op = [0, 0, 1, 2 + i]
    return op[k], op[l]


def rho_tables():
    """spinIndices_rho[768][4], lp_rp_rho[768][2], coef_rho[768][2] (devTools/comb_rho.cpp:98-180)."""
    spin, lprp, coef = [], [], []
    for l in range(4):
        for k in range(4):
            for i in range(3):
                for s1, s2, s3, s4 in product(range(4), repeat=4):
                    a = _rhoj(k + 1, i, s4, s2, True)
                    if l * 4 + k < 12:
                        a = _cneg(a)
                    c = _cmul(_cmul(_cmul(a, G5[s2][s2]), G5[s1][s1]), _rhoj(l + 1, i, s1, s3))
                    if _nz(c):
                        spin.append((s1, s2, s3, s4))
                        lprp.append(_lp_rp(l, k, i))
                        coef.append(c)
    return (np.array(spin, np.int16), np.array(lprp, np.int16), np.array(coef, np.float64))


def rhopi_tables():
    """spinIndices_rhopi[768][6], ip_rhopi[768], coef_rhopi[768][2] (devTools/comb_rhopi.cpp:90-160)."""
    spin, ip, coef = [], [], []
    for idir in range(3):
        for iop in range(4):
            for s1, s2, s3, s4, s5, s6 in product(range(4), repeat=6):
                c = _cmul(_cmul(_rhoj(iop + 1, idir, s4, s5), G5[s3][s4]), G5[s6][s1])
                if _nz(c):
                    spin.append((s1, s2, s3, s4, s5, s6))
                    ip.append([0, 0, 1, 2 + idir][iop])
                    coef.append(c)
    return (np.array(spin, np.int16), np.array(ip, np.int16), np.array(coef, np.float64))


def pipi_tables():
    """square / doubleTriangle [256][6] and doubleTriangle_hor [256][4] (devTools/comb_pipi.cpp)."""
    sq, sqc, dt, dtc = [], [], [], []
    for s in product(range(4), repeat=6):
        s1, s2, s3, s4, s5, s6 = s
        c = _cmul(G5[s4][s5], G5[s6][s1])
        if _nz(c):
            sq.append(s)
            sqc.append(c)
        c = _cmul(G5[s2][s3], G5[s6][s1])
        if _nz(c):
            dt.append(s)
            dtc.append(c)
    hor = list(product(range(4), repeat=4))
    horc = [(1.0, 0.0)] * 256
    return {
        "spinIndices_pipi_square": np.array(sq, np.int16),
        "coef_pipi_square": np.array(sqc, np.float64),
        "spinIndices_pipi_doubleTriangle": np.array(dt, np.int16),
        "coef_pipi_doubleTriangle": np.array(dtc, np.float64),
        "spinIndices_pipi_doubleTriangle_hor": np.array(hor, np.int16),
        "coef_pipi_doubleTriangle_hor": np.array(horc, np.float64),
    }


def sigma_tables():
    """spinIndices_sigma[64][4], lp_rp_sigma[64][2], coef_sigma[64][2] (devTools/comb_sigma.cpp)."""
    spin, lprp, coef = [], [], []
    for l in range(2):
        for k in range(2):
            for s1, s2, s3, s4 in product(range(4), repeat=4):
                c = _cmul(G5[s2][s3], G5[s4][s1])
                if _nz(c):
                    spin.append((s1, s2, s3, s4))
                    lprp.append((l, k))
                    coef.append(c)
    return (np.array(spin, np.int16), np.array(lprp, np.int16), np.array(coef, np.float64))


def sigmapi_tables():
    """hor_fish [16][2], triangle [128][5] + ip (devTools/comb_sigmapi.cpp)."""
    hf = list(product(range(4), repeat=2))
    hfc = [(1.0, 0.0)] * 16
    spin, ip, coef = [], [], []
    for ik in range(2):
        for s in product(range(4), repeat=5):
            s1, s2, s3, s4, s5 = s
            c = _cmul(G5[s1][s2], G5[s3][s4])
            if _nz(c):
                spin.append(s)
                ip.append(ik)
                coef.append(c)
    return {
        "spinIndices_sigmapi_hor_fish": np.array(hf, np.int16),
        "coef_sigmapi_hor_fish": np.array(hfc, np.float64),
        "spinIndices_sigmapi_triangle": np.array(spin, np.int16),
        "ip_sigmapi_triangle": np.array(ip, np.int16),
        "coef_sigmapi_triangle": np.array(coef, np.float64),
    }


def all_tables():
    """Every table, keyed by the reference's array names."""
    out = {}
    s, lr, c = rho_tables()
    out.update(spinIndices_rho=s, lp_rp_rho=lr, coef_rho=c)
    s, ip, c = rhopi_tables()
    out.update(spinIndices_rhopi=s, ip_rhopi=ip, coef_rhopi=c)
    out.update(pipi_tables())
    s, lr, c = sigma_tables()
    out.update(spinIndices_sigma=s, lp_rp_sigma=lr, coef_sigma=c)
    out.update(sigmapi_tables())
    return out


def format_values(arr):
    """Tokens as the generators print them: ``%d`` for indices, ``%+3.2f`` for coefficients."""
    a = np.asarray(arr)
    if a.dtype.kind == "f":
        return ["%+3.2f" % float(v) for v in a.reshape(-1)]
    return ["%d" % int(v) for v in a.reshape(-1)]
