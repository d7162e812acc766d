"""ctypes binding of the C oracle (test infrastructure, never the product path).

Every wrapper takes and returns numpy complex128 arrays in the reference's
layouts (see oracle.c) and calls the OpenMP restatement of one reference
routine.  Tables default to the ones generated by ``oracle.tables``.
"""

import ctypes
import os
import subprocess

import numpy as np

from . import tables as T

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


def build():
    subprocess.check_call(["make", "-s", "-C", _HERE])


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        src = os.path.join(_HERE, "oracle.c")
        if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(src):
            build()
        _LIB = ctypes.CDLL(path)
    return _LIB


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _c(a):
    a = np.ascontiguousarray(a, dtype=np.complex128)
    return a


def _i16(a):
    return np.ascontiguousarray(a, dtype=np.int16)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


_RHO = None
_RHOPI = None
_PIPI = None
_SIGMA = None
_SIGMAPI = None


def _tables():
    global _RHO, _RHOPI, _PIPI, _SIGMA, _SIGMAPI
    if _RHO is None:
        _RHO = T.rho_tables()
        _RHOPI = T.rhopi_tables()
        _PIPI = T.pipi_tables()
        _SIGMA = T.sigma_tables()
        _SIGMAPI = T.sigmapi_tables()


def prop_diag(prop):
    """tau(t,t) gather (lib/contract.cpp:559-565). prop: [Nt,Nt,4,4,N,N]."""
    nt = prop.shape[0]
    return np.ascontiguousarray(prop[np.arange(nt), np.arange(nt)])


def rho_row(prop, mom5, tf):
    """One t_sink row of run_ContractRho. prop [Nt,Nt,4,4,N,N], mom5 [Nt,5,N,N].
    Returns (rows [Nt,768], corr [Nt,16,3])."""
    _tables()
    nt, n = prop.shape[0], prop.shape[-1]
    row = _c(prop[tf])
    mom5 = _c(mom5)
    spin, lprp, coef = _RHO
    rows = np.zeros((nt, 768), np.complex128)
    corr = np.zeros((nt, 16, 3), np.complex128)
    lib().oracle_rho_row(n, nt, tf, _p(row), _p(mom5), _p(_i16(spin)), _p(_i16(lprp)), _p(_f32(coef)),
                         _p(rows), _p(corr))
    return rows, corr


def rho(prop, mom5):
    """All t_sink rows: corr [Nt(tf), Nt(ti), 16, 3] (Contract_rho_rho h_elem)."""
    nt = prop.shape[0]
    return np.stack([rho_row(prop, mom5, tf)[1] for tf in range(nt)])


def rhopi_row(prop, mom_p1, mom_p2, mom5_p1p2, tf, idir):
    _tables()
    nt, n = prop.shape[0], prop.shape[-1]
    spin, ip, coef = _RHOPI
    row = _c(prop[tf])
    diag = _c(prop_diag(prop))
    rows = np.zeros((nt, 256), np.complex128)
    corr = np.zeros((nt, 4), np.complex128)
    lib().oracle_rhopi_row(n, nt, tf, idir, _p(row), _p(diag), _p(_c(mom_p1)), _p(_c(mom_p2)), _p(_c(mom5_p1p2)),
                           _p(_i16(spin)), _p(_i16(ip)), _p(_f32(coef)), _p(rows), _p(corr))
    return rows, corr


def rhopi(prop, mom_p1, mom_p2, mom5_p1p2, idir):
    nt = prop.shape[0]
    return np.stack([rhopi_row(prop, mom_p1, mom_p2, mom5_p1p2, tf, idir)[1] for tf in range(nt)])


def pipi_row(prop, p1, p2, p3, p4, tf, iso):
    """iso: 1 for I=1, 0 for I=0.  Returns dict of per-row arrays and corr [Nt,5]."""
    _tables()
    nt, n = prop.shape[0], prop.shape[-1]
    t = _PIPI
    row = _c(prop[tf])
    diag = _c(prop_diag(prop))
    sq = np.zeros((nt, 256), np.complex128)
    dt = np.zeros((nt, 256), np.complex128)
    dth = np.zeros((nt, 256), np.complex128)
    star = np.zeros((2, nt, 16), np.complex128)
    fish = np.zeros((2, nt, 16), np.complex128)
    corr = np.zeros((nt, 5), np.complex128)
    lib().oracle_pipi_row(n, nt, tf, iso, _p(row), _p(diag), _p(_c(p1)), _p(_c(p2)), _p(_c(p3)), _p(_c(p4)),
                          _p(_i16(t["spinIndices_pipi_square"])), _p(_f32(t["coef_pipi_square"])),
                          _p(_i16(t["spinIndices_pipi_doubleTriangle"])), _p(_f32(t["coef_pipi_doubleTriangle"])),
                          _p(_i16(t["spinIndices_pipi_doubleTriangle_hor"])), _p(_f32(t["coef_pipi_doubleTriangle_hor"])),
                          _p(sq), _p(dt), _p(dth), _p(star), _p(fish), _p(corr))
    return dict(square=sq, dtri=dt, dtri_hor=dth, star=star, fish=fish, corr=corr)


def pipi(prop, p1, p2, p3, p4, iso):
    nt = prop.shape[0]
    return np.stack([pipi_row(prop, p1, p2, p3, p4, tf, iso)["corr"] for tf in range(nt)])


def loop_unity(prop, mom, with_rows=False):
    """loop [Nt] (and, with_rows, the per-spin traces [Nt, 4])."""
    nt, n = prop.shape[0], prop.shape[-1]
    diag = _c(prop_diag(prop))
    rows = np.zeros((nt, 4), np.complex128)
    loop = np.zeros((nt,), np.complex128)
    lib().oracle_loop_unity(n, nt, _p(diag), _p(_c(mom)), _p(rows), _p(loop))
    return (loop, rows) if with_rows else loop


def sigma_row(prop, mom2, tf):
    _tables()
    nt, n = prop.shape[0], prop.shape[-1]
    spin, lprp, coef = _SIGMA
    rows = np.zeros((nt, 64), np.complex128)
    corr = np.zeros((nt, 4), np.complex128)
    lib().oracle_sigma_row(n, nt, tf, _p(_c(prop[tf])), _p(_c(mom2)), _p(_i16(spin)), _p(_i16(lprp)),
                           _p(_f32(coef)), _p(rows), _p(corr))
    return rows, corr


def sigma(prop, mom2):
    nt = prop.shape[0]
    return np.stack([sigma_row(prop, mom2, tf)[1] for tf in range(nt)])


def sigmapi_hor_fish(prop, p1, p2, with_rows=False):
    """hor_fish [Nt] (and, with_rows, the coefficient-weighted spin rows [Nt, 16])."""
    _tables()
    nt, n = prop.shape[0], prop.shape[-1]
    t = _SIGMAPI
    rows = np.zeros((nt, 16), np.complex128)
    corr = np.zeros((nt,), np.complex128)
    lib().oracle_sigmapi_hor_fish(n, nt, _p(_c(prop_diag(prop))), _p(_c(p1)), _p(_c(p2)),
                                  _p(_i16(t["spinIndices_sigmapi_hor_fish"])), _p(_f32(t["coef_sigmapi_hor_fish"])),
                                  _p(rows), _p(corr))
    return (corr, rows) if with_rows else corr


def sigmapi_triangle_row(prop, p1, p2, mom2_p1p2, tf):
    _tables()
    nt, n = prop.shape[0], prop.shape[-1]
    t = _SIGMAPI
    rows = np.zeros((nt, 128), np.complex128)
    corr = np.zeros((nt, 2), np.complex128)
    lib().oracle_sigmapi_triangle_row(n, nt, tf, _p(_c(prop[tf])), _p(_c(prop_diag(prop))), _p(_c(p1)), _p(_c(p2)),
                                      _p(_c(mom2_p1p2)), _p(_i16(t["spinIndices_sigmapi_triangle"])),
                                      _p(_i16(t["ip_sigmapi_triangle"])), _p(_f32(t["coef_sigmapi_triangle"])),
                                      _p(rows), _p(corr))
    return rows, corr


def sigmapi_triangle(prop, p1, p2, mom2_p1p2):
    nt = prop.shape[0]
    return np.stack([sigmapi_triangle_row(prop, p1, p2, mom2_p1p2, tf)[1] for tf in range(nt)])


def source_average(corr):
    """corr [Nt(tf), Nt(ti), ...] -> avg [Nt(dt), ...] (dumpData, lib/contract.cpp:621-631)."""
    corr = _c(corr)
    nt = corr.shape[0]
    tail = corr.shape[2:]
    nc = int(np.prod(tail)) if tail else 1
    avg = np.zeros((nt,) + tail, np.complex128)
    lib().oracle_source_average(nt, nc, _p(corr), _p(avg))
    return avg


def reorder_prop(file_payload, n, nt):
    """File order [s1][v1][t1][s2][v2][t2] -> [t1][t2][s1][s2][v1][v2] (lib/contract.cpp:524-534)."""
    src = _c(file_payload)
    out = np.zeros((nt, nt, 4, 4, n, n), np.complex128)
    lib().oracle_reorder_prop(n, nt, _p(src), _p(out))
    return out


def twosided_rows(prop_row, phi, rows, coef, tf, ti0, ti1):
    """Generic two-sided rows (oracle_twosided): prop_row [Nt,4,4,N,N] = tau(tf, .),
    phi [Nt,nphi,N,N], rows int16 [nrows,6], coef [nrows,2].  Returns [ti1-ti0, nrows]."""
    nt, n = phi.shape[0], phi.shape[-1]
    rows = _i16(rows)
    out = np.zeros((ti1 - ti0, rows.shape[0]), np.complex128)
    lib().oracle_twosided(n, nt, tf, ti0, ti1, _p(_c(prop_row)), _p(_c(phi)), phi.shape[1], rows.shape[0],
                          _p(rows), _p(_f32(coef)), _p(out))
    return out
