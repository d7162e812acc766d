"""The C-ABI library loads without a GPU, exports every symbol include/*.h
declares, and rejects bad arguments with status codes (no compute calls)."""
import ctypes

import numpy as np
import pytest

from contractions_code_scattering_gb300 import _lib
from contractions_code_scattering_gb300._lib import lib


def test_library_loads_and_exports_all_declared_symbols():
    L = lib()
    names = _lib.exported_functions()
    assert "ctr_twosided" in names and "ctr_rho" in names
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_version_and_error_strings():
    L = lib()
    assert L.ctr_version() >= 100
    assert L.ctr_error_string(1) == b"invalid argument"


def _args(engine=0, nev=4, nt=2, tf0=0, tf1=2, ptr=16):
    p = ctypes.c_void_p(ptr)
    return [engine, nev, nt, tf0, tf1, p, p, p, None]


@pytest.mark.parametrize("kw", [dict(engine=7), dict(nev=0), dict(nt=0), dict(tf0=1, tf1=1), dict(tf1=3),
                                dict(ptr=8), dict(ptr=0)])
def test_rho_rejects_bad_arguments(kw):
    L = lib()
    rc = L.ctr_rho(*_args(**kw))
    assert rc == 1
    assert len(L.ctr_last_error()) > 0


def test_twosided_rejects_bad_rows():
    L = lib()
    p = ctypes.c_void_p(16)
    rows = np.array([[0, 0, 0, 4, 0, 0]], np.int16)  # spin index 4 out of range
    coef = np.ones((1, 2), np.float32)
    oi = np.zeros(1, np.int32)
    rc = L.ctr_twosided(0, 4, 2, 0, 2, p, p, 1, 1, rows.ctypes.data_as(ctypes.c_void_p),
                        coef.ctypes.data_as(ctypes.c_void_p), oi.ctypes.data_as(ctypes.c_void_p), 1, p, None)
    assert rc == 1
    assert b"spin index" in L.ctr_last_error()


def test_momentum_set_calls_reject_bad_arguments():
    """The set calls check their sizes, isospin, pointers and elemental indices before
    touching a device (no GPU needed)."""
    L = lib()
    fake = ctypes.c_void_p(1 << 20)  # aligned stand-in: rejected before any use
    sets = (ctypes.c_int32 * 4)(0, 1, 0, 5)
    rc = L.ctr_pipi_sets(0, 8, 4, 0, 4, 0, fake, fake, fake, 3, 1, ctypes.cast(sets, ctypes.c_void_p), fake, None)
    assert rc == 1 and b"not in [0,3)" in L.ctr_last_error()
    assert L.ctr_pipi_sets(0, 8, 4, 0, 4, 2, fake, fake, fake, 3, 1, ctypes.cast(sets, ctypes.c_void_p), fake,
                           None) == 1
    assert L.ctr_pipi_sets(0, 8, 4, 0, 4, 0, None, fake, fake, 3, 1, ctypes.cast(sets, ctypes.c_void_p), fake,
                           None) == 1
    pairs = (ctypes.c_int32 * 2)(0, 7)
    rc = L.ctr_rhopi_sigmapi_sets(0, 8, 4, 0, 4, fake, fake, fake, 3, fake, fake, 1,
                                  ctypes.cast(pairs, ctypes.c_void_p), fake, fake, fake, None)
    assert rc == 1 and b"not in [0,3)" in L.ctr_last_error()
    assert L.ctr_rhopi_sigmapi_sets(0, 8, 4, 2, 1, fake, fake, fake, 3, fake, fake, 1,
                                    ctypes.cast(pairs, ctypes.c_void_p), fake, fake, fake, None) == 1
