"""Host-level API without a GPU: the momentum-list reader (lib/catchOpts.cpp:108-233)
and the perambulator-file checks of readPropH (lib/contract.cpp:91-160)."""
import ctypes
import os
import struct

import numpy as np
import pytest

from contractions_code_scattering_gb300._lib import lib


def _mom(path, nmom, momcomb):
    L = lib()
    L.ctr_read_momenta.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    p = np.zeros((4, 3, momcomb), np.int32)
    rc = L.ctr_read_momenta(str(path).encode(), nmom, momcomb, p.ctypes.data_as(ctypes.c_void_p))
    return rc, p


def test_momenta_four(tmp_path):
    f = tmp_path / "mom_pipi.dat"
    f.write_text("1 0 0\t-1 0 0\t1 0 0\t-1 0 0\n")  # the reference's tests/mom_pipi.dat line
    rc, p = _mom(f, 4, 1)
    assert rc == 0
    assert p[:, :, 0].tolist() == [[1, 0, 0], [-1, 0, 0], [1, 0, 0], [-1, 0, 0]]


def test_momenta_two_derives_total(tmp_path):
    f = tmp_path / "mom_sigmapi.dat"
    f.write_text("+1 0 0\t-1 0 0\n+2 0 0\t-2 0 0\n")
    rc, p = _mom(f, 2, 2)
    assert rc == 0
    assert p[0, :, 1].tolist() == [2, 0, 0] and p[1, :, 1].tolist() == [-2, 0, 0]
    assert p[2, :, 0].tolist() == [0, 0, 0]  # p3 = p1 + p2


def test_momenta_one_without_final_newline(tmp_path):
    f = tmp_path / "mom_rho.dat"
    f.write_text("0 0 1")
    rc, p = _mom(f, 1, 1)
    assert rc == 0 and p[0, :, 0].tolist() == [0, 0, 1]


@pytest.mark.parametrize("text,nmom,nc", [("1 0 0\n", 1, 2), ("1 0 0 2\n", 1, 1), ("1 0 0\n", 3, 1), ("1 0 0\n", 1, 0)])
def test_momenta_rejects(tmp_path, text, nmom, nc):
    f = tmp_path / "bad.dat"
    f.write_text(text)
    rc, _ = _mom(f, nmom, nc)
    assert rc != 0
    assert len(lib().ctr_last_error()) > 0


def _prop_file(path, nt, nvec, payload_elems):
    with open(path, "wb") as fh:
        fh.write(b"cfg0001".ljust(100, b"\0"))
        fh.write(struct.pack("<II", nt, nvec))
        fh.write(np.zeros(payload_elems, np.complex128).tobytes())


def _read(path, nev, nt):
    L = lib()
    L.ctr_read_prop.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    out = np.zeros((nt, nt, 4, 4, nev, nev), np.complex128)
    return L.ctr_read_prop(str(path).encode(), nev, nt, 0, out.ctypes.data_as(ctypes.c_void_p))


def test_readprop_missing_file(tmp_path):
    assert _read(tmp_path / "nope.bin", 2, 2) == 6
    assert b"cannot find file" in lib().ctr_last_error()


def test_readprop_size_mismatch(tmp_path):
    f = tmp_path / "p.bin"
    _prop_file(f, 2, 3, 2 * 2 * 16 * 9)
    assert _read(f, 4, 2) == 6 and b"NeV" in lib().ctr_last_error()
    assert _read(f, 3, 3) == 6 and b"Nt" in lib().ctr_last_error()


def test_readprop_truncated(tmp_path):
    f = tmp_path / "p.bin"
    _prop_file(f, 2, 3, 2 * 2 * 16 * 9 - 5)
    assert _read(f, 3, 2) == 6 and b"expected size" in lib().ctr_last_error()


def test_cpp_api_symbols_exported():
    """The reference's C++ entry points (include/interface.h, include/contract.h) are in libctr.so."""
    import subprocess
    from contractions_code_scattering_gb300 import _build
    out = subprocess.run(["nm", "-DC", _build.LIB], capture_output=True, text=True).stdout
    for sym in ("calculateRho(contract::contractInfo", "calculateRhoPi(int, contract::contractInfo",
                "calculatePiPi(contract::contractInfo", "calculateSigma(contract::contractInfo",
                "calculateSigmaPi(contract::contractInfo", "contract::initContract(", "contract::destroyContract()",
                "contract::readPropH("):
        assert sym in out, sym
