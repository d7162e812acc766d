"""GPU tests of the reference-compatible API layer: readPropH's file format,
the calculate* output files (the reference's dumpData text blocks) against the
oracle, and a C++ program written against include/interface.h linked to libctr.so.
Text holds 7 significant digits ("%+e"), so values compare to 1e-6 relative to
the largest |value| of each block."""
import ctypes
import os
import re
import shutil
import struct
import subprocess

import numpy as np
import pytest

from contractions_code_scattering_gb300 import _build, synth
from contractions_code_scattering_gb300._lib import check, lib
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
vp, ci = ctypes.c_void_p, ctypes.c_int


def _p(a):
    return a.ctypes.data_as(vp)


def _setup():
    L = lib()
    L.ctr_contract_init.argtypes = [ci, ci, ci]
    L.ctr_read_prop.argtypes = [ctypes.c_char_p, ci, ci, ci, vp]
    L.ctr_calculate_rho.argtypes = [ci, ci, vp, vp, ci, ctypes.c_char_p]
    L.ctr_calculate_rhopi.argtypes = [ci, ci, ci, vp, vp, vp, vp, ci, ctypes.c_char_p]
    L.ctr_calculate_pipi.argtypes = [ci, ci, vp, vp, vp, vp, vp, ci, ctypes.c_char_p, ci]
    L.ctr_calculate_sigma.argtypes = [ci, ci, vp, vp, ci, ctypes.c_char_p]
    L.ctr_calculate_sigmapi.argtypes = [ci, ci, vp, vp, vp, vp, ci, ctypes.c_char_p]
    return L


@pytest.fixture
def session(cuda):
    L = _setup()
    yield L
    L.ctr_contract_destroy()


def _write_prop_file(path, prop):
    nt, n = prop.shape[0], prop.shape[-1]
    file_order = np.ascontiguousarray(np.transpose(prop, (2, 4, 0, 3, 5, 1)))  # [s1][v1][t1][s2][v2][t2]
    with open(path, "wb") as fh:
        fh.write(b"synthetic".ljust(100, b"\0"))
        fh.write(struct.pack("<II", nt, n))
        fh.write(file_order.astype(np.complex128).tobytes())


def _numbers(line):
    return [float(x) for x in re.findall(r"[-+]\d\.\d+e[-+]\d+", line)]


def _close(got, ref, tol=1e-6):
    got, ref = np.asarray(got), np.asarray(ref)
    assert got.shape == ref.shape
    err = np.abs(got - ref).max() / np.abs(ref).max()
    assert err <= tol, "error %.3e" % err


def test_read_prop_roundtrip(session, tmp_path):
    prop = synth.make_prop(3, 7, seed=5)
    f = tmp_path / "prop.bin"
    _write_prop_file(f, prop)
    out = np.zeros_like(prop)
    check(session.ctr_read_prop(str(f).encode(), 7, 3, 0, _p(out)))
    assert np.array_equal(out, prop)
    out32 = np.zeros(prop.shape, np.complex64)
    check(session.ctr_read_prop(str(f).encode(), 7, 3, 1, _p(out32)))
    assert np.array_equal(out32, prop.astype(np.complex64))


def test_calculate_rho_file(session, tmp_path):
    nt, n = 4, 10
    check(session.ctr_contract_init(n, nt, 0))
    prop = synth.make_prop(nt, n, seed=8)
    rng = np.random.default_rng(9)
    mom = np.ascontiguousarray(np.stack([synth.make_phi_random(nt, n, rng) for _ in range(5)]))  # [5][Nt][N][N]
    f = tmp_path / "rho.dat"
    check(session.ctr_calculate_rho(n, nt, _p(prop), _p(mom), 0, str(f).encode()))
    lines = [l for l in open(f).read().split("\n") if l.strip()]
    assert len(lines) == 16 * nt
    avg = O.source_average(O.rho(prop, np.ascontiguousarray(np.transpose(mom, (1, 0, 2, 3)))))
    got = np.zeros((nt, 16, 3), np.complex128)
    for l in lines:
        iop, it = [int(x) for x in l.split()[:2]]
        v = _numbers(l)
        got[it, iop] = [complex(v[0], v[1]), complex(v[2], v[3]), complex(v[4], v[5])]
    _close(got, avg)


def test_calculate_pipi_sigma_sigmapi_rhopi_files(session, tmp_path):
    nt, n = 3, 8
    check(session.ctr_contract_init(n, nt, 0))
    prop = synth.make_prop(nt, n, seed=21)
    rng = np.random.default_rng(22)
    p = [np.ascontiguousarray(synth.make_phi_random(nt, n, rng)) for _ in range(4)]
    f = tmp_path / "pipi.dat"
    check(session.ctr_calculate_pipi(n, nt, _p(prop), *[_p(x) for x in p], 0, str(f).encode(), 0))
    avg = O.source_average(O.pipi(prop, *p, 0))
    blocks = [b for b in open(f).read().split("\n\n") if b.strip()]
    assert [b.split(":")[0] for b in blocks] == ["Square", "DoubleTriangle", "Star", "Fish", "DoubleTriangle_Hor"]
    for k, b in enumerate(blocks):
        vals = [_numbers(l) for l in b.strip().split("\n")]
        _close([complex(*v) for v in vals], avg[:, k])
    # sigma: four loop blocks, then twop = -C
    mom4 = np.ascontiguousarray(np.stack([synth.make_phi_random(nt, n, rng) for _ in range(4)]))
    f = tmp_path / "sigma.dat"
    check(session.ctr_calculate_sigma(n, nt, _p(prop), _p(mom4), 0, str(f).encode()))
    blocks = [b for b in open(f).read().split("\n\n") if b.strip()]
    assert len(blocks) == 5
    for i in range(4):
        vals = [_numbers(l) for l in blocks[i].strip().split("\n")]
        _close([complex(*v) for v in vals], O.loop_unity(prop, mom4[i]))
    ref = -O.source_average(O.sigma(prop, np.ascontiguousarray(np.stack([mom4[1], mom4[3]], axis=1))))
    vals = {}
    for l in blocks[4].strip().split("\n"):
        iop, it = [int(x) for x in l.split()[1:3]]
        vals[(iop, it)] = complex(*_numbers(l))
    _close([[vals[(iop, it)] for iop in range(4)] for it in range(nt)], ref)
    # sigma -> pi pi: two loops, fish_hor, triangle * (-2/sqrt(6))
    p12 = np.ascontiguousarray(np.stack([synth.make_phi_random(nt, n, rng) for _ in range(2)]))
    f = tmp_path / "sigmapi.dat"
    check(session.ctr_calculate_sigmapi(n, nt, _p(prop), _p(p[0]), _p(p[1]), _p(p12), 0, str(f).encode()))
    blocks = [b for b in open(f).read().split("\n\n") if b.strip()]
    assert [b.split(":")[0] for b in blocks] == ["loop", "loop", "fish_hor", "triangle"]
    _close([complex(*_numbers(l)) for l in blocks[2].strip().split("\n")], O.sigmapi_hor_fish(prop, p[0], p[1]))
    ref = -2 / np.sqrt(6) * O.source_average(O.sigmapi_triangle(prop, p[0], p[1], np.ascontiguousarray(np.transpose(p12, (1, 0, 2, 3)))))
    got = np.zeros((nt, 2), np.complex128)
    for l in blocks[3].strip().split("\n"):
        iop, it = [int(x) for x in l.split()[1:3]]
        got[it, iop] = complex(*_numbers(l))
    _close(got, ref)
    # rho -> pi pi with idir = 2; the label column is the option parser's i_dir (0 here)
    mom5 = np.ascontiguousarray(np.stack([synth.make_phi_random(nt, n, rng) for _ in range(5)]))
    f = tmp_path / "rhopi.dat"
    check(session.ctr_calculate_rhopi(2, n, nt, _p(prop), _p(p[0]), _p(p[1]), _p(mom5), 0, str(f).encode()))
    ref = 2 * O.source_average(O.rhopi(prop, p[0], p[1], np.ascontiguousarray(np.transpose(mom5, (1, 0, 2, 3))), 2))
    got = np.zeros((nt, 4), np.complex128)
    for l in open(f).read().strip().split("\n"):
        iop, idl, it = [int(x) for x in l.split()[:3]]
        assert idl == 0
        got[it, iop] = complex(*_numbers(l))
    _close(got, ref)


CPP = r"""
#include <cstdio>
#include <cstdlib>
#include <vector>
#include "interface.h"
int main(int argc, char** argv) {
  contract::contractInfo info;
  info.NeV = atoi(argv[1]); info.Nt = atoi(argv[2]); info.dev = 0; info.PropH_fileName = argv[3];
  contract::initContract(info);
  void* prop = contract::readPropH(info.PropH_fileName, contract::DOUBLE);
  size_t n = (size_t)5 * info.Nt * info.NeV * info.NeV * 2;
  std::vector<double> mom(n);
  FILE* f = fopen(argv[4], "rb");
  if (fread(mom.data(), sizeof(double), n, f) != n) return 2;
  fclose(f);
  calculateRho(info, prop, mom.data(), contract::DOUBLE, argv[5]);
  free(prop);
  contract::destroyContract();
  return 0;
}
"""


@pytest.mark.skipif(shutil.which("g++") is None, reason="no C++ compiler")
def test_cpp_driver_against_interface_h(cuda, tmp_path):
    """A reference-style driver (initContract, readPropH, calculateRho, destroyContract)
    compiled against include/interface.h and linked with libctr.so."""
    nt, n = 3, 9
    prop = synth.make_prop(nt, n, seed=31)
    rng = np.random.default_rng(32)
    mom = np.ascontiguousarray(np.stack([synth.make_phi_random(nt, n, rng) for _ in range(5)]))
    _write_prop_file(tmp_path / "prop.bin", prop)
    mom.tofile(tmp_path / "mom.bin")
    src = tmp_path / "driver.cpp"
    src.write_text(CPP)
    exe = tmp_path / "driver"
    pkg = os.path.dirname(_build.LIB)
    from tests.test_cpp_boundary import cuda_home
    subprocess.check_call(["g++", "-O1", "-o", str(exe), str(src), "-I", os.path.join(ROOT, "include"),
                           "-I", os.path.join(cuda_home(), "include"), "-L", pkg, "-lctr", "-Wl,-rpath," + pkg])
    out = tmp_path / "rho.dat"
    r = subprocess.run([str(exe), str(n), str(nt), str(tmp_path / "prop.bin"), str(tmp_path / "mom.bin"), str(out)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "Elapsed time is" in r.stdout
    avg = O.source_average(O.rho(prop, np.ascontiguousarray(np.transpose(mom, (1, 0, 2, 3)))))
    got = np.zeros((nt, 16, 3), np.complex128)
    for l in open(out).read().strip().split("\n"):
        iop, it = [int(x) for x in l.split()[:2]]
        v = _numbers(l)
        got[it, iop] = [complex(v[0], v[1]), complex(v[2], v[3]), complex(v[4], v[5])]
    _close(got, avg)
    # the driver's errors terminate the process as the reference's ABORT does
    r = subprocess.run([str(exe), str(n + 1), str(nt), str(tmp_path / "prop.bin"), str(tmp_path / "mom.bin"), str(out)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode != 0 and "NeV" in r.stderr
