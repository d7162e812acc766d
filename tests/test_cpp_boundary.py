"""The reference's C++ boundary (include/contract.h): the nine run_Contract* and
five run_CopyConstants* launchers on texture objects, and the Base / LapH_prop /
Mom_* / Contract_* classes with H_elem(), driven by tests/cpp/reference_driver.cpp
the way the reference's own classes and drivers use them (texture objects over
linear device memory, the perambulator staged row by row).

CPU: the driver compiles against include/contract.h and links against
libctr.so, i.e. every C++ entry point it calls is exported.  GPU: on the golden
inputs (Nev = 100, Nt = 2) every launcher's and every class's results match the
reference's own kernels per entry (tests/parity.py; 1e-12 for DOUBLE), and the
float instantiations match to single-precision rounding."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from tests import parity as P

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "reference_driver.cpp")
GOLD = os.path.join(ROOT, "tests", "golden", "ref_outputs.npz")


def cuda_home():
    for cand in (os.environ.get("CUDA_HOME"), os.environ.get("CUDA_PATH")):
        if cand and os.path.isdir(os.path.join(cand, "include")):
            return cand
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    return "/usr/local/cuda"


def compile_cpp(src, exe):
    """g++ against include/ and the CUDA headers, linked with libctr.so and cudart."""
    from contractions_code_scattering_gb300 import _build, lib
    lib()  # builds libctr.so if it is missing
    pkg = os.path.dirname(_build.LIB)
    cuda = cuda_home()
    libdir = next((d for d in (os.path.join(cuda, "lib64"), os.path.join(cuda, "lib"))
                   if os.path.isdir(d)), os.path.join(cuda, "lib64"))
    cmd = ["g++", "-std=c++17", "-O1", "-o", str(exe), str(src), "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(cuda, "include"), "-L", pkg, "-lctr", "-L", libdir, "-lcudart",
           "-Wl,-rpath," + pkg, "-Wl,-rpath," + libdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, "compile failed:\n%s\n%s" % (" ".join(cmd), r.stderr)
    return exe


@pytest.mark.skipif(shutil.which("g++") is None, reason="no C++ compiler")
def test_reference_driver_compiles_and_links(tmp_path):
    compile_cpp(SRC, tmp_path / "driver")
    assert os.path.exists(tmp_path / "driver")


def _load(path, shape, dtype=np.float64):
    a = np.fromfile(path, dtype=dtype)
    return a.view(np.complex128 if dtype == np.float64 else np.complex64).reshape(shape)


@pytest.mark.gpu
@pytest.mark.skipif(shutil.which("g++") is None, reason="no C++ compiler")
@pytest.mark.skipif(not os.path.exists(GOLD), reason="reference golden vectors not recorded")
def test_launchers_and_classes_match_reference_kernels(cuda, tmp_path):
    from tests.golden.make_ref_fixtures import NEV, NT, inputs
    gold = dict(np.load(GOLD))
    d = inputs()
    for k in ("prop", "mom5", "mom2", "p1", "p2", "p3", "p4"):
        np.ascontiguousarray(d[k], dtype=np.complex128).tofile(tmp_path / (k + ".bin"))
    exe = compile_cpp(SRC, tmp_path / "driver")
    r = subprocess.run([str(exe), str(tmp_path), str(NEV), str(NT)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    nt = NT
    ab = {
        "rho": P.rho_rows_abs(gold["rho_rows"]),
        "sigma": P.sigma_rows_abs(gold["sigma_rows"]),
        "triangle": P.triangle_rows_abs(gold["sigmapi_triangle_rows"]),
        "hor_fish": P.sum_rows_abs(gold["sigmapi_hor_fish_rows"]),
        "loop": P.sum_rows_abs(gold["loop_rows"]),
    }
    for idir in range(3):
        ab["rhopi%d" % idir] = P.rhopi_rows_abs(gold["rhopi%d_rows" % idir])
    for iso in (0, 1):
        g = {k: gold["pipi_I%d_%s" % (iso, k)] for k in ("square", "dtri", "dtri_hor")}
        g["star"] = np.moveaxis(gold["pipi_I%d_star" % iso], 2, 0)
        g["fish"] = np.moveaxis(gold["pipi_I%d_fish" % iso], 2, 0)
        ab["pipi%d" % iso] = P.pipi_rows_abs(g, iso)

    def check(name, shape, ref, key, tol=1e-12, dtype=np.float64, floor=P.FLOOR):
        got = _load(tmp_path / name, shape, dtype).astype(np.complex128)
        P.entrywise(got, ref, tol, ab[key], name, floor=floor)

    # launchers on texture objects
    check("launch_rho.bin", (nt, nt, 16, 3), gold["rho_corr"], "rho")
    for idir in range(3):
        check("launch_rhopi%d.bin" % idir, (nt, nt, 4), gold["rhopi%d_corr" % idir], "rhopi%d" % idir)
    check("launch_pipi0.bin", (nt, nt, 5), gold["pipi_I0_corr"], "pipi0")
    check("launch_pipi1.bin", (nt, nt, 5), gold["pipi_I1_corr"], "pipi1")
    check("launch_sigma.bin", (nt, nt, 4), gold["sigma_corr"], "sigma")
    check("launch_triangle.bin", (nt, nt, 2), gold["sigmapi_triangle"], "triangle")
    check("launch_hor_fish.bin", (nt,), gold["sigmapi_hor_fish"], "hor_fish")
    check("launch_loop.bin", (nt,), gold["loop"], "loop")
    # classes: H_elem() after contract*()
    check("class_rho.bin", (nt, nt, 16, 3), gold["rho_corr"], "rho")
    check("class_rhopi1.bin", (nt, nt, 4), gold["rhopi1_corr"], "rhopi1")
    check("class_pipi0.bin", (nt, nt, 5), gold["pipi_I0_corr"], "pipi0")
    check("class_pipi1.bin", (nt, nt, 5), gold["pipi_I1_corr"], "pipi1")
    check("class_sigma.bin", (nt, nt, 4), gold["sigma_corr"], "sigma")
    sp = _load(tmp_path / "class_sigmapi.bin", (nt + nt * nt * 2,))
    P.entrywise(sp[:nt], gold["sigmapi_hor_fish"], 1e-12, ab["hor_fish"], "class hor fish")
    P.entrywise(sp[nt:].reshape(nt, nt, 2), gold["sigmapi_triangle"], 1e-12, ab["triangle"], "class triangle")
    check("class_loop.bin", (nt,), gold["loop"], "loop")
    # float instantiations: inputs rounded to float (2^-24), results narrowed to float
    check("single_rho.bin", (nt, nt, 16, 3), gold["rho_corr"], "rho", tol=1e-5, dtype=np.float32, floor=2.0 ** -20)
    check("single_pipi0.bin", (nt, nt, 5), gold["pipi_I0_corr"], "pipi0", tol=1e-5, dtype=np.float32,
          floor=2.0 ** -20)
    # the classes' text dumps (the reference's dumpData formats)
    txt = open(tmp_path / "class_pipi.txt").read()
    for label in ("Square:", "DoubleTriangle:", "Star:", "Fish:", "DoubleTriangle_Hor:"):
        assert label in txt
    assert "twop:" in open(tmp_path / "class_sigma.txt").read()
    s = open(tmp_path / "class_sigmapi.txt").read()
    assert "fish_hor:" in s and "triangle:" in s
    assert len(open(tmp_path / "class_rho.txt").read().strip().split("\n")) == 16 * nt
