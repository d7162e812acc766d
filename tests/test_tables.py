"""Diagram tables: the oracle's generator and the library's generator both
reproduce the reference's shipped include/constants_*.h token for token."""
import json
import os

import numpy as np
import pytest

from oracle import tables as T
from tests.golden.make_table_fixtures import digest, parse_header

HERE = os.path.dirname(os.path.abspath(__file__))
REF = json.load(open(os.path.join(HERE, "golden", "tables_ref.json")))


def test_fixture_lists_every_table():
    assert len(REF) == 20


@pytest.mark.parametrize("name", sorted(REF))
def test_oracle_generator_matches_reference_digest(name):
    mine = T.all_tables()[name]
    assert list(mine.shape) == REF[name]["shape"]
    assert digest(T.format_values(mine)) == REF[name]["sha256"]


def test_library_tables_match_oracle():
    from contractions_code_scattering_gb300 import api
    lib_t = api.tables()
    ora = T.all_tables()
    assert set(lib_t) == set(ora)
    for k in ora:
        a, b = lib_t[k], ora[k]
        assert a.shape == b.shape, k
        if b.dtype.kind == "f":
            # float32 in the library, as in the reference's __constant__ copies; signs of zero included
            assert T.format_values(a.astype(np.float64)) == T.format_values(b), k
            assert np.array_equal(np.signbit(a), np.signbit(b.astype(np.float32))), k
        else:
            assert np.array_equal(a, b), k
        assert digest(T.format_values(a)) == REF[k]["sha256"], k


def test_gamma5_is_chiral_diag():
    g1, g2, g3, g4, g5 = T.gamma_matrices()
    assert np.allclose(g5, np.diag([1, 1, -1, -1]))
    for g in (g1, g2, g3, g4):
        assert np.allclose(g @ g, np.eye(4))
        assert np.allclose(g, g.conj().T)
        assert np.allclose(g @ g5, -g5 @ g)


REF_ROOT = os.environ.get("CTR_REFERENCE_ROOT", "")


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF_ROOT, "include")) if REF_ROOT else True,
                    reason="reference tree not given (CTR_REFERENCE_ROOT)")
def test_direct_against_reference_headers():
    import glob
    for f in glob.glob(os.path.join(REF_ROOT, "include", "constants_*.h")):
        for name, t in parse_header(f).items():
            assert T.format_values(T.all_tables()[name]) == t["tokens"], name


HEADERS = ["constants_rho.h", "constants_rhopi.h", "constants_pipi.h", "constants_sigma.h", "constants_sigmapi.h"]
INCLUDE = os.path.join(os.path.dirname(HERE), "include")


def test_shipped_headers_are_the_generated_ones():
    """include/constants_*.h are exactly what the generator renders from the
    library's own tables (contractions_code_scattering_gb300/constants_headers.py)."""
    from contractions_code_scattering_gb300 import constants_headers as CH
    files = CH.render(CH.library_tables())
    for f in HEADERS + ["constants.h"]:
        assert open(os.path.join(INCLUDE, f)).read() == files[f], f


def test_shipped_headers_match_reference_digests():
    """Every array of the shipped headers has the reference header's name, type,
    shape and token digest (tests/golden/tables_ref.json)."""
    seen = set()
    for f in HEADERS:
        for name, t in parse_header(os.path.join(INCLUDE, f)).items():
            assert REF[name]["header"] == "include/" + f, name
            assert t["shape"] == REF[name]["shape"] and t["type"] == REF[name]["type"], name
            assert digest(t["tokens"]) == REF[name]["sha256"], name
            seen.add(name)
    assert seen == set(REF)


@pytest.mark.skipif(__import__("shutil").which("g++") is None, reason="no C++ compiler")
def test_shipped_headers_compile(tmp_path):
    src = tmp_path / "t.cpp"
    src.write_text('#include <constants.h>\n#include <cstdio>\nint main() { printf("%d %+3.2f %d\\n", '
                   'spinIndices_rho[1][3], coef_rho[8][1], ip_sigmapi_triangle[127]); return 0; }\n')
    import subprocess
    subprocess.check_call(["g++", "-o", str(tmp_path / "t"), str(src), "-I", INCLUDE])
    out = subprocess.check_output([str(tmp_path / "t")], text=True).split()
    tabs = T.all_tables()
    assert out == ["%d" % tabs["spinIndices_rho"][1][3], "%+3.2f" % tabs["coef_rho"][8][1],
                   "%d" % tabs["ip_sigmapi_triangle"][127]]
