"""Golden vectors recorded from the reference's own kernels (see
tests/golden/make_ref_fixtures.py): the oracle must reproduce them (this pins
the oracle), and the GPU engines must reproduce them through the C ABI.

Every entry is gated on its own (tests/parity.py): 1e-12 relative for FP64
paths (the reference kernels and the oracle differ only in summation order and
FMA contraction), 1e-9 for the split engine, plus the FP64 rounding floor of
entries whose spin rows cancel.  Spin rows are compared per row at 1e-12
relative to each row's own magnitude."""
import os

import numpy as np
import pytest

from tests import parity as P
from tests.golden.make_ref_fixtures import NT, inputs

HERE = os.path.dirname(os.path.abspath(__file__))
PATH = os.path.join(HERE, "golden", "ref_outputs.npz")

pytestmark = pytest.mark.skipif(not os.path.exists(PATH), reason="reference golden vectors not recorded")


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(PATH))


@pytest.fixture(scope="module")
def data():
    return inputs()


def _rows(got, ref, tol=1e-12):
    """Spin rows, each against its own magnitude."""
    P.entrywise(np.asarray(got), ref, tol, None, "rows")


def test_oracle_rho(gold, data):
    from oracle import pyoracle as O
    for tf in range(NT):
        rows, corr = O.rho_row(data["prop"], data["mom5"], tf)
        _rows(rows, gold["rho_rows"][tf])
        P.entrywise(corr, gold["rho_corr"][tf], 1e-12, P.rho_rows_abs(gold["rho_rows"][tf]), "rho")


def test_oracle_sigma_and_loop(gold, data):
    from oracle import pyoracle as O
    for tf in range(NT):
        rows, corr = O.sigma_row(data["prop"], data["mom2"], tf)
        _rows(rows, gold["sigma_rows"][tf])
        P.entrywise(corr, gold["sigma_corr"][tf], 1e-12, P.sigma_rows_abs(gold["sigma_rows"][tf]), "sigma")
    loop, rows = O.loop_unity(data["prop"], data["p1"], with_rows=True)
    _rows(rows, gold["loop_rows"])
    P.entrywise(loop, gold["loop"], 1e-12, P.sum_rows_abs(gold["loop_rows"]), "loop")


def test_oracle_rhopi(gold, data):
    from oracle import pyoracle as O
    for idir in range(3):
        rows, corr = O.rhopi_row(data["prop"], data["p1"], data["p2"], data["mom5"], 0, idir)
        _rows(rows, gold["rhopi%d_rows" % idir][0])
        P.entrywise(corr, gold["rhopi%d_corr" % idir][0], 1e-12, P.rhopi_rows_abs(gold["rhopi%d_rows" % idir][0]),
                    "rhopi")


def test_oracle_pipi(gold, data):
    """t_sink = 0 row, isospin 0 (which evaluates every pi-pi diagram); the I=1
    weights are checked on the same rows."""
    from oracle import pyoracle as O
    d = O.pipi_row(data["prop"], data["p1"], data["p2"], data["p3"], data["p4"], 0, iso=0)
    for k in ("square", "dtri", "dtri_hor"):
        _rows(d[k], gold["pipi_I0_%s" % k][0])
    _rows(np.transpose(d["star"], (1, 0, 2)), gold["pipi_I0_star"][0])
    _rows(np.transpose(d["fish"], (1, 0, 2)), gold["pipi_I0_fish"][0])
    ab0 = P.pipi_rows_abs(d, 0)
    P.entrywise(d["corr"], gold["pipi_I0_corr"][0], 1e-12, ab0, "pipi I0")
    i1 = gold["pipi_I1_corr"][0]
    ab1 = P.pipi_rows_abs(d, 1)
    sq, dt = d["square"].sum(-1), d["dtri"].sum(-1)
    P.entrywise(-2 * sq, i1[:, 0], 1e-12, ab1[:, 0], "pipi I1 square")
    P.entrywise(2 * dt, i1[:, 1], 1e-12, ab1[:, 1], "pipi I1 double triangle")
    P.entrywise(-d["corr"][:, 2], i1[:, 2], 1e-12, ab1[:, 2], "pipi I1 star")
    P.entrywise(d["corr"][:, 3], i1[:, 3], 1e-12, ab1[:, 3], "pipi I1 fish")
    assert np.all(i1[:, 4] == 0)


def test_oracle_sigmapi(gold, data):
    from oracle import pyoracle as O
    hf, hrows = O.sigmapi_hor_fish(data["prop"], data["p1"], data["p2"], with_rows=True)
    _rows(hrows, gold["sigmapi_hor_fish_rows"])
    P.entrywise(hf, gold["sigmapi_hor_fish"], 1e-12, P.sum_rows_abs(gold["sigmapi_hor_fish_rows"]), "hor fish")
    rows, corr = O.sigmapi_triangle_row(data["prop"], data["p1"], data["p2"], data["mom2"], 0)
    _rows(rows, gold["sigmapi_triangle_rows"][0])
    P.entrywise(corr, gold["sigmapi_triangle"][0], 1e-12, P.triangle_rows_abs(gold["sigmapi_triangle_rows"][0]),
                "triangle")


@pytest.mark.gpu
@pytest.mark.parametrize("engine,tol", [("fp64", 1e-12), ("split", 1e-9)])
def test_engine_rho_and_sigma(cuda, gold, data, engine, tol):
    import torch
    from contractions_code_scattering_gb300 import api
    prop = torch.from_numpy(data["prop"]).to(cuda)
    got = api.run_contract_rho(prop, torch.from_numpy(data["mom5"]).to(cuda), engine=engine)
    P.entrywise(got.cpu().numpy(), gold["rho_corr"], tol, P.rho_rows_abs(gold["rho_rows"]), "rho %s" % engine)
    got = api.run_contract_sigma(prop, torch.from_numpy(data["mom2"]).to(cuda), engine=engine)
    api.sync()
    P.entrywise(got.cpu().numpy(), gold["sigma_corr"], tol, P.sigma_rows_abs(gold["sigma_rows"]), "sigma %s" % engine)
