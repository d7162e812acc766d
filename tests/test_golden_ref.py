"""Golden vectors recorded from the reference's own kernels (see
tests/golden/make_ref_fixtures.py): the oracle must reproduce them (this pins
the oracle), and the GPU engines must reproduce them through the C ABI.

Tolerance: 1e-12 relative to the largest |value| of each compared array for
FP64 paths (the reference kernels and the oracle differ only in summation order
and FMA contraction), 1e-9 for the split engine."""
import os

import numpy as np
import pytest

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


def _close(got, ref, tol):
    err = np.abs(np.asarray(got) - ref).max() / np.abs(ref).max()
    assert err <= tol, "error %.3e relative to max |value| (tolerance %.1e)" % (err, tol)


def test_oracle_rho(gold, data):
    from oracle import pyoracle as O
    for tf in range(NT):
        rows, corr = O.rho_row(data["prop"], data["mom5"], tf)
        _close(rows, gold["rho_rows"][tf], 1e-12)
        _close(corr, gold["rho_corr"][tf], 1e-12)


def test_oracle_sigma_and_loop(gold, data):
    from oracle import pyoracle as O
    for tf in range(NT):
        rows, corr = O.sigma_row(data["prop"], data["mom2"], tf)
        _close(rows, gold["sigma_rows"][tf], 1e-12)
        _close(corr, gold["sigma_corr"][tf], 1e-12)
    _close(O.loop_unity(data["prop"], data["p1"]), gold["loop"], 1e-12)


def test_oracle_rhopi(gold, data):
    from oracle import pyoracle as O
    for idir in range(3):
        rows, corr = O.rhopi_row(data["prop"], data["p1"], data["p2"], data["mom5"], 0, idir)
        _close(rows, gold["rhopi%d_rows" % idir][0], 1e-12)
        _close(corr, gold["rhopi%d_corr" % idir][0], 1e-12)


def test_oracle_pipi(gold, data):
    """t_sink = 0 row, isospin 0 (which evaluates every pi-pi diagram); the I=1
    weights are checked on the same rows."""
    from oracle import pyoracle as O
    d = O.pipi_row(data["prop"], data["p1"], data["p2"], data["p3"], data["p4"], 0, iso=0)
    for k in ("square", "dtri", "dtri_hor"):
        _close(d[k], gold["pipi_I0_%s" % k][0], 1e-12)
    _close(np.transpose(d["star"], (1, 0, 2)), gold["pipi_I0_star"][0], 1e-12)
    _close(np.transpose(d["fish"], (1, 0, 2)), gold["pipi_I0_fish"][0], 1e-12)
    _close(d["corr"], gold["pipi_I0_corr"][0], 1e-12)
    i1 = gold["pipi_I1_corr"][0]
    sq, dt = d["square"].sum(-1), d["dtri"].sum(-1)
    _close(-2 * sq, i1[:, 0], 1e-12)
    _close(2 * dt, i1[:, 1], 1e-12)
    _close(-d["corr"][:, 2], i1[:, 2], 1e-12)
    _close(d["corr"][:, 3], i1[:, 3], 1e-12)
    assert np.all(i1[:, 4] == 0)


def test_oracle_sigmapi(gold, data):
    from oracle import pyoracle as O
    _close(O.sigmapi_hor_fish(data["prop"], data["p1"], data["p2"]), gold["sigmapi_hor_fish"], 1e-12)
    rows, corr = O.sigmapi_triangle_row(data["prop"], data["p1"], data["p2"], data["mom2"], 0)
    _close(rows, gold["sigmapi_triangle_rows"][0], 1e-12)
    _close(corr, gold["sigmapi_triangle"][0], 1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("engine,tol", [("fp64", 1e-12), ("split", 1e-9)])
def test_engine_rho_and_sigma(cuda, gold, data, engine, tol):
    import torch
    from contractions_code_scattering_gb300 import api
    prop = torch.from_numpy(data["prop"]).to(cuda)
    got = api.run_contract_rho(prop, torch.from_numpy(data["mom5"]).to(cuda), engine=engine)
    _close(got.cpu().numpy(), gold["rho_corr"], tol)
    got = api.run_contract_sigma(prop, torch.from_numpy(data["mom2"]).to(cuda), engine=engine)
    api.sync()
    _close(got.cpu().numpy(), gold["sigma_corr"], tol)
