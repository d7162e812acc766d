"""GPU parity of the rho-type (two-sided) contractions against the oracle.

Every entry is gated on its own (tests/parity.py): plain FP64 engine <= 1e-12
relative, split engine <= 1e-9 relative, plus the FP64 rounding floor
2^-44 x (sum of the magnitudes of the entry's spin rows) for entries whose rows
cancel."""
import numpy as np
import pytest
import torch

from contractions_code_scattering_gb300 import api, synth
from oracle import pyoracle as O
from tests import parity as P

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-12, "split": 1e-9}


def _inputs(nt, n, seed, nops=5):
    prop = synth.make_prop(nt, n, seed=seed)
    rng = np.random.default_rng(seed + 1)
    mom = np.stack([synth.make_phi_random(nt, n, rng) for _ in range(nops)], axis=1)
    return prop, np.ascontiguousarray(mom)


def ref_rho(prop, mom5):
    """Oracle correlators [Nt, Nt, 16, 3] and their row magnitudes."""
    rc = [O.rho_row(prop, mom5, tf) for tf in range(prop.shape[0])]
    return np.stack([c for _, c in rc]), np.stack([P.rho_rows_abs(r) for r, _ in rc])


def ref_sigma(prop, mom2):
    rc = [O.sigma_row(prop, mom2, tf) for tf in range(prop.shape[0])]
    return np.stack([c for _, c in rc]), np.stack([P.sigma_rows_abs(r) for r, _ in rc])


@pytest.mark.parametrize("engine", ["fp64", "split"])
@pytest.mark.parametrize("nt,n", [(3, 16), (2, 37), (1, 1), (4, 8)])
def test_rho_matches_oracle(cuda, engine, nt, n):
    prop, mom5 = _inputs(nt, n, seed=100 + n)
    ref, ab = ref_rho(prop, mom5)
    got = api.run_contract_rho(torch.from_numpy(prop).to(cuda), torch.from_numpy(mom5).to(cuda), engine=engine)
    P.entrywise(got.cpu().numpy(), ref, TOL[engine], ab, "rho %s Nev=%d" % (engine, n))


@pytest.mark.parametrize("engine", ["fp64", "split"])
def test_rho_single_row_buffer(cuda, engine):
    """Row-by-row use, as Contract_rho_rho::contractRho drives run_ContractRho (lib/contract.cpp:602-605)."""
    nt, n = 4, 12
    prop, mom5 = _inputs(nt, n, seed=7)
    d_mom = torch.from_numpy(mom5).to(cuda)
    for tf in range(nt):
        row = torch.from_numpy(np.ascontiguousarray(prop[tf:tf + 1])).to(cuda)
        got = api.run_contract_rho(row, d_mom, engine=engine, tf_range=(tf, tf + 1))
        rows, ref = O.rho_row(prop, mom5, tf)
        P.entrywise(got[0].cpu().numpy(), ref, TOL[engine], P.rho_rows_abs(rows), "rho row %d" % tf)


@pytest.mark.parametrize("n", [9, 37, 100, 128])
def test_grouped_traces_match_per_trace_kernel(cuda, n):
    """The grouped closing-trace kernels (trace_rows candidate 9: blocks shared
    by a group of traces staged once in shared memory by bulk copies; 10 and 11:
    quad groups of at most 2 + 2 blocks loaded once into registers) give the
    oracle's rho and sigma at the split tolerance, and the per-trace kernel's
    values to float-float rounding: 1e-12 of each entry plus 2^-40 of its rows'
    magnitudes (each form's float-float trace sums carry ~2^-44 of them)."""
    nt = 2
    prop, mom5 = _inputs(nt, n, seed=300 + n)
    d_prop, d_mom = torch.from_numpy(prop).to(cuda), torch.from_numpy(mom5).to(cuda)
    want_rho, ab_rho = ref_rho(prop, mom5)
    want_sig, ab_sig = ref_sigma(prop, np.ascontiguousarray(mom5[:, :2]))
    got = {}
    try:
        for v in (9, 10, 11, 6):
            api.tune_force("trace_rows", v)
            got[v] = (api.run_contract_rho(d_prop, d_mom, engine="split").cpu().numpy(),
                      api.run_contract_sigma(d_prop, torch.from_numpy(np.ascontiguousarray(mom5[:, :2])).to(cuda),
                                             engine="split").cpu().numpy())
    finally:
        api.tune_force("trace_rows", -1)
    for v in (9, 10, 11):
        P.entrywise(got[v][0], want_rho, TOL["split"], ab_rho, "rho, trace form %d" % v)
        P.entrywise(got[v][1], want_sig, TOL["split"], ab_sig, "sigma, trace form %d" % v)
        P.entrywise(got[v][0], got[6][0], 1e-12, ab_rho, "rho, trace form %d vs 6" % v, floor=2.0 ** -40)
        P.entrywise(got[v][1], got[6][1], 1e-12, ab_sig, "sigma, trace form %d vs 6" % v, floor=2.0 ** -40)


@pytest.mark.parametrize("n", [9, 37, 100, 128])
def test_staged_slicer_writes_the_same_bytes(cuda, n):
    """The staged perambulator slicers (slice_tau form 1: one read of the operand
    through shared memory; form 2: the same with direct stores of the digits)
    write the same operand bytes as form 0, so the split engine's rho values are
    bitwise identical."""
    nt = 2
    prop, mom5 = _inputs(nt, n, seed=500 + n)
    d_prop, d_mom = torch.from_numpy(prop).to(cuda), torch.from_numpy(mom5).to(cuda)
    got = {}
    try:
        for form in (0, 1, 2):
            api.tune_force("slice_tau", form)
            got[form] = api.run_contract_rho(d_prop, d_mom, engine="split").cpu().numpy()
    finally:
        api.tune_force("slice_tau", -1)
    assert np.array_equal(got[0], got[1])
    assert np.array_equal(got[0], got[2])
    ref, ab = ref_rho(prop, mom5)
    P.entrywise(got[1], ref, TOL["split"], ab, "rho, staged slicer")


@pytest.mark.parametrize("shift", [60, 110])
def test_split_rho_beyond_float_float_range(cuda, shift):
    """Perambulators scaled by 2^-shift push the split engine's two-sided form
    out of its float-float range: at 2^-60 the products' traces would reach
    FP32's subnormals (their error scales fall below 2^-90), at 2^-110 the
    product scales themselves (below 2^-100, written as NaN).  Those entries are
    flagged and recomputed with FP64 range, so the results still meet the oracle."""
    nt, n = 2, 16
    prop, mom5 = _inputs(nt, n, seed=700 + shift)
    prop = prop * 2.0 ** -shift
    ref, ab = ref_rho(prop, mom5)
    got = api.run_contract_rho(torch.from_numpy(prop).to(cuda), torch.from_numpy(mom5).to(cuda), engine="split")
    got = got.cpu().numpy()
    assert np.isfinite(got).all()
    P.entrywise(got, ref, TOL["split"], ab, "rho scaled by 2^-%d" % shift)


@pytest.mark.parametrize("engine", ["fp64", "split"])
def test_sigma_matches_oracle(cuda, engine):
    nt, n = 3, 20
    prop, mom2 = _inputs(nt, n, seed=9, nops=2)
    ref, ab = ref_sigma(prop, mom2)
    got = api.run_contract_sigma(torch.from_numpy(prop).to(cuda), torch.from_numpy(mom2).to(cuda), engine=engine)
    P.entrywise(got.cpu().numpy(), ref, TOL[engine], ab, "sigma %s" % engine)


def test_rho_config0_shape(cuda):
    """CPU-sized rho two-point: Nev=32, Lt=16, p=0 Hermitian elementals."""
    nt, n = 16, 32
    prop = synth.make_prop(nt, n, seed=1000)
    phi0 = synth.make_phi_hermitian(nt, n, seed=1001)
    rng = np.random.default_rng(1002)
    mom5 = np.stack([phi0] + [synth.make_phi_random(nt, n, rng) for _ in range(4)], axis=1)
    mom5 = np.ascontiguousarray(mom5)
    ref, ab = ref_rho(prop, mom5)
    got = api.run_contract_rho(torch.from_numpy(prop).to(cuda), torch.from_numpy(mom5).to(cuda), engine="fp64")
    got = got.cpu().numpy()
    P.entrywise(got, ref, 1e-12, ab, "rho Nev=32 Lt=16")
    avg = api.source_average(torch.from_numpy(got).to(cuda)).cpu().numpy()
    # the average of Nt entries: its floor is the mean of their row magnitudes
    ab_avg = O.source_average(ab).real
    P.entrywise(avg, O.source_average(ref), 1e-12, ab_avg, "source average")


def test_source_average(cuda):
    rng = np.random.default_rng(0)
    corr = rng.normal(size=(6, 6, 4)) + 1j * rng.normal(size=(6, 6, 4))
    got = api.source_average(torch.from_numpy(corr).to(cuda), scale=-2.0).cpu().numpy()
    assert np.allclose(got, -2.0 * O.source_average(corr), rtol=1e-14, atol=1e-15)


def _refine(tol):
    from contractions_code_scattering_gb300._lib import check, lib
    check(lib().ctr_split_set_refine(tol))


def test_split_entrywise_refinement(cuda):
    """Per-entry accuracy of the split engine: with the refinement tolerance at
    1e-9 every entry meets 1e-9 relative to itself against the oracle; with a
    tolerance below the engine's error every entry is recomputed on the
    high-precision configuration (~2^-53 of the operand scales) and matches the
    oracle to 1e-11; with 0 nothing is recomputed."""
    from contractions_code_scattering_gb300._lib import lib
    nt, n = 4, 24
    prop, mom5 = _inputs(nt, n, seed=77)
    ref, ab = ref_rho(prop, mom5)
    args = (torch.from_numpy(prop).to(cuda), torch.from_numpy(mom5).to(cuda))
    try:
        _refine(1e-9)
        got = api.run_contract_rho(*args, engine="split").cpu().numpy()
        P.entrywise(got, ref, 1e-9, ab, "rho split, refinement at 1e-9")
        _refine(1e-15)
        got = api.run_contract_rho(*args, engine="split").cpu().numpy()
        assert lib().ctr_split_refined() == ref.size
        P.entrywise(got, ref, 1e-11, ab, "rho split, every entry recomputed")
        _refine(0.0)
        api.run_contract_rho(*args, engine="split")
        assert lib().ctr_split_refined() == 0
    finally:
        _refine(1e-9)
