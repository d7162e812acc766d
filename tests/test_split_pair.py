"""The CTA-pair form of the split-precision GEMM (clusters of two CTAs issuing
M = 256 tcgen05 MMAs with cta_group::2, each CTA loading its own 128 rows of
the left operand and half of the right one).

Every launch is pinned to the pair form through the "split_gemm.form" knob,
including the one-M-tile calls, where the odd CTA of each pair computes
padding rows only.  The products must meet the same bounds as the single-CTA
form (tests/test_split_gemm.py), the exact levels must be bit-identical to
the exact emulation, and the rho and pi pi correlators must agree with the
single-CTA form and with the oracle entry by entry."""
import numpy as np
import pytest
import torch

from contractions_code_scattering_gb300 import api, synth
from oracle import pyoracle as O
from tests import parity as P
from tests import test_split_gemm as S

pytestmark = pytest.mark.gpu


@pytest.fixture
def pair_form(cuda):
    api.tune_force("split_gemm.form", 1)
    yield
    api.tune_force("split_gemm.form", -1)


@pytest.mark.parametrize("n", [100, 16, 37, 128, 1])
def test_pair_split_gemm_random(cuda, pair_form, n):
    rng = np.random.default_rng(100 + n)
    S._check(S._rand(rng, (3, n, n)), S._rand(rng, (3, n, n)), cuda)


def test_pair_split_gemm_identity_is_exact(cuda, pair_form):
    S.test_split_gemm_identity_is_exact(cuda)


def test_pair_split_gemm_row_and_column_scales(cuda, pair_form):
    S.test_split_gemm_row_and_column_scales(cuda)


def test_pair_split_gemm_zero_and_sparse(cuda, pair_form):
    S.test_split_gemm_zero_and_sparse(cuda)


def test_pair_accumulation_levels(cuda, pair_form):
    S.test_tensor_core_accumulation_levels(cuda)


def _rho_inputs(nt, nev, seed):
    prop = synth.make_prop(nt, nev, seed=seed)
    rng = np.random.default_rng(seed + 1)
    mom5 = np.ascontiguousarray(np.stack([synth.make_phi_random(nt, nev, rng) for _ in range(5)], axis=1))
    return prop, mom5


def test_pair_rho_matches_single_and_oracle(cuda):
    nt, nev = 4, 100
    prop, mom5 = _rho_inputs(nt, nev, 71)
    d_prop, d_mom = torch.from_numpy(prop).to(cuda), torch.from_numpy(mom5).to(cuda)
    got = {}
    try:
        for form in (0, 1):
            api.tune_force("split_gemm.form", form)
            got[form] = api.run_contract_rho(d_prop, d_mom, engine="split").cpu().numpy()
    finally:
        api.tune_force("split_gemm.form", -1)
    same = np.array_equal(got[0], got[1])
    print("pair form bitwise equal to the single-CTA form: %s" % same)
    scale = np.abs(got[0]).max()
    assert np.abs(got[1] - got[0]).max() <= 1e-13 * scale
    for tf in range(nt):
        rows, ref = O.rho_row(prop, mom5, tf)
        P.entrywise(got[1][tf], ref, 1e-9, P.rho_rows_abs(rows), "t_sink %d" % tf)


def test_pair_pipi_sets_match_single(cuda):
    nt, nev = 3, 100
    prop = synth.make_prop(nt, nev, seed=81)
    rng = np.random.default_rng(82)
    phi = np.ascontiguousarray(np.stack([synth.make_phi_random(nt, nev, rng) for _ in range(4)], axis=1))
    d_prop = torch.from_numpy(prop).to(cuda)
    d_phi = torch.from_numpy(phi).to(cuda)
    diag = api.prop_diag(d_prop)
    sets = [(0, 1, 2, 3), (2, 3, 0, 1)]
    got = {}
    try:
        for form in (0, 1):
            api.tune_force("split_gemm.form", form)
            got[form] = api.run_contract_pipi_sets(d_prop, diag, d_phi, sets, 0, engine="split").cpu().numpy()
    finally:
        api.tune_force("split_gemm.form", -1)
    print("pair form bitwise equal to the single-CTA form: %s" % np.array_equal(got[0], got[1]))
    assert np.abs(got[1] - got[0]).max() <= 1e-13 * np.abs(got[0]).max()
