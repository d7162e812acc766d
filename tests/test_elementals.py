"""Elementals from Laplacian eigenvectors (include/ctr.h: ctr_elementals; the
reference drivers' loops tests/compute_rho.cpp:116-223).

CPU: the numpy restatement (oracle/elementals.py) against identities that pin
it independently of any implementation: orthonormal eigenvectors give the unit
matrix at p = 0; Phi(-p) = Phi(p)^dagger for the plain and smeared operators
and -Phi(p)^dagger for the commutators; every operator is invariant under a
lattice gauge transformation (which checks the covariant derivative); with
unit links the derivative is the symmetric difference.
GPU: ctr_elementals against the restatement (1e-12 of the largest entry), on a
non-cubic lattice with negative momenta, at tile edges 32 and 50."""
import numpy as np
import pytest

from contractions_code_scattering_gb300 import synth
from oracle import elementals as E

MOMS = [(0, 0, 0), (1, 0, 0), (-1, 0, 0), (0, 1, -1), (0, -1, 1), (1, 1, 1)]


def _inputs(nt, nev, nx, ny, nz, seed):
    return synth.make_eigvecs(nt, nev, nx, ny, nz, seed), synth.make_links(nt, nx, ny, nz, seed + 1)


def test_plain_elemental_at_zero_momentum_is_the_identity():
    V, U = _inputs(2, 5, 3, 4, 2, 10)
    out = E.elementals(V, [(0, 0, 0)], U)
    assert np.abs(out[0, 0] - np.eye(5)).max() < 1e-13


def test_momentum_reversal():
    V, U = _inputs(2, 5, 4, 3, 5, 20)
    out = E.elementals(V, MOMS, U)
    pairs = [(1, 2), (3, 4)]
    for a, b in pairs:
        for op in (0, 1):
            assert np.abs(out[b, op] - out[a, op].conj().swapaxes(-1, -2)).max() < 1e-13
        for op in (2, 3, 4):
            assert np.abs(out[b, op] + out[a, op].conj().swapaxes(-1, -2)).max() < 1e-13


def test_gauge_covariance():
    nt, nev, nx, ny, nz = 1, 4, 3, 4, 5
    V, U = _inputs(nt, nev, nx, ny, nz, 30)
    W = synth.make_links(nt, nx, ny, nz, 99)[:, :, :, :, 0]  # Omega(x) in SU(3), [nt, nz, ny, nx, 3, 3]
    V2 = np.einsum("tzyxab,tczyxb->tczyxa", W, V)
    U2 = np.empty_like(U)
    for j, ax in ((0, 3), (1, 2), (2, 1)):
        Wp = np.roll(W, -1, axis=ax)  # Omega(x + j)
        U2[:, :, :, :, j] = np.einsum("tzyxab,tzyxbc,tzyxdc->tzyxad", W, U[:, :, :, :, j], Wp.conj())
    a = E.elementals(V, MOMS[:3], U)
    b = E.elementals(V2, MOMS[:3], U2)
    assert np.abs(a - b).max() < 1e-12 * np.abs(a).max()


def test_unit_links_give_the_symmetric_difference():
    nt, nev, nx, ny, nz = 1, 3, 4, 3, 5
    V = synth.make_eigvecs(nt, nev, nx, ny, nz, 40)
    U = np.zeros((nt, nz, ny, nx, 3, 3, 3), np.complex128)
    U[..., :, :] = np.eye(3)
    for j, ax in ((0, 3), (1, 2), (2, 1)):
        d = E.covderiv(V[0], U[0], j)
        assert np.abs(d - (np.roll(V[0], -1, axis=ax) - np.roll(V[0], 1, axis=ax))).max() < 1e-15


@pytest.mark.gpu
@pytest.mark.parametrize("nev", [7, 50])
def test_gpu_elementals_match_the_restatement(cuda, nev):
    import torch
    from contractions_code_scattering_gb300 import api
    nt, nx, ny, nz = 2, 4, 3, 5
    V, U = _inputs(nt, nev, nx, ny, nz, 50 + nev)
    ref = E.elementals(V, MOMS, U)
    got = api.elementals(torch.from_numpy(V).to(cuda), MOMS, links=torch.from_numpy(U).to(cuda)).cpu().numpy()
    assert got.shape == ref.shape
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
    plain = api.elementals(torch.from_numpy(V).to(cuda), MOMS).cpu().numpy()
    assert plain.shape == (len(MOMS), 1, nt, nev, nev)
    assert np.abs(plain[:, 0] - ref[:, 0]).max() <= 1e-12 * np.abs(ref[:, 0]).max()


@pytest.mark.gpu
def test_gpu_elementals_feed_the_rho_contraction(cuda):
    """The drivers' path: elementals built on the GPU, in the [op][t][r][c] layout
    calculateRho takes, contracted on both engines against the oracle's rho on
    the same elementals."""
    import torch
    from contractions_code_scattering_gb300 import api
    from oracle import pyoracle as O
    nt, nev, nx, ny, nz = 3, 12, 4, 4, 4
    V, U = _inputs(nt, nev, nx, ny, nz, 70)
    phi = api.elementals(torch.from_numpy(V).to(cuda), [(1, 0, 0)], links=torch.from_numpy(U).to(cuda))[0]
    mom5 = phi.permute(1, 0, 2, 3).contiguous()  # [op][t] -> [t][op], as calculateRho re-lays it out
    prop = synth.make_prop(nt, nev, seed=71)
    ref = O.rho(prop, mom5.cpu().numpy())
    for engine, tol in (("fp64", 1e-12), ("split", 1e-9)):
        got = api.run_contract_rho(torch.from_numpy(prop).to(cuda), mom5, engine=engine).cpu().numpy()
        assert np.abs(got - ref).max() <= tol * np.abs(ref).max(), engine
