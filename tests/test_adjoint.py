"""Distillation-profile adjoint (include/ctr.h: ctr_chain_adjoint, ctr_rho_profile_vjp,
ctr_pipi_profile_vjp) against
  * the oracle's correlators with the profile applied to the elementals (forward),
  * torch.autograd through a plain-PyTorch FP64 restatement (reference gradient),
  * FP64 central finite differences with h = 1e-6 (tolerance 1e-6 of max|grad|)."""
import numpy as np
import pytest
import torch

from contractions_code_scattering_gb300 import CtrError, adjoint, api, synth
from oracle import pyoracle as O
from oracle import torch_ref as R

pytestmark = pytest.mark.gpu


def _data(nt, n, seed):
    prop = synth.make_prop(nt, n, seed=seed)
    rng = np.random.default_rng(seed + 1)
    mom5 = np.stack([synth.make_phi_hermitian(nt, n, seed + 2)] +
                    [synth.make_phi_random(nt, n, rng) for _ in range(4)], axis=1)
    p1 = synth.make_phi_random(nt, n, rng)
    P = [p1, p1.conj().transpose(0, 2, 1).copy(), p1.copy(), p1.conj().transpose(0, 2, 1).copy()]
    f = adjoint.default_profile(n, seed=seed + 3)
    return prop, np.ascontiguousarray(mom5), [np.ascontiguousarray(p) for p in P], f


def _dev(a, cuda):
    return torch.from_numpy(np.ascontiguousarray(a)).to(cuda)


def _prof(f, phi):
    return f[:, None] * phi * f[None, :]


def test_rho_forward_matches_oracle(cuda):
    nt, n = 4, 12
    prop, mom5, _, f = _data(nt, n, 10)
    w = torch.ones((nt, nt, 48), dtype=torch.complex128, device=cuda)
    corr, _ = api.rho_profile_vjp(_dev(prop, cuda), _dev(mom5, cuda), _dev(f, cuda), w, grad=False)
    ref = O.rho(prop, _prof(f, mom5)).reshape(nt, nt, 48)
    err = np.abs(corr.cpu().numpy() - ref).max() / np.abs(ref).max()
    assert err < 1e-12, err


@pytest.mark.parametrize("iso", [0, 1])
def test_pipi_forward_matches_oracle(cuda, iso):
    nt, n = 4, 10
    prop, _, P, f = _data(nt, n, 20)
    w = torch.zeros((nt, nt, 5), dtype=torch.complex128, device=cuda)
    w[1, 3] = 1.0
    w[2, 2] = 1.0
    corr, _ = api.pipi_profile_vjp(_dev(prop, cuda), *[_dev(p, cuda) for p in P], _dev(f, cuda), w, iso, grad=False)
    ref = O.pipi(prop, *[_prof(f, p) for p in P], iso)
    got = corr.cpu().numpy()
    for tf, ti in ((1, 3), (2, 2)):
        err = np.abs(got[tf, ti] - ref[tf, ti]).max() / np.abs(ref[tf, ti]).max()
        assert err < 1e-12, (tf, ti, err)
    assert np.all(got[0] == 0)


def _objective_inputs(cuda, nt=6, n=10, seed=30):
    prop, mom5, P, f = _data(nt, n, seed)
    return prop, mom5, P, f, dict(rho_ts=(1, 3), pipi_dt=2, isospin=0)


@pytest.mark.parametrize("engine,tol", [("fp64", 1e-10), ("split", 1e-8)])
def test_gradient_matches_torch_reference(cuda, engine, tol):
    prop, mom5, P, f, kw = _objective_inputs(cuda)
    fd = torch.tensor(f, device=cuda, requires_grad=True)
    L = adjoint.objective(fd, _dev(prop, cuda), _dev(mom5, cuda), tuple(_dev(p, cuda) for p in P), engine=engine,
                          **kw)
    L.backward()
    fr = torch.tensor(f, requires_grad=True)
    Lr = R.objective(fr, torch.from_numpy(prop), torch.from_numpy(mom5), tuple(torch.from_numpy(p) for p in P), **kw)
    Lr.backward()
    assert abs(L.item() - Lr.item()) <= tol * abs(Lr.item())
    g, gr = fd.grad.cpu().numpy(), fr.grad.numpy()
    err = np.abs(g - gr).max() / np.abs(gr).max()
    print("%s: objective %.6e, grad rel err vs torch autograd %.3e" % (engine, Lr.item(), err))
    assert err < tol, err


def test_gradient_matches_finite_differences(cuda):
    prop, mom5, P, f, kw = _objective_inputs(cuda, seed=40)
    args = (_dev(prop, cuda), _dev(mom5, cuda), tuple(_dev(p, cuda) for p in P))
    fd = torch.tensor(f, device=cuda, requires_grad=True)
    adjoint.objective(fd, *args, **kw).backward()
    g = fd.grad.cpu().numpy()
    h = 1e-6
    worst = 0.0
    for k in (0, 3, 7, 9):
        fp, fm = f.copy(), f.copy()
        fp[k] += h
        fm[k] -= h
        with torch.no_grad():
            lp = adjoint.objective(torch.tensor(fp, device=cuda), *args, **kw).item()
            lm = adjoint.objective(torch.tensor(fm, device=cuda), *args, **kw).item()
        worst = max(worst, abs((lp - lm) / (2 * h) - g[k]))
    print("max |FD - adjoint| / max|grad| = %.3e" % (worst / np.abs(g).max()))
    assert worst <= 1e-6 * np.abs(g).max()


def test_generic_chains_match_autograd(cuda):
    """Random chains of 2..8 factors with conjugate transposes against torch.autograd."""
    nt, n, nphi = 3, 9, 3
    rng = np.random.default_rng(50)
    prop = synth.make_prop(nt, n, seed=51)
    phi = np.stack([synth.make_phi_random(nt, n, rng) for _ in range(nphi)], axis=1)
    f = adjoint.default_profile(n, seed=52)
    chains = []
    for c in range(40):
        L = int(rng.integers(2, 9))
        ch = []
        for j in range(L):
            if rng.random() < 0.5:
                ch.append((api.FACTOR_PHI, int(rng.integers(2)), int(rng.integers(nt)), int(rng.integers(nphi)), 0, 0))
            else:
                ch.append((api.FACTOR_TAU, int(rng.integers(2)), int(rng.integers(nt)), int(rng.integers(nt)),
                           int(rng.integers(4)), int(rng.integers(4))))
        chains.append(ch)
    w = rng.normal(size=40) + 1j * rng.normal(size=40)
    vals, g = api.chain_adjoint(_dev(prop, cuda), _dev(phi, cuda), _dev(f, cuda), chains, w)
    vs, gs = api.chain_adjoint(_dev(prop, cuda), _dev(phi, cuda), _dev(f, cuda), chains, w, engine="split")
    ft = torch.tensor(f, requires_grad=True)
    pt, ph = torch.from_numpy(prop), R.profiled(ft, torch.from_numpy(phi))
    total = 0
    ref_vals = []
    for ch, wc in zip(chains, w):
        m = None
        for kind, dag, a, b, s1, s2 in ch:
            x = pt[a, b, s1, s2] if kind == api.FACTOR_TAU else ph[a, b]
            if dag:
                x = x.conj().transpose(0, 1)
            m = x if m is None else m @ x
        v = torch.diagonal(m).sum()
        ref_vals.append(v.detach().numpy())
        total = total + (complex(wc) * v).real
    total.backward()
    rv = np.array(ref_vals)
    assert np.abs(vals.cpu().numpy() - rv).max() <= 1e-12 * np.abs(rv).max()
    err = np.abs(g.cpu().numpy() - ft.grad.numpy()).max() / np.abs(ft.grad.numpy()).max()
    assert err < 1e-12, err
    # tensor-core chain products: chains of up to 8 factors spanning several decades
    assert np.abs(vs.cpu().numpy() - rv).max() <= 1e-9 * np.abs(rv).max()
    err = np.abs(gs.cpu().numpy() - ft.grad.numpy()).max() / np.abs(ft.grad.numpy()).max()
    assert err < 1e-9, err


def test_zero_profile_entry_is_rejected(cuda):
    nt, n = 2, 6
    prop, mom5, _, f = _data(nt, n, 60)
    f[2] = 0.0
    w = torch.ones((nt, nt, 48), dtype=torch.complex128, device=cuda)
    with pytest.raises(CtrError):
        api.rho_profile_vjp(_dev(prop, cuda), _dev(mom5, cuda), _dev(f, cuda), w)
