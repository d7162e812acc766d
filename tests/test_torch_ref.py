"""The plain-PyTorch restatement used as the reference gradient of the profile
adjoint (oracle/torch_ref.py) against the C oracle's correlators (CPU)."""
import numpy as np
import pytest
import torch

from contractions_code_scattering_gb300 import synth
from oracle import pyoracle as O
from oracle import torch_ref as R


def _inputs(nt=4, n=6, seed=3):
    prop = synth.make_prop(nt, n, seed=seed)
    rng = np.random.default_rng(seed + 1)
    mom5 = np.stack([synth.make_phi_random(nt, n, rng) for _ in range(5)], axis=1)
    P = [synth.make_phi_random(nt, n, rng) for _ in range(4)]
    f = np.exp(-np.sort(rng.uniform(size=n)) / 0.3)
    return prop, mom5, P, f


def test_rho_pair_matches_oracle():
    prop, mom5, _, f = _inputs()
    ref = O.rho(prop, f[:, None] * mom5 * f[None, :]).reshape(4, 4, 48)
    got = R.rho_pair(torch.from_numpy(prop), R.profiled(torch.from_numpy(f), torch.from_numpy(mom5)), 2, 1,
                     list(range(48)))
    assert np.abs(got.numpy() - ref[2, 1]).max() <= 1e-13 * np.abs(ref).max()


@pytest.mark.parametrize("iso", [0, 1])
def test_pipi_pair_matches_oracle(iso):
    prop, _, P, f = _inputs()
    Pp = [f[:, None] * p * f[None, :] for p in P]
    ref = O.pipi(prop, *Pp, iso)
    got = R.pipi_pair(torch.from_numpy(prop), tuple(torch.from_numpy(p) for p in Pp), 3, 1, iso)
    assert np.abs(got.numpy() - ref[3, 1]).max() <= 1e-13 * np.abs(ref[3, 1]).max()
