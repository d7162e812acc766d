"""GPU parity of the chain diagrams (rho->pipi, pipi I=1/I=0, loop-unity,
sigma->pipi) on the plain FP64 engine: against the reference's own kernel
outputs (golden vectors, Nev=100) and against the oracle at other sizes.
Tolerance 1e-12 relative to the largest |entry| of each compared array."""
import os

import numpy as np
import pytest
import torch

from contractions_code_scattering_gb300 import api, synth
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-12
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_outputs.npz")


def _close(got, ref, tol=TOL):
    got = got.cpu().numpy() if hasattr(got, "cpu") else got
    err = np.abs(got - ref).max() / np.abs(ref).max()
    assert err <= tol, "error %.3e relative to max |entry| (tolerance %.1e)" % (err, tol)


def _dev(a, cuda):
    return torch.from_numpy(np.ascontiguousarray(a)).to(cuda)


@pytest.fixture(scope="module")
def small(cuda):
    nt, n = 3, 12
    prop = synth.make_prop(nt, n, seed=300)
    rng = np.random.default_rng(301)
    ph = [synth.make_phi_random(nt, n, rng) for _ in range(4)]
    mom5 = np.ascontiguousarray(np.stack([synth.make_phi_random(nt, n, rng) for _ in range(5)], axis=1))
    mom2 = np.ascontiguousarray(mom5[:, 1:3])
    d = dict(prop=prop, ph=ph, mom5=mom5, mom2=mom2)
    t = {k: _dev(v, cuda) for k, v in (("prop", prop), ("mom5", mom5), ("mom2", mom2))}
    t["ph"] = [_dev(p, cuda) for p in ph]
    t["diag"] = api.prop_diag(t["prop"])
    return d, t


@pytest.mark.parametrize("iso", [1, 0])
def test_pipi_vs_oracle(small, iso):
    d, t = small
    ref = O.pipi(d["prop"], *d["ph"], iso)
    got = api.run_contract_pipi(t["prop"], t["diag"], *t["ph"], iso)
    _close(got, ref)


@pytest.mark.parametrize("idir", [0, 1, 2])
def test_rhopi_vs_oracle(small, idir):
    d, t = small
    ref = O.rhopi(d["prop"], d["ph"][0], d["ph"][1], d["mom5"], idir)
    got = api.run_contract_rhopi(t["prop"], t["diag"], t["ph"][0], t["ph"][1], t["mom5"], idir)
    _close(got, ref)


def test_sigmapi_and_loop_vs_oracle(small):
    d, t = small
    hf, tri = api.run_contract_sigmapi(t["prop"], t["diag"], t["ph"][0], t["ph"][1], t["mom2"])
    _close(hf, O.sigmapi_hor_fish(d["prop"], d["ph"][0], d["ph"][1]))
    _close(tri, O.sigmapi_triangle(d["prop"], d["ph"][0], d["ph"][1], d["mom2"]))
    _close(api.run_contract_loop_unity(t["diag"], t["ph"][2]), O.loop_unity(d["prop"], d["ph"][2]))


def test_row_range(small):
    """A single t_sink row held on the device, as the reference stages it."""
    d, t = small
    ref = O.pipi(d["prop"], *d["ph"], 0)
    for tf in range(d["prop"].shape[0]):
        row = t["prop"][tf:tf + 1].contiguous()
        got = api.run_contract_pipi(row, t["diag"], *t["ph"], 0, tf_range=(tf, tf + 1))
        _close(got[0], ref[tf])


@pytest.mark.skipif(not os.path.exists(GOLD), reason="reference golden vectors not recorded")
def test_chains_vs_reference_kernels(cuda):
    from tests.golden.make_ref_fixtures import inputs
    gold = dict(np.load(GOLD))
    d = inputs()
    prop = _dev(d["prop"], cuda)
    diag = api.prop_diag(prop)
    p = [_dev(d[k], cuda) for k in ("p1", "p2", "p3", "p4")]
    mom5, mom2 = _dev(d["mom5"], cuda), _dev(d["mom2"], cuda)
    for idir in range(3):
        _close(api.run_contract_rhopi(prop, diag, p[0], p[1], mom5, idir), gold["rhopi%d_corr" % idir])
    for iso in (0, 1):
        _close(api.run_contract_pipi(prop, diag, *p, iso), gold["pipi_I%d_corr" % iso])
    hf, tri = api.run_contract_sigmapi(prop, diag, p[0], p[1], mom2)
    _close(hf, gold["sigmapi_hor_fish"])
    _close(tri, gold["sigmapi_triangle"])
    _close(api.run_contract_loop_unity(diag, p[0]), gold["loop"])
