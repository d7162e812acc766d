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


# ---- split engine: every block product of the chains on the tensor cores
SPLIT_TOL = 1e-10


@pytest.mark.parametrize("iso", [1, 0])
def test_pipi_split_vs_oracle(small, iso):
    d, t = small
    ref = O.pipi(d["prop"], *d["ph"], iso)
    got = api.run_contract_pipi(t["prop"], t["diag"], *t["ph"], iso, engine="split")
    _close(got, ref, SPLIT_TOL)


@pytest.mark.parametrize("idir", [0, 2])
def test_rhopi_split_vs_oracle(small, idir):
    d, t = small
    ref = O.rhopi(d["prop"], d["ph"][0], d["ph"][1], d["mom5"], idir)
    got = api.run_contract_rhopi(t["prop"], t["diag"], t["ph"][0], t["ph"][1], t["mom5"], idir, engine="split")
    _close(got, ref, SPLIT_TOL)


def test_sigmapi_split_vs_oracle(small):
    d, t = small
    hf, tri = api.run_contract_sigmapi(t["prop"], t["diag"], t["ph"][0], t["ph"][1], t["mom2"], engine="split")
    _close(hf, O.sigmapi_hor_fish(d["prop"], d["ph"][0], d["ph"][1]), SPLIT_TOL)
    _close(tri, O.sigmapi_triangle(d["prop"], d["ph"][0], d["ph"][1], d["mom2"]), SPLIT_TOL)


@pytest.mark.skipif(not os.path.exists(GOLD), reason="reference golden vectors not recorded")
def test_split_chains_vs_reference_kernels(cuda):
    """Nev = 100: four-term block products (K = 400, leading digit halved) on the split engine."""
    from tests.golden.make_ref_fixtures import inputs
    gold = dict(np.load(GOLD))
    d = inputs()
    prop = _dev(d["prop"], cuda)
    diag = api.prop_diag(prop)
    p = [_dev(d[k], cuda) for k in ("p1", "p2", "p3", "p4")]
    mom5, mom2 = _dev(d["mom5"], cuda), _dev(d["mom2"], cuda)
    _close(api.run_contract_rhopi(prop, diag, p[0], p[1], mom5, 1, engine="split"), gold["rhopi1_corr"], SPLIT_TOL)
    for iso in (0, 1):
        _close(api.run_contract_pipi(prop, diag, *p, iso, engine="split"), gold["pipi_I%d_corr" % iso], SPLIT_TOL)
    hf, tri = api.run_contract_sigmapi(prop, diag, p[0], p[1], mom2, engine="split")
    _close(hf, gold["sigmapi_hor_fish"], SPLIT_TOL)
    _close(tri, gold["sigmapi_triangle"], SPLIT_TOL)


def test_block_product_tasks_split_vs_fp64(cuda):
    """The task form directly (include/ctr.h: ctr_zgemm_tasks): four-term
    gamma_5-weighted block products with conjugate transposes, as in X = M1 G M2^dagger,
    on both engines against numpy (rows of M1 scaled over 8 decades)."""
    n = 100
    rng = np.random.default_rng(5)
    M1 = (rng.normal(size=(16, n, n)) + 1j * rng.normal(size=(16, n, n))) * np.exp(-rng.uniform(0, 18, (16, n, 1)))
    M2 = rng.normal(size=(16, n, n)) + 1j * rng.normal(size=(16, n, n))
    g5 = [1.0, 1.0, -1.0, -1.0]
    ref = np.zeros((16, n, n), np.complex128)
    tasks = []
    for a in range(4):
        for b in range(4):
            for k in range(4):
                ref[a * 4 + b] += g5[k] * M1[a * 4 + k] @ M2[b * 4 + k].conj().T
            tasks.append(([a * 4 + k for k in range(4)], [b * 4 + k for k in range(4)], a * 4 + b))
    x, y = _dev(M1, cuda), _dev(M2, cuda)
    for engine, tol in (("fp64", 1e-14), ("split", 1e-12)):
        out = api.zgemm_tasks(x, y, tasks, weights=g5, b_dagger=True, engine=engine)
        api.sync()
        got = out.cpu().numpy()
        # entry error against the scale of its row of M1 and the columns of M2
        scale = np.abs(M1).reshape(4, 4, n, n).max(axis=(1, 3))[:, None, :, None] * np.abs(M2).max() * 4 * n
        err = (np.abs(got - ref).reshape(4, 4, n, n) / scale).max()
        assert err <= tol, (engine, err)


def _refine(tol):
    from contractions_code_scattering_gb300._lib import check, lib
    check(lib().ctr_split_set_refine(tol))


def test_split_chain_refinement(small):
    """Per-entry accuracy of the split chain engine: with the tolerance below the
    engine's error every pair is recomputed by the FP64 engine (results equal to
    FP64 rounding); with 1e-9 every entry meets 1e-9 relative to itself."""
    from contractions_code_scattering_gb300._lib import lib
    d, t = small
    nt = d["prop"].shape[0]
    ref_pp = O.pipi(d["prop"], *d["ph"], 0)
    ref_rp = O.rhopi(d["prop"], d["ph"][0], d["ph"][1], d["mom5"], 1)
    ref_hf = O.sigmapi_hor_fish(d["prop"], d["ph"][0], d["ph"][1])
    ref_tr = O.sigmapi_triangle(d["prop"], d["ph"][0], d["ph"][1], d["mom2"])

    def rel(got, ref):
        got = got.cpu().numpy()
        return (np.abs(got - ref) / np.abs(ref)).max()
    try:
        _refine(1e-15)
        assert rel(api.run_contract_pipi(t["prop"], t["diag"], *t["ph"], 0, engine="split"), ref_pp) < 1e-12
        assert lib().ctr_split_refined() == nt * nt * 5
        assert rel(api.run_contract_rhopi(t["prop"], t["diag"], t["ph"][0], t["ph"][1], t["mom5"], 1,
                                          engine="split"), ref_rp) < 1e-12
        assert lib().ctr_split_refined() == nt * nt * 4
        hf, tri = api.run_contract_sigmapi(t["prop"], t["diag"], t["ph"][0], t["ph"][1], t["mom2"], engine="split")
        assert rel(hf, ref_hf) < 1e-12 and rel(tri, ref_tr) < 1e-12
        assert lib().ctr_split_refined() == nt + nt * nt * 2
        _refine(1e-9)
        assert rel(api.run_contract_pipi(t["prop"], t["diag"], *t["ph"], 0, engine="split"), ref_pp) <= 1e-9
        hf, tri = api.run_contract_sigmapi(t["prop"], t["diag"], t["ph"][0], t["ph"][1], t["mom2"], engine="split")
        assert rel(hf, ref_hf) <= 1e-9 and rel(tri, ref_tr) <= 1e-9
    finally:
        _refine(1e-9)
