"""Checks of the oracle itself: its C restatement against independent numpy
formulas of the same reference routines, and the synthetic-data identities."""
import numpy as np
import pytest

from contractions_code_scattering_gb300 import synth
from oracle import pyoracle as O
from oracle import tables as T

N, NT = 5, 3


@pytest.fixture(scope="module")
def data():
    prop = synth.make_prop(NT, N, seed=11, decay=0.3)
    rng = np.random.default_rng(5)
    mom5 = np.stack([synth.make_phi_random(NT, N, rng) for _ in range(5)], axis=1)
    moms = [synth.make_phi_random(NT, N, rng) for _ in range(4)]
    return prop, mom5, moms


def test_prop_gamma5_hermiticity(data):
    prop = data[0]
    g5 = synth.G5
    for t1 in range(NT):
        for t2 in range(NT):
            lhs = prop[t1, t2]
            rhs = np.conj(np.transpose(prop[t2, t1], (1, 0, 3, 2))) * (g5[:, None, None, None] * g5[None, :, None, None])
            assert np.allclose(lhs, rhs, atol=0, rtol=0)


def test_prop_decay():
    prop = synth.make_prop(6, 8, seed=1, decay=0.35)
    m = [np.abs(prop[t, 0]).mean() for t in range(6)]
    ratios = [m[t + 1] / m[t] for t in range(1, 5)]
    assert np.allclose(ratios, np.exp(-0.35), rtol=0.15)


def test_rho_rows_against_numpy(data):
    prop, mom5, _ = data
    spin, lprp, coef = T.rho_tables()
    tf = 1
    rows, corr = O.rho_row(prop, mom5, tf)
    for ti in range(NT):
        for r in (0, 17, 300, 767):
            s1, s2, s3, s4 = spin[r]
            lp, rp = lprp[r]
            t1 = prop[tf, ti, s3, s4] @ mom5[ti, lp]
            t2 = mom5[tf, rp] @ prop[tf, ti, s1, s2]
            c = complex(np.float32(coef[r, 0]), np.float32(coef[r, 1]))
            assert np.isclose(rows[ti, r], c * np.sum(np.conj(t2) * t1), rtol=1e-13, atol=0)
    assert np.allclose(corr, rows.reshape(NT, 16, 3, 16).sum(-1), rtol=1e-13, atol=1e-15)


def test_sigma_rows_against_numpy(data):
    prop, mom5, _ = data
    mom2 = np.ascontiguousarray(mom5[:, :2])
    spin, lprp, coef = T.sigma_tables()
    tf = 2
    rows, _ = O.sigma_row(prop, mom2, tf)
    for ti in range(NT):
        for r in (0, 31, 63):
            s1, s2, s3, s4 = spin[r]
            lp, rp = lprp[r]
            t1 = prop[tf, ti, s3, s4] @ mom2[ti, rp]
            t2 = mom2[tf, lp] @ prop[tf, ti, s2, s1]
            c = complex(np.float32(coef[r, 0]), np.float32(coef[r, 1]))
            assert np.isclose(rows[ti, r], c * np.sum(np.conj(t2) * t1), rtol=1e-13, atol=0)


def test_pipi_chains_against_numpy(data):
    prop, _, (p1, p2, p3, p4) = data
    t = T.pipi_tables()
    tf = 2
    d = O.pipi_row(prop, p1, p2, p3, p4, tf, iso=0)
    diag = O.prop_diag(prop)
    ti = 1
    tau = prop[tf, ti]
    r = 77
    s = t["spinIndices_pipi_square"][r]
    x = p3[tf] @ diag[tf, s[2], s[3]] @ p4[tf] @ tau[s[4], s[5]] @ p2[ti] @ diag[ti, s[0], s[1]] @ p1[ti]
    c = complex(*t["coef_pipi_square"][r])
    assert np.isclose(d["square"][ti, r], c * np.sum(x * np.conj(tau[s[2], s[1]])), rtol=1e-12)
    s = t["spinIndices_pipi_doubleTriangle"][r]
    x = p3[tf] @ diag[tf, s[4], s[5]] @ p4[tf] @ tau[s[0], s[1]] @ p1[ti] @ diag[ti, s[2], s[3]] @ p2[ti]
    c = complex(*t["coef_pipi_doubleTriangle"][r])
    assert np.isclose(d["dtri"][ti, r], c * np.sum(x * np.conj(tau[s[4], s[3]])), rtol=1e-12)
    s = t["spinIndices_pipi_doubleTriangle_hor"][r]
    x = p3[tf] @ tau[s[0], s[1]] @ p1[ti] @ tau[s[2], s[1]].conj().T @ p4[tf] @ tau[s[2], s[3]] @ p2[ti]
    assert np.isclose(d["dtri_hor"][ti, r], np.sum(x * np.conj(tau[s[0], s[3]])), rtol=1e-12)
    # star (P4 at the sink of trace 1) and fish (P3), with the isospin weights of I=0
    st = [sum(np.sum((pa[tf] @ tau[a, b] @ pb[ti]) * np.conj(tau[a, b])) for a in range(4) for b in range(4))
          for pa, pb in ((p4, p1), (p3, p2))]
    fi = [sum(np.sum((pa[tf] @ tau[a, b] @ pb[ti]) * np.conj(tau[a, b])) for a in range(4) for b in range(4))
          for pa, pb in ((p3, p1), (p4, p2))]
    assert np.isclose(d["corr"][ti, 2], st[0] * st[1], rtol=1e-12)
    assert np.isclose(d["corr"][ti, 3], fi[0] * fi[1], rtol=1e-12)
    assert np.isclose(d["corr"][ti, 0], -1 / 3 * d["square"][ti].sum(), rtol=1e-12)
    assert np.isclose(d["corr"][ti, 4], -5 / 3 * d["dtri_hor"][ti].sum(), rtol=1e-12)
    d1 = O.pipi_row(prop, p1, p2, p3, p4, tf, iso=1)
    assert np.isclose(d1["corr"][ti, 0], -2 * d1["square"][ti].sum(), rtol=1e-12)
    assert np.isclose(d1["corr"][ti, 2], -st[0] * st[1], rtol=1e-12)
    assert d1["corr"][ti, 4] == 0


def test_rhopi_and_sigmapi_against_numpy(data):
    prop, mom5, (p1, p2, p3, _) = data
    diag = O.prop_diag(prop)
    tf, ti, idir = 0, 2, 1
    spin, ip, coef = T.rhopi_tables()
    rows, corr = O.rhopi_row(prop, p1, p2, mom5, tf, idir)
    tau = prop[tf, ti]
    for bx in (0, 100, 255):
        r = idir * 256 + bx
        s1, s2, s3, s4, s5, s6 = spin[r]
        x = mom5[tf, ip[r]] @ tau[s5, s6] @ p2[ti] @ diag[ti, s1, s2] @ p1[ti]
        c = complex(*coef[r])
        assert np.isclose(rows[ti, bx], c * np.sum(x * np.conj(tau[s3, s2])), rtol=1e-12)
    mom2 = np.ascontiguousarray(mom5[:, :2])
    t = T.sigmapi_tables()
    rows, _ = O.sigmapi_triangle_row(prop, p1, p2, mom2, tf)
    for bx in (0, 64, 127):
        s = t["spinIndices_sigmapi_triangle"][bx]
        ipx = t["ip_sigmapi_triangle"][bx]
        x = mom2[tf, ipx] @ tau[s[1], s[2]] @ p2[ti] @ diag[ti, s[3], s[4]] @ p1[ti]
        c = complex(*t["coef_sigmapi_triangle"][bx])
        assert np.isclose(rows[ti, bx], c * np.sum(x * np.conj(tau[s[0], s[4]])), rtol=1e-12)
    hf = O.sigmapi_hor_fish(prop, p1, p2)
    for tt in range(NT):
        ref = sum(np.sum((p2[tt] @ diag[tt, a, b] @ p1[tt]) * np.conj(diag[tt, a, b])) for a in range(4) for b in range(4))
        assert np.isclose(hf[tt], ref, rtol=1e-12)
    lp = O.loop_unity(prop, p3)
    for tt in range(NT):
        assert np.isclose(lp[tt], sum(np.trace(diag[tt, s, s] @ p3[tt]) for s in range(4)), rtol=1e-12)


def test_source_average_and_reorder():
    rng = np.random.default_rng(3)
    corr = rng.normal(size=(4, 4, 2)) + 1j * rng.normal(size=(4, 4, 2))
    avg = O.source_average(corr)
    for dt in range(4):
        assert np.allclose(avg[dt], np.mean([corr[(ti + dt) % 4, ti] for ti in range(4)], axis=0))
    prop = synth.make_prop(2, 3, seed=4)
    file_order = np.ascontiguousarray(np.transpose(prop, (2, 4, 0, 3, 5, 1)))  # [s1][v1][t1][s2][v2][t2]
    assert np.array_equal(O.reorder_prop(file_order, 3, 2), prop)
