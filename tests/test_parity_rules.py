"""The per-entry gate's row groupings (tests/parity.py) follow the reference's
host reductions: grouped and weighted the same way, the signed spin rows the
oracle returns must reproduce its correlators.  CPU only."""
import numpy as np

from contractions_code_scattering_gb300 import synth
from oracle import pyoracle as O
from tests import parity as P


def _data(nt=3, n=8, seed=11):
    prop = synth.make_prop(nt, n, seed=seed)
    rng = np.random.default_rng(seed + 1)
    ph = [synth.make_phi_random(nt, n, rng) for _ in range(4)]
    mom5 = np.ascontiguousarray(np.stack([synth.make_phi_random(nt, n, rng) for _ in range(5)], axis=1))
    return prop, ph, mom5


def _signed(rows, per):
    r = np.asarray(rows)
    return r.reshape(r.shape[:-1] + (r.shape[-1] // per, per)).sum(-1)


def _close(a, b):
    assert np.abs(a - b).max() <= 1e-14 * np.abs(b).max()


def test_two_sided_groupings():
    prop, ph, mom5 = _data()
    rows, corr = O.rho_row(prop, mom5, 1)
    _close(_signed(rows, 16).reshape(corr.shape), corr)
    assert P.rho_rows_abs(rows).shape == corr.shape
    rows, corr = O.sigma_row(prop, np.ascontiguousarray(mom5[:, :2]), 1)
    _close(_signed(rows, 16), corr)
    assert P.sigma_rows_abs(rows).shape == corr.shape


def test_chain_groupings():
    prop, ph, mom5 = _data()
    for idir in range(3):
        rows, corr = O.rhopi_row(prop, ph[0], ph[1], mom5, 1, idir)
        _close(_signed(rows, 64), corr)
        assert P.rhopi_rows_abs(rows).shape == corr.shape
    rows, corr = O.sigmapi_triangle_row(prop, ph[0], ph[1], np.ascontiguousarray(mom5[:, :2]), 1)
    _close(_signed(rows, 64), corr)
    hf, hrows = O.sigmapi_hor_fish(prop, ph[0], ph[1], with_rows=True)
    _close(hrows.sum(-1), hf)
    loop, lrows = O.loop_unity(prop, ph[2], with_rows=True)
    _close(lrows.sum(-1), loop)


def test_pipi_weights():
    prop, ph, _ = _data()
    for iso in (0, 1):
        d = O.pipi_row(prop, *ph, 1, iso)
        sq, dt, dth = d["square"].sum(-1), d["dtri"].sum(-1), d["dtri_hor"].sum(-1)
        star = d["star"][0].sum(-1) * d["star"][1].sum(-1)
        fish = d["fish"][0].sum(-1) * d["fish"][1].sum(-1)
        if iso == 1:
            want = np.stack([-2 * sq, 2 * dt, -star, fish, 0 * sq], axis=-1)
        else:
            want = np.stack([-sq / 3, -dt / 3, star, fish, -5 * dth / 3], axis=-1)
        _close(want, d["corr"])
        ab = P.pipi_rows_abs(d, iso)
        assert ab.shape == d["corr"].shape
        # each magnitude bounds its entry
        assert np.all(np.abs(d["corr"]) <= ab * (1 + 1e-12) + 1e-300)


def test_gate_uses_the_floor_only_for_cancelling_entries():
    ref = np.array([1.0, 1e-6])
    rows_abs = np.array([4.0, 4.0])  # the second entry cancels to 1e-6 of its rows
    got = ref + np.array([1e-13, 1e-14])
    st = P.entrywise(got, ref, 1e-12, rows_abs)
    assert st["needed_floor"] == 1
    try:
        P.entrywise(ref + np.array([1e-11, 0.0]), ref, 1e-12, rows_abs)
    except AssertionError:
        pass
    else:
        raise AssertionError("a well-conditioned entry off by 1e-11 passed the 1e-12 gate")
