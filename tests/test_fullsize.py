"""Parity at the production size of the rho workload (Nev=100, Lt=64, the 7
momenta |p|^2 <= 1, 3 polarisations, all 64 x 64 (t_src, t_sink): 86 016
correlator entries), through properties that need no CPU oracle at this size:

* every split-engine entry is within 1e-9 (relative, entry by entry) of the
  plain FP64 engine, whose parity with the oracle and the reference's own
  kernels is tested at smaller sizes;
* a whole t_sink row (t_sink = 0: 64 source times x 21 outputs = 1 344 entries)
  matches the oracle entry by entry on both engines;
* scaling the perambulator by 2^3 scales every correlator by exactly 2^6, on
  both engines, bit for bit: the split engine's slice scales are powers of two,
  so its digits, products, error estimates and refinement decisions are the
  same at both scales."""
import numpy as np
import pytest
import torch

from contractions_code_scattering_gb300 import api, synth
from tests import parity as P

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def workload(cuda):
    nt, nev = 64, 100
    moms = synth.momenta(1)
    rows, coef, oi = api.rho_rows_for_momenta(len(moms))
    tau = synth.make_prop(nt, nev, seed=1001, decay=0.35, backend="torch")
    phi = synth.make_phi_momenta_torch(nt, nev, moms, seed=1002)
    torch.cuda.synchronize()
    return tau, phi, rows, coef, oi, 3 * len(moms)


def _run(w, engine, tau=None):
    t, phi, rows, coef, oi, nout = w
    out = api.twosided(tau if tau is not None else t, phi, rows, coef, oi, nout, engine=engine)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def test_split_entries_within_1e9_of_fp64(workload):
    split = _run(workload, "split")
    fp64 = _run(workload, "fp64")
    assert split.shape == (64, 64, 21)
    rel = np.abs(split - fp64) / np.abs(fp64)
    assert rel.max() <= 1e-9, "largest entry error %.3e" % rel.max()


def test_power_of_two_scaling_is_exact(workload):
    tau = workload[0]
    tau8 = tau * 8.0
    for engine in ("split", "fp64"):
        a = _run(workload, engine)
        b = _run(workload, engine, tau=tau8)
        assert np.array_equal(b, a * 64.0), engine
    del tau8


def test_sink_row_matches_oracle_per_entry(workload):
    """t_sink = 0 of the production workload against the oracle (the reference's
    chain order: every spin row recomputes both of its products)."""
    from oracle import pyoracle as O
    tau, phi, rows, coef, oi, nout = workload
    vals = O.twosided_rows(tau[0].cpu().numpy(), phi.cpu().numpy(), rows, coef, 0, 0, tau.shape[0])
    ref = np.zeros((tau.shape[0], nout), np.complex128)
    ab = np.zeros((tau.shape[0], nout))
    for r, o in enumerate(oi):
        ref[:, o] += vals[:, r]
        ab[:, o] += np.abs(vals[:, r])
    for engine, tol in (("fp64", 1e-12), ("split", 1e-9)):
        got = _run(workload, engine)[0]
        st = P.entrywise(got, ref, tol, ab, "t_sink 0, %s engine" % engine)
        print("full-size t_sink 0, %s: worst per-entry rel %.2e, %d entries needed the floor"
              % (engine, st["max_rel"], st["needed_floor"]))
