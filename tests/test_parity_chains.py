"""GPU parity of the chain diagrams (rho->pipi, pipi I=1/I=0, loop-unity,
sigma->pipi) on both engines: against the reference's own kernel outputs
(golden vectors, Nev=100) and against the oracle at other sizes and at the
shapes of the benchmark configurations.

Every entry is gated on its own (tests/parity.py): |err| <= tol |ref| plus the
FP64 rounding floor 2^-44 x (sum of the magnitudes of the entry's spin rows),
which matters only where the rows cancel.  tol = 1e-12 for the plain FP64
engine and 1e-9 for the split engine (1e-10 on the small random data)."""
import os

import numpy as np
import pytest
import torch

from contractions_code_scattering_gb300 import api, synth
from oracle import pyoracle as O
from tests import parity as P

pytestmark = pytest.mark.gpu

TOL = 1e-12
SPLIT_TOL = 1e-10
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_outputs.npz")


def _np(x):
    return x.cpu().numpy() if hasattr(x, "cpu") else np.asarray(x)


def _dev(a, cuda):
    return torch.from_numpy(np.ascontiguousarray(a)).to(cuda)


class trace_form:
    """Forces the split engine's closing-trace form of the momentum-set calls
    (chains.trace_form: 0 the FP64 trace kernel, 1 Gram products on the tensor
    cores) inside a with block."""

    def __init__(self, form):
        self.form = form

    def __enter__(self):
        api.tune_force("chains.trace_form", self.form)

    def __exit__(self, *exc):
        api.tune_force("chains.trace_form", -1)


# ---- oracle references with their per-entry row magnitudes
def ref_pipi(prop, ph, iso, tfs=None):
    tfs = range(prop.shape[0]) if tfs is None else tfs
    ds = [O.pipi_row(prop, *ph, tf, iso) for tf in tfs]
    return np.stack([d["corr"] for d in ds]), np.stack([P.pipi_rows_abs(d, iso) for d in ds])


def ref_rhopi(prop, p1, p2, mom5, idir, tfs=None):
    tfs = range(prop.shape[0]) if tfs is None else tfs
    rc = [O.rhopi_row(prop, p1, p2, mom5, tf, idir) for tf in tfs]
    return np.stack([c for _, c in rc]), np.stack([P.rhopi_rows_abs(r) for r, _ in rc])


def ref_triangle(prop, p1, p2, mom2, tfs=None):
    tfs = range(prop.shape[0]) if tfs is None else tfs
    rc = [O.sigmapi_triangle_row(prop, p1, p2, mom2, tf) for tf in tfs]
    return np.stack([c for _, c in rc]), np.stack([P.triangle_rows_abs(r) for r, _ in rc])


def ref_hor_fish(prop, p1, p2):
    c, r = O.sigmapi_hor_fish(prop, p1, p2, with_rows=True)
    return c, P.sum_rows_abs(r)


def ref_loop(prop, mom):
    c, r = O.loop_unity(prop, mom, with_rows=True)
    return c, P.sum_rows_abs(r)


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


@pytest.mark.parametrize("engine,tol", [("fp64", TOL), ("split", SPLIT_TOL)])
@pytest.mark.parametrize("iso", [1, 0])
def test_pipi_vs_oracle(small, iso, engine, tol):
    d, t = small
    ref, ab = ref_pipi(d["prop"], d["ph"], iso)
    got = api.run_contract_pipi(t["prop"], t["diag"], *t["ph"], iso, engine=engine)
    P.entrywise(_np(got), ref, tol, ab, "pipi I%d %s" % (iso, engine))


@pytest.mark.parametrize("engine,tol", [("fp64", TOL), ("split", SPLIT_TOL)])
@pytest.mark.parametrize("idir", [0, 1, 2])
def test_rhopi_vs_oracle(small, idir, engine, tol):
    d, t = small
    ref, ab = ref_rhopi(d["prop"], d["ph"][0], d["ph"][1], d["mom5"], idir)
    got = api.run_contract_rhopi(t["prop"], t["diag"], t["ph"][0], t["ph"][1], t["mom5"], idir, engine=engine)
    P.entrywise(_np(got), ref, tol, ab, "rhopi idir %d %s" % (idir, engine))


@pytest.mark.parametrize("engine,tol", [("fp64", TOL), ("split", SPLIT_TOL)])
def test_sigmapi_and_loop_vs_oracle(small, engine, tol):
    d, t = small
    hf, tri = api.run_contract_sigmapi(t["prop"], t["diag"], t["ph"][0], t["ph"][1], t["mom2"], engine=engine)
    ref, ab = ref_hor_fish(d["prop"], d["ph"][0], d["ph"][1])
    P.entrywise(_np(hf), ref, tol, ab, "hor fish %s" % engine)
    ref, ab = ref_triangle(d["prop"], d["ph"][0], d["ph"][1], d["mom2"])
    P.entrywise(_np(tri), ref, tol, ab, "triangle %s" % engine)
    ref, ab = ref_loop(d["prop"], d["ph"][2])
    P.entrywise(_np(api.run_contract_loop_unity(t["diag"], t["ph"][2], engine=engine)), ref, tol, ab, "loop")


def test_row_range(small):
    """A single t_sink row held on the device, as the reference stages it."""
    d, t = small
    ref, ab = ref_pipi(d["prop"], d["ph"], 0)
    for tf in range(d["prop"].shape[0]):
        row = t["prop"][tf:tf + 1].contiguous()
        got = api.run_contract_pipi(row, t["diag"], *t["ph"], 0, tf_range=(tf, tf + 1))
        P.entrywise(_np(got[0]), ref[tf], TOL, ab[tf], "pipi row %d" % tf)


# ---- golden vectors: the reference's own kernels at Nev = 100
def _gold_abs(gold):
    out = {}
    for idir in range(3):
        out["rhopi%d" % idir] = P.rhopi_rows_abs(gold["rhopi%d_rows" % idir])
    for iso in (0, 1):
        g = {k: gold["pipi_I%d_%s" % (iso, k)] for k in ("square", "dtri", "dtri_hor")}
        g["star"] = np.moveaxis(gold["pipi_I%d_star" % iso], 2, 0)  # [2][tf][ti][16]
        g["fish"] = np.moveaxis(gold["pipi_I%d_fish" % iso], 2, 0)
        out["pipi%d" % iso] = P.pipi_rows_abs(g, iso)
    out["hor_fish"] = P.sum_rows_abs(gold["sigmapi_hor_fish_rows"])
    out["triangle"] = P.triangle_rows_abs(gold["sigmapi_triangle_rows"])
    out["loop"] = P.sum_rows_abs(gold["loop_rows"])
    return out


@pytest.mark.skipif(not os.path.exists(GOLD), reason="reference golden vectors not recorded")
@pytest.mark.parametrize("engine,tol", [("fp64", TOL), ("split", 1e-9)])
def test_chains_vs_reference_kernels(cuda, engine, tol):
    """Nev = 100; on the split engine the chains' four-term block products have
    K = 400 (leading digit halved)."""
    from tests.golden.make_ref_fixtures import inputs
    gold = dict(np.load(GOLD))
    ab = _gold_abs(gold)
    d = inputs()
    prop = _dev(d["prop"], cuda)
    diag = api.prop_diag(prop)
    p = [_dev(d[k], cuda) for k in ("p1", "p2", "p3", "p4")]
    mom5, mom2 = _dev(d["mom5"], cuda), _dev(d["mom2"], cuda)
    for idir in range(3):
        got = api.run_contract_rhopi(prop, diag, p[0], p[1], mom5, idir, engine=engine)
        P.entrywise(_np(got), gold["rhopi%d_corr" % idir], tol, ab["rhopi%d" % idir], "rhopi%d" % idir)
    for iso in (0, 1):
        got = api.run_contract_pipi(prop, diag, *p, iso, engine=engine)
        P.entrywise(_np(got), gold["pipi_I%d_corr" % iso], tol, ab["pipi%d" % iso], "pipi I%d" % iso)
    hf, tri = api.run_contract_sigmapi(prop, diag, p[0], p[1], mom2, engine=engine)
    P.entrywise(_np(hf), gold["sigmapi_hor_fish"], tol, ab["hor_fish"], "hor fish")
    P.entrywise(_np(tri), gold["sigmapi_triangle"], tol, ab["triangle"], "triangle")
    P.entrywise(_np(api.run_contract_loop_unity(diag, p[0], engine=engine)), gold["loop"], tol, ab["loop"], "loop")


# ---- the chain shapes of the benchmark configurations
def test_mixed_config_shape_split(cuda):
    """The mixed cross-correlator configuration's chain shape on the split engine:
    Nev = 128, so the four-term gamma_5 tasks have K = 4 x 128 = 512, the bound up to
    which the split engine's leading level stays exact; perambulator decay 0.25,
    momentum elementals Phi(+-p) for p = (1,1,1) and random rho / sigma operators.
    rho -> pi pi (3 polarisations), sigma -> pi pi (triangle and horizontal fish) and
    the sigma loops, per entry against the oracle on t_sink rows 0 and 2; the batched
    ctr_rhopi_sigmapi_sets gives the same bits."""
    nt, n = 3, 128
    prop = synth.make_prop(nt, n, seed=900, decay=0.25)
    moms = [(1, 1, 1), (-1, -1, -1)]
    phis = synth.make_phi_momenta(nt, n, moms, seed=901)
    p1, p2 = phis[moms[0]], phis[moms[1]]
    rng = np.random.default_rng(902)
    sd = np.sqrt(0.5 / n)
    mom5 = np.ascontiguousarray(rng.normal(0, sd, (nt, 5, n, n)) + 1j * rng.normal(0, sd, (nt, 5, n, n)))
    mom2 = np.ascontiguousarray(mom5[:, :2])
    tp, dp1, dp2, d5, d2 = (_dev(x, cuda) for x in (prop, p1, p2, mom5, mom2))
    diag = api.prop_diag(tp)
    rows = [0, 2]
    tol = 1e-9
    for idir in range(3):
        got = _np(api.run_contract_rhopi(tp, diag, dp1, dp2, d5, idir, engine="split"))[rows]
        ref, ab = ref_rhopi(prop, p1, p2, mom5, idir, rows)
        P.entrywise(got, ref, tol, ab, "rhopi idir %d" % idir)
    hf, tri = api.run_contract_sigmapi(tp, diag, dp1, dp2, d2, engine="split")
    ref, ab = ref_triangle(prop, p1, p2, mom2, rows)
    P.entrywise(_np(tri)[rows], ref, tol, ab, "sigma-pipi triangle")
    ref, ab = ref_hor_fish(prop, p1, p2)
    P.entrywise(_np(hf), ref, tol, ab, "hor fish")
    for k in range(2):
        got = _np(api.run_contract_loop_unity(diag, d2[:, k].contiguous(), engine="split"))
        ref, ab = ref_loop(prop, mom2[:, k])
        P.entrywise(got, ref, tol, ab, "sigma loop %d" % k)
    # the same pair through the batched call (with the reversed pair as a second set): bitwise
    # with the FP64 closing traces the per-set calls use
    phi_all = torch.stack([dp1, dp2], dim=1).contiguous()
    with trace_form(0):
        bat = {k: _np(v) for k, v in api.run_contract_rhopi_sigmapi_sets(tp, diag, phi_all, [(0, 1), (1, 0)], d5, d2,
                                                                         engine="split").items()}
    for idir in range(3):
        assert np.array_equal(bat["rhopi"][0, idir], _np(api.run_contract_rhopi(tp, diag, dp1, dp2, d5, idir,
                                                                                 engine="split")))
    assert np.array_equal(bat["triangle"][0], _np(tri)) and np.array_equal(bat["hor_fish"][0], _np(hf))
    # and with the closing traces as Gram products (K = 128^2 in 32 pieces of 512), per entry
    # against the oracle
    with trace_form(1):
        gr = {k: _np(v) for k, v in api.run_contract_rhopi_sigmapi_sets(tp, diag, phi_all, [(0, 1), (1, 0)], d5, d2,
                                                                        engine="split").items()}
    for idir in range(3):
        ref, ab = ref_rhopi(prop, p1, p2, mom5, idir, rows)
        P.entrywise(gr["rhopi"][0, idir][rows], ref, tol, ab, "Gram traces: rhopi idir %d" % idir)
        ref, ab = ref_rhopi(prop, p2, p1, mom5, idir, rows)
        P.entrywise(gr["rhopi"][1, idir][rows], ref, tol, ab, "Gram traces: reversed set, rhopi idir %d" % idir)
    ref, ab = ref_triangle(prop, p1, p2, mom2, rows)
    P.entrywise(gr["triangle"][0][rows], ref, tol, ab, "Gram traces: sigma-pipi triangle")
    assert np.array_equal(gr["hor_fish"][0], _np(hf))


@pytest.fixture(scope="module")
def pipi19(cuda):
    """The pi pi configuration's 19 momentum pairs (p, -p), |p|^2 <= 2, at Nev = 100
    (Nt = 4, t_sink row 1 sampled), with the oracle's I=0 rows for every pair; the
    I=1 weights are applied to the same rows."""
    nt, n, tf = 4, 100, 1
    prop = synth.make_prop(nt, n, seed=1200, decay=0.35)
    moms = synth.momenta(2)
    phis = synth.make_phi_momenta(nt, n, moms, seed=1201)
    pairs = [(p, tuple(-c for c in p)) for p in moms]
    refs = {}
    for a, b in pairs:
        d = O.pipi_row(prop, phis[a], phis[b], phis[a], phis[b], tf, 0)
        refs[(a, b)] = d
    dev = {"prop": _dev(prop, cuda), "phi": {p: _dev(phis[p], cuda) for p in moms}}
    dev["diag"] = api.prop_diag(dev["prop"])
    return dict(nt=nt, tf=tf, pairs=pairs, refs=refs, dev=dev)


def _i1_from_i0_rows(d):
    sq, dt = d["square"].sum(-1), d["dtri"].sum(-1)
    star = d["star"][0].sum(-1) * d["star"][1].sum(-1)
    fish = d["fish"][0].sum(-1) * d["fish"][1].sum(-1)
    return np.stack([-2 * sq, 2 * dt, -star, fish, 0 * sq], axis=-1)


@pytest.mark.parametrize("engine,tol", [("fp64", TOL), ("split", 1e-9)])
@pytest.mark.parametrize("iso", [0, 1])
def test_pipi_19_pair_set(pipi19, engine, iso, tol):
    """Each pair through ctr_pipi, and all 19 sets in one ctr_pipi_sets call (bitwise the same)."""
    c = pipi19
    dv, tf = c["dev"], c["tf"]
    row = dv["prop"][tf:tf + 1].contiguous()
    moms = list(dv["phi"])
    phi_all = torch.stack([dv["phi"][p] for p in moms], dim=1).contiguous()
    sets = [(moms.index(a), moms.index(b), moms.index(a), moms.index(b)) for a, b in c["pairs"]]
    batched = _np(api.run_contract_pipi_sets(row, dv["diag"], phi_all, sets, iso, engine=engine,
                                             tf_range=(tf, tf + 1)))
    stats = []
    for k, (a, b) in enumerate(c["pairs"]):
        d = c["refs"][(a, b)]
        ref = d["corr"] if iso == 0 else _i1_from_i0_rows(d)
        pa, pb = dv["phi"][a], dv["phi"][b]
        got = _np(api.run_contract_pipi(row, dv["diag"], pa, pb, pa, pb, iso, engine=engine, tf_range=(tf, tf + 1)))
        stats.append(P.entrywise(got[0], ref, tol, P.pipi_rows_abs(d, iso), "pair %s I%d %s" % (a, iso, engine)))
        assert np.array_equal(batched[k], got), "set %d: ctr_pipi_sets differs from ctr_pipi" % k
    print("pipi 19 pairs I%d %s: worst per-entry rel %.2e, %d entries needed the floor"
          % (iso, engine, max(s["max_rel"] for s in stats), sum(s["needed_floor"] for s in stats)))


@pytest.mark.parametrize("engine", ["fp64", "split"])
@pytest.mark.parametrize("iso", [0, 1])
def test_pipi_sets_bitwise_equal_to_per_set_calls(cuda, engine, iso):
    """ctr_pipi_sets on sets that share elementals (p, -p), (-p, p), an asymmetric set and
    p = 0: every set's entries are bitwise those of its own ctr_pipi call, over a t_sink
    row range."""
    nt, n = 4, 12
    prop = synth.make_prop(nt, n, seed=1500)
    moms = [(0, 0, 0), (1, 0, 0), (-1, 0, 0), (0, 1, 1), (0, -1, -1)]
    phis = synth.make_phi_momenta(nt, n, moms, seed=1501)
    phi_all = _dev(np.stack([phis[p] for p in moms], axis=1), cuda)
    sets = [(1, 2, 1, 2), (2, 1, 2, 1), (1, 2, 3, 4), (0, 0, 0, 0), (3, 4, 3, 4)]
    tp = _dev(prop, cuda)
    diag = api.prop_diag(tp)
    tr = (1, 3)
    rows = tp[tr[0]:tr[1]].contiguous()
    got = _np(api.run_contract_pipi_sets(rows, diag, phi_all, sets, iso, engine=engine, tf_range=tr))
    for k, q in enumerate(sets):
        ps = [phi_all[:, j].contiguous() for j in q]
        one = _np(api.run_contract_pipi(rows, diag, *ps, iso, engine=engine, tf_range=tr))
        assert np.array_equal(got[k], one), "set %d (%s engine)" % (k, engine)
    ref, ab = ref_pipi(prop, [phis[moms[j]] for j in sets[2]], iso, range(tr[0], tr[1]))
    P.entrywise(got[2], ref, TOL if engine == "fp64" else SPLIT_TOL, ab, "asymmetric set vs oracle")


@pytest.mark.parametrize("engine", ["fp64", "split"])
def test_rhopi_sigmapi_sets_bitwise_equal_to_per_set_calls(cuda, engine):
    """ctr_rhopi_sigmapi_sets: every set's rho -> pi pi (three polarisations), sigma -> pi pi
    triangle and horizontal fish are bitwise those of its own ctr_rhopi / ctr_sigmapi calls,
    over a t_sink row range, with sets that share elementals; one set against the oracle."""
    nt, n = 4, 12
    prop = synth.make_prop(nt, n, seed=1600, decay=0.25)
    moms = [(0, 0, 0), (1, 1, 0), (-1, -1, 0), (0, 0, 1), (0, 0, -1)]
    phis = synth.make_phi_momenta(nt, n, moms, seed=1601)
    phi_all = _dev(np.stack([phis[p] for p in moms], axis=1), cuda)
    rng = np.random.default_rng(1602)
    mom5 = np.ascontiguousarray(np.stack([synth.make_phi_random(nt, n, rng) for _ in range(5)], axis=1))
    mom2 = np.ascontiguousarray(np.stack([synth.make_phi_random(nt, n, rng) for _ in range(2)], axis=1))
    d5, d2 = _dev(mom5, cuda), _dev(mom2, cuda)
    sets = [(1, 2), (2, 1), (3, 4), (0, 0), (1, 4)]
    tp = _dev(prop, cuda)
    diag = api.prop_diag(tp)
    tr = (1, 3)
    rows = tp[tr[0]:tr[1]].contiguous()
    with trace_form(0):
        got = {k: _np(v) for k, v in api.run_contract_rhopi_sigmapi_sets(rows, diag, phi_all, sets, d5, d2,
                                                                         engine=engine, tf_range=tr).items()}
    for k, (a, b) in enumerate(sets):
        pa, pb = phi_all[:, a].contiguous(), phi_all[:, b].contiguous()
        for idir in range(3):
            one = _np(api.run_contract_rhopi(rows, diag, pa, pb, d5, idir, engine=engine, tf_range=tr))
            assert np.array_equal(got["rhopi"][k, idir], one), "set %d idir %d (%s)" % (k, idir, engine)
        hf, tri = api.run_contract_sigmapi(rows, diag, pa, pb, d2, engine=engine, tf_range=tr)
        assert np.array_equal(got["triangle"][k], _np(tri)), "set %d triangle (%s)" % (k, engine)
        assert np.array_equal(got["hor_fish"][k], _np(hf)), "set %d hor fish (%s)" % (k, engine)
    tol = TOL if engine == "fp64" else SPLIT_TOL
    ref, ab = ref_rhopi(prop, phis[moms[1]], phis[moms[4]], mom5, 2, range(tr[0], tr[1]))
    P.entrywise(got["rhopi"][4, 2], ref, tol, ab, "set (1,4) rho-pipi idir 2 vs oracle")
    ref, ab = ref_triangle(prop, phis[moms[1]], phis[moms[4]], mom2, range(tr[0], tr[1]))
    P.entrywise(got["triangle"][4], ref, tol, ab, "set (1,4) triangle vs oracle")
    ref, ab = ref_hor_fish(prop, phis[moms[1]], phis[moms[4]])
    P.entrywise(got["hor_fish"][4], ref, tol, ab, "set (1,4) hor fish vs oracle")


@pytest.mark.parametrize("n", [12, 100])
def test_rhopi_sigmapi_sets_gram_traces(cuda, n):
    """ctr_rhopi_sigmapi_sets on the split engine with its closing traces as Gram
    products (one group per pair and tau column block s2: the sets' X blocks against
    the sink operators' Z blocks): every set's rho -> pi pi and sigma -> pi pi
    triangle per entry against the oracle, and against the FP64 closing traces.
    Nev = 12: one K piece of 144 elements; Nev = 100: 20 pieces, the last one
    272 elements long."""
    nt = 3 if n == 100 else 4
    prop = synth.make_prop(nt, n, seed=1700 + n, decay=0.25)
    moms = [(0, 0, 0), (1, 1, 0), (-1, -1, 0), (0, 0, 1), (0, 0, -1)]
    phis = synth.make_phi_momenta(nt, n, moms, seed=1701 + n)
    cuda_phi = _dev(np.stack([phis[p] for p in moms], axis=1), cuda)
    rng = np.random.default_rng(1702 + n)
    mom5 = np.ascontiguousarray(np.stack([synth.make_phi_random(nt, n, rng) for _ in range(5)], axis=1))
    mom2 = np.ascontiguousarray(np.stack([synth.make_phi_random(nt, n, rng) for _ in range(2)], axis=1))
    d5, d2 = _dev(mom5, cuda), _dev(mom2, cuda)
    sets = [(1, 2), (2, 1), (3, 4), (0, 0), (1, 4)]
    tp = _dev(prop, cuda)
    diag = api.prop_diag(tp)
    tr = (1, 3)
    rows = tp[tr[0]:tr[1]].contiguous()
    got = {}
    for form in (0, 1):
        with trace_form(form):
            got[form] = {k: _np(v) for k, v in api.run_contract_rhopi_sigmapi_sets(
                rows, diag, cuda_phi, sets, d5, d2, engine="split", tf_range=tr).items()}
    g, f = got[1], got[0]
    tol = 1e-9 if n == 100 else SPLIT_TOL
    for k, (a, b) in enumerate(sets):
        pa, pb = phis[moms[a]], phis[moms[b]]
        for idir in range(3):
            ref, ab = ref_rhopi(prop, pa, pb, mom5, idir, range(tr[0], tr[1]))
            P.entrywise(g["rhopi"][k, idir], ref, tol, ab, "set %d rhopi idir %d, Gram traces" % (k, idir))
            P.entrywise(g["rhopi"][k, idir], f["rhopi"][k, idir], tol, ab, "set %d idir %d, Gram vs FP64 traces" % (k, idir))
        ref, ab = ref_triangle(prop, pa, pb, mom2, range(tr[0], tr[1]))
        P.entrywise(g["triangle"][k], ref, tol, ab, "set %d triangle, Gram traces" % k)
        # the horizontal fish keeps its per-time-slice FP64 traces
        assert np.array_equal(g["hor_fish"][k], f["hor_fish"][k])
    if n != 12:
        return
    # refinement with the Gram traces' error scales: a tolerance below the engine's
    # error flags every entry, and the FP64 reruns give the FP64 engine's accuracy
    from contractions_code_scattering_gb300._lib import lib
    try:
        _refine(1e-15)
        with trace_form(1):
            rf = {k: _np(v) for k, v in api.run_contract_rhopi_sigmapi_sets(
                rows, diag, cuda_phi, sets, d5, d2, engine="split", tf_range=tr).items()}
        assert lib().ctr_split_refined() > 0
    finally:
        _refine(1e-9)
    for k, (a, b) in enumerate(sets):
        pa, pb = phis[moms[a]], phis[moms[b]]
        ref, ab = ref_rhopi(prop, pa, pb, mom5, 2, range(tr[0], tr[1]))
        P.entrywise(rf["rhopi"][k, 2], ref, TOL, ab, "set %d rhopi idir 2, refined" % k)
        ref, ab = ref_triangle(prop, pa, pb, mom2, range(tr[0], tr[1]))
        P.entrywise(rf["triangle"][k], ref, TOL, ab, "set %d triangle, refined" % k)


def test_rhopi_sigmapi_sets_gram_traces_two_m_tiles(cuda):
    """36 momentum sets over 7 elementals: 36 set combinations, so each Gram group has
    144 X blocks, two M tiles of its instances.  Every set's rho -> pi pi and triangle
    with Gram traces per entry against the FP64 closing traces, and one set against the
    oracle."""
    nt, n = 3, 12
    prop = synth.make_prop(nt, n, seed=1800, decay=0.25)
    moms = [(0, 0, 0), (1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)]
    phis = synth.make_phi_momenta(nt, n, moms, seed=1801)
    cuda_phi = _dev(np.stack([phis[p] for p in moms], axis=1), cuda)
    rng = np.random.default_rng(1802)
    mom5 = np.ascontiguousarray(np.stack([synth.make_phi_random(nt, n, rng) for _ in range(5)], axis=1))
    mom2 = np.ascontiguousarray(mom5[:, :2])
    d5, d2 = _dev(mom5, cuda), _dev(mom2, cuda)
    sets = [(a, b) for a in range(1, 7) for b in range(1, 7)]
    tp = _dev(prop, cuda)
    diag = api.prop_diag(tp)
    got = {}
    for form in (0, 1):
        with trace_form(form):
            got[form] = {k: _np(v) for k, v in api.run_contract_rhopi_sigmapi_sets(
                tp, diag, cuda_phi, sets, d5, d2, engine="split").items()}
    g, f = got[1], got[0]
    for k, (a, b) in enumerate(sets):
        pa, pb = phis[moms[a]], phis[moms[b]]
        for idir in range(3):
            ref, ab = ref_rhopi(prop, pa, pb, mom5, idir)
            P.entrywise(g["rhopi"][k, idir], f["rhopi"][k, idir], SPLIT_TOL, ab,
                        "set %d idir %d, Gram vs FP64 traces" % (k, idir))
            if (a, b) == (3, 6):
                P.entrywise(g["rhopi"][k, idir], ref, SPLIT_TOL, ab, "set (3, 6) rhopi idir %d, Gram traces" % idir)
        ref, ab = ref_triangle(prop, pa, pb, mom2)
        P.entrywise(g["triangle"][k], f["triangle"][k], SPLIT_TOL, ab, "set %d triangle, Gram vs FP64 traces" % k)
        if (a, b) == (3, 6):
            P.entrywise(g["triangle"][k], ref, SPLIT_TOL, ab, "set (3, 6) triangle, Gram traces")


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


def test_block_product_tasks_power_of_two_weights(cuda):
    """Term weights of both signs and several powers of two, with the left blocks
    conjugate-transposed, on operands far from 1 (2^-600 and 2^500): the split
    engine applies the weights and conjugations as exponent offsets and signs
    while slicing, the FP64 engine multiplies them in."""
    n = 64
    rng = np.random.default_rng(9)
    M1 = (rng.normal(size=(8, n, n)) + 1j * rng.normal(size=(8, n, n))) * 2.0 ** -600
    M1 *= np.exp(-rng.uniform(0, 10, (8, 1, n)))  # columns of M1 (rows of M1^dagger) over 4 decades
    M2 = (rng.normal(size=(8, n, n)) + 1j * rng.normal(size=(8, n, n))) * 2.0 ** 500
    w = [0.5, -2.0, 0.25, -1.0]
    ref = np.zeros((2, n, n), np.complex128)
    tasks = []
    for c in range(2):
        for k in range(4):
            ref[c] += w[k] * M1[c * 4 + k].conj().T @ M2[c * 4 + k]
        tasks.append(([c * 4 + k for k in range(4)], [c * 4 + k for k in range(4)], c))
    x, y = _dev(M1, cuda), _dev(M2, cuda)
    # entry error against the scale of its row of op(M1) and the largest |M2|
    scale = np.abs(M1).max(axis=1).reshape(2, 4, n).max(axis=1)[:, :, None] * np.abs(M2).max() * 4 * n * 2
    for engine, tol in (("fp64", 1e-14), ("split", 1e-12)):
        out = api.zgemm_tasks(x, y, tasks, weights=w, a_dagger=True, engine=engine)
        api.sync()
        err = (np.abs(out.cpu().numpy() - ref) / scale).max()
        assert err <= tol, (engine, err)


def _refine(tol):
    from contractions_code_scattering_gb300._lib import check, lib
    check(lib().ctr_split_set_refine(tol))


def test_split_chain_refinement(small):
    """Per-entry accuracy of the split chain engine: with the tolerance below the
    engine's error every pair is recomputed by the FP64 engine (results at the FP64
    engine's per-entry tolerance); with 1e-9 every entry meets 1e-9 relative to itself."""
    from contractions_code_scattering_gb300._lib import lib
    d, t = small
    nt = d["prop"].shape[0]
    ref_pp = ref_pipi(d["prop"], d["ph"], 0)
    ref_rp = ref_rhopi(d["prop"], d["ph"][0], d["ph"][1], d["mom5"], 1)
    ref_hf = ref_hor_fish(d["prop"], d["ph"][0], d["ph"][1])
    ref_tr = ref_triangle(d["prop"], d["ph"][0], d["ph"][1], d["mom2"])
    try:
        _refine(1e-15)
        P.entrywise(_np(api.run_contract_pipi(t["prop"], t["diag"], *t["ph"], 0, engine="split")), ref_pp[0],
                    TOL, ref_pp[1], "pipi refined")
        assert lib().ctr_split_refined() == nt * nt * 5
        P.entrywise(_np(api.run_contract_rhopi(t["prop"], t["diag"], t["ph"][0], t["ph"][1], t["mom5"], 1,
                                               engine="split")), ref_rp[0], TOL, ref_rp[1], "rhopi refined")
        assert lib().ctr_split_refined() == nt * nt * 4
        hf, tri = api.run_contract_sigmapi(t["prop"], t["diag"], t["ph"][0], t["ph"][1], t["mom2"], engine="split")
        P.entrywise(_np(hf), ref_hf[0], TOL, ref_hf[1], "hor fish refined")
        P.entrywise(_np(tri), ref_tr[0], TOL, ref_tr[1], "triangle refined")
        assert lib().ctr_split_refined() == nt + nt * nt * 2
        _refine(1e-9)
        P.entrywise(_np(api.run_contract_pipi(t["prop"], t["diag"], *t["ph"], 0, engine="split")), ref_pp[0], 1e-9,
                    ref_pp[1], "pipi at 1e-9")
        hf, tri = api.run_contract_sigmapi(t["prop"], t["diag"], t["ph"][0], t["ph"][1], t["mom2"], engine="split")
        P.entrywise(_np(hf), ref_hf[0], 1e-9, ref_hf[1], "hor fish at 1e-9")
        P.entrywise(_np(tri), ref_tr[0], 1e-9, ref_tr[1], "triangle at 1e-9")
    finally:
        _refine(1e-9)
