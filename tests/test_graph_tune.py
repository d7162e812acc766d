"""CUDA-graph recording/replay of library calls and the autotuner.

Host-side logic (argument checks, the tuning table's save/load/force/report)
runs without a GPU.  The GPU tests check that a replayed graph gives the same
correlators as the eager calls (bitwise: the same kernels on the same data),
that a replay sees in-place refills of the inputs, that the split engine's
refinement runs between graph segments, and that every autotuner candidate
meets the oracle within the engine's tolerance."""
import ctypes

import numpy as np
import pytest
import torch

from contractions_code_scattering_gb300 import api, synth
from contractions_code_scattering_gb300._lib import CtrError, check, lib
from oracle import pyoracle as O


# ------------------------------------------------------------------ host side
def test_graph_argument_errors():
    L = lib()
    assert L.ctr_graph_begin(None) != 0  # the legacy default stream cannot be recorded
    assert b"created stream" in L.ctr_last_error()
    g = ctypes.c_void_p()
    assert L.ctr_graph_end(None, ctypes.byref(g)) != 0  # nothing is being recorded
    assert L.ctr_graph_launch(None, None) != 0
    assert L.ctr_graph_info(None, None, None, None) != 0
    L.ctr_graph_destroy(None)  # no-op


def test_tune_table_roundtrip(tmp_path):
    api.tune_clear()
    p = tmp_path / "tune.txt"
    p.write_text("trace_rows|nev=100,ntr=224 2\ntwosided.batch|nev=100,ncd=16 8\n")
    api.tune_load(p)
    rep = api.tune_report()
    assert rep["trace_rows|nev=100,ntr=224"]["choice"] == 2
    assert rep["twosided.batch|nev=100,ncd=16"]["choice"] == 8
    q = tmp_path / "out.txt"
    api.tune_save(q)
    assert sorted(q.read_text().split("\n")) == sorted(p.read_text().split("\n"))
    api.tune_force("split_gemm.order", 1)
    assert api.tune_report()["split_gemm.order|forced"]["choice"] == 1
    api.tune_force("split_gemm.order", -1)
    assert "split_gemm.order|forced" not in api.tune_report()
    api.tune_clear()
    assert api.tune_report() == {}


@pytest.mark.parametrize("text", ["no separator line 3\n", "trace_rows|x -1\n", "trace_rows|x two\n"])
def test_tune_load_rejects_malformed(tmp_path, text):
    p = tmp_path / "bad.txt"
    p.write_text(text)
    with pytest.raises(CtrError):
        api.tune_load(p)


def test_tune_mode_and_force_checks():
    with pytest.raises(CtrError):
        api.tune_set_mode(3)
    with pytest.raises(CtrError):
        api.tune_force("a|b", 1)
    api.tune_set_mode(0)


# ------------------------------------------------------------------ GPU side
def _refine(tol):
    check(lib().ctr_split_set_refine(tol))


def _rho_inputs(nt, n, seed):
    prop = synth.make_prop(nt, n, seed=seed)
    rng = np.random.default_rng(seed + 1)
    mom5 = np.ascontiguousarray(np.stack([synth.make_phi_random(nt, n, rng) for _ in range(5)], axis=1))
    return prop, mom5


@pytest.mark.gpu
@pytest.mark.parametrize("engine", ["fp64", "split"])
def test_graph_rho_replay_matches_eager(cuda, engine):
    nt, n = 4, 20
    prop, mom5 = _rho_inputs(nt, n, seed=501)
    d_prop, d_mom = torch.from_numpy(prop).to(cuda), torch.from_numpy(mom5).to(cuda)
    s = torch.cuda.Stream()
    eager = api.run_contract_rho(d_prop, d_mom, engine=engine, stream=s)
    s.synchronize()
    eager = eager.cpu().numpy()
    out = torch.zeros((nt, nt, 16, 3), dtype=torch.complex128, device=cuda)
    torch.cuda.synchronize()
    g = api.Graph(s)
    with g:
        api.run_contract_rho(d_prop, d_mom, engine=engine, out=out, stream=s)
    assert out.abs().max().item() == 0.0  # recording executes nothing
    nseg, nker, nbytes = g.info()
    assert nseg >= 1 and nker >= 3 and nbytes > 0
    for _ in range(2):
        out.zero_()
        torch.cuda.synchronize()
        g.launch(s)
        s.synchronize()
        assert np.array_equal(out.cpu().numpy(), eager)
    # refill the inputs in place: the replay computes on the new contents
    prop2, mom2 = _rho_inputs(nt, n, seed=733)
    d_prop.copy_(torch.from_numpy(prop2))
    d_mom.copy_(torch.from_numpy(mom2))
    torch.cuda.synchronize()
    g.launch(s)
    s.synchronize()
    ref = O.rho(prop2, mom2)
    got = out.cpu().numpy()
    assert np.abs(got - ref).max() / np.abs(ref).max() <= (1e-12 if engine == "fp64" else 1e-9)
    g.close()


@pytest.mark.gpu
def test_graph_split_refinement_between_segments(cuda):
    """The recomputation of flagged entries (a host step) runs at every replay."""
    nt, n = 3, 24
    prop, mom5 = _rho_inputs(nt, n, seed=77)
    ref = O.rho(prop, mom5)
    d_prop, d_mom = torch.from_numpy(prop).to(cuda), torch.from_numpy(mom5).to(cuda)
    out = torch.empty((nt, nt, 16, 3), dtype=torch.complex128, device=cuda)
    s = torch.cuda.Stream()
    torch.cuda.synchronize()
    try:
        _refine(1e-15)  # every entry is flagged
        with api.Graph(s) as g:
            api.run_contract_rho(d_prop, d_mom, engine="split", out=out, stream=s)
        assert g.info()[0] >= 2  # the host step split the recording
        for _ in range(2):
            out.zero_()
            torch.cuda.synchronize()
            g.launch(s)
            s.synchronize()
            assert lib().ctr_split_refined() == ref.size
            got = out.cpu().numpy()
            assert (np.abs(got - ref) / np.abs(ref)).max() <= 1e-11
        g.close()
    finally:
        _refine(1e-9)


@pytest.fixture(scope="module")
def chains(cuda):
    nt, n = 3, 12
    prop = synth.make_prop(nt, n, seed=300)
    rng = np.random.default_rng(301)
    ph = [synth.make_phi_random(nt, n, rng) for _ in range(4)]
    mom5 = np.ascontiguousarray(np.stack([synth.make_phi_random(nt, n, rng) for _ in range(5)], axis=1))
    mom2 = np.ascontiguousarray(mom5[:, 1:3])
    d = dict(prop=prop, ph=ph, mom5=mom5, mom2=mom2)
    t = {k: torch.from_numpy(v).to(cuda) for k, v in (("prop", prop), ("mom5", mom5), ("mom2", mom2))}
    t["ph"] = [torch.from_numpy(p).to(cuda) for p in ph]
    t["diag"] = api.prop_diag(t["prop"])
    return d, t


@pytest.mark.gpu
@pytest.mark.parametrize("engine,tol", [("fp64", 1e-15), ("split", 1e-15), ("split", 1e-9)])
def test_graph_chain_families(cuda, chains, engine, tol):
    """pi pi, rho pi pi, sigma pi pi and the loop recorded in one graph; replay equals eager."""
    d, t = chains
    nt = d["prop"].shape[0]
    s = torch.cuda.Stream()

    def outs():
        return dict(pp=torch.empty((nt, nt, 5), dtype=torch.complex128, device=cuda),
                    rp=torch.empty((nt, nt, 4), dtype=torch.complex128, device=cuda),
                    hf=torch.empty((nt,), dtype=torch.complex128, device=cuda),
                    tr=torch.empty((nt, nt, 2), dtype=torch.complex128, device=cuda),
                    lp=torch.empty((nt,), dtype=torch.complex128, device=cuda))

    def calls(o):
        api.run_contract_pipi(t["prop"], t["diag"], *t["ph"], 0, engine=engine, out=o["pp"], stream=s)
        api.run_contract_rhopi(t["prop"], t["diag"], t["ph"][0], t["ph"][1], t["mom5"], 1, engine=engine,
                               out=o["rp"], stream=s)
        api.run_contract_sigmapi(t["prop"], t["diag"], t["ph"][0], t["ph"][1], t["mom2"], engine=engine,
                                 out=(o["hf"], o["tr"]), stream=s)
        api.run_contract_loop_unity(t["diag"], t["ph"][0], engine=engine, out=o["lp"], stream=s)

    try:
        _refine(tol)
        eager, rec = outs(), outs()
        torch.cuda.synchronize()
        calls(eager)
        s.synchronize()
        with api.Graph(s) as g:
            calls(rec)
        g.launch(s)
        s.synchronize()
        for k in eager:
            assert np.array_equal(rec[k].cpu().numpy(), eager[k].cpu().numpy()), k
        ref_pp = O.pipi(d["prop"], *d["ph"], 0)
        assert np.abs(rec["pp"].cpu().numpy() - ref_pp).max() / np.abs(ref_pp).max() <= 1e-9
        g.close()
    finally:
        _refine(1e-9)


@pytest.mark.gpu
@pytest.mark.parametrize("engine,tol", [("fp64", 1e-15), ("split", 1e-15), ("split", 1e-9)])
def test_graph_momentum_set_calls(cuda, engine, tol):
    """ctr_pipi_sets and ctr_rhopi_sigmapi_sets recorded in one graph (the split engine's
    refinement between segments at tol 1e-15): the replay equals the eager calls bitwise."""
    nt, n = 3, 12
    prop = torch.from_numpy(synth.make_prop(nt, n, seed=1700)).to(cuda)
    moms = [(0, 0, 0), (1, 0, 0), (-1, 0, 0)]
    phis = synth.make_phi_momenta(nt, n, moms, seed=1701)
    phi = torch.from_numpy(np.ascontiguousarray(np.stack([phis[p] for p in moms], axis=1))).to(cuda)
    rng = np.random.default_rng(1702)
    mom5 = torch.from_numpy(np.ascontiguousarray(np.stack([synth.make_phi_random(nt, n, rng) for _ in range(5)],
                                                          axis=1))).to(cuda)
    mom2 = mom5[:, :2].contiguous()
    diag = api.prop_diag(prop)
    s = torch.cuda.Stream()
    pp_sets, rs_sets = [(1, 2, 1, 2), (2, 1, 2, 1), (0, 0, 0, 0)], [(1, 2), (2, 1), (0, 0)]

    def outs():
        kw = dict(dtype=torch.complex128, device=cuda)
        return dict(pp=torch.empty((3, nt, nt, 5), **kw),
                    rs=dict(rhopi=torch.empty((3, 3, nt, nt, 4), **kw), triangle=torch.empty((3, nt, nt, 2), **kw),
                            hor_fish=torch.empty((3, nt), **kw)))

    def calls(o):
        api.run_contract_pipi_sets(prop, diag, phi, pp_sets, 0, engine=engine, out=o["pp"], stream=s)
        api.run_contract_rhopi_sigmapi_sets(prop, diag, phi, rs_sets, mom5, mom2, engine=engine, out=o["rs"], stream=s)

    try:
        _refine(tol)
        eager, rec = outs(), outs()
        torch.cuda.synchronize()
        calls(eager)
        s.synchronize()
        with api.Graph(s) as g:
            calls(rec)
        g.launch(s)
        s.synchronize()
        assert np.array_equal(rec["pp"].cpu().numpy(), eager["pp"].cpu().numpy())
        for k in eager["rs"]:
            assert np.array_equal(rec["rs"][k].cpu().numpy(), eager["rs"][k].cpu().numpy()), k
        g.close()
    finally:
        _refine(1e-9)


@pytest.mark.gpu
def test_graph_rejects_host_planned_calls(cuda):
    """A call that plans on device data cannot be recorded: ctr_graph_end fails and the stream stays usable."""
    nt, n = 2, 8
    prop, mom5 = _rho_inputs(nt, n, seed=5)
    d_prop, d_mom = torch.from_numpy(prop).to(cuda), torch.from_numpy(mom5).to(cuda)
    f = torch.ones(n, dtype=torch.float64, device=cuda)
    w = torch.ones((nt, nt, 48), dtype=torch.complex128, device=cuda)
    s = torch.cuda.Stream()
    torch.cuda.synchronize()
    g = api.Graph(s)
    with pytest.raises(CtrError):
        with g:
            api.rho_profile_vjp(d_prop, d_mom[:, :5].contiguous(), f, w, stream=s)
    assert lib().ctr_graph_end(ctypes.c_void_p(s.cuda_stream), ctypes.byref(ctypes.c_void_p())) != 0  # closed
    got = api.run_contract_rho(d_prop, d_mom, engine="fp64", stream=s)
    s.synchronize()
    ref = O.rho(prop, mom5)
    assert np.abs(got.cpu().numpy() - ref).max() / np.abs(ref).max() <= 1e-12


@pytest.mark.gpu
def test_autotuner_measures_and_candidates_agree(cuda):
    """Mode 1 measures the knobs on a live call; every candidate of every knob
    meets the oracle at the split engine's tolerance."""
    nt, n = 8, 24
    prop, mom5 = _rho_inputs(nt, n, seed=91)
    ref = O.rho(prop, mom5)
    d_prop, d_mom = torch.from_numpy(prop).to(cuda), torch.from_numpy(mom5).to(cuda)
    scale = np.abs(ref).max()
    try:
        api.tune_clear()
        api.tune_set_mode(1)
        got = api.run_contract_rho(d_prop, d_mom, engine="split").cpu().numpy()
        assert np.abs(got - ref).max() / scale <= 1e-9
        rep = api.tune_report()
        knobs = {k.split("|")[0] for k in rep}
        assert {"trace_rows", "split_gemm.order", "twosided.batch"} <= knobs, rep
        for k, v in rep.items():
            assert v["ms"] and all(x > 0 for x in v["ms"]), (k, v)
        api.tune_set_mode(0)
        for knob, values in (("trace_rows", range(12)), ("split_gemm.order", range(2)), ("slice_tau", range(3)),
                             ("twosided.batch", (1, 3, 64))):
            for v in values:
                api.tune_force(knob, v)
                got = api.run_contract_rho(d_prop, d_mom, engine="split").cpu().numpy()
                assert np.abs(got - ref).max() / scale <= 1e-9, (knob, v)
            api.tune_force(knob, -1)
    finally:
        api.tune_set_mode(0)
        api.tune_clear()


@pytest.mark.gpu
@pytest.mark.parametrize("n", [20, 37, 50, 72, 100, 128])
def test_fp64_gemm_tile_variants(cuda, n):
    """Every FP64 block-GEMM variant gives the oracle's rho to 1e-12: DFMA tile
    edges 32, 50, 20, and above Nev = 64 the FP64 matrix-instruction forms."""
    nt = 2
    prop, mom5 = _rho_inputs(nt, n, seed=404 + n)
    ref = O.rho(prop, mom5)
    d_prop, d_mom = torch.from_numpy(prop).to(cuda), torch.from_numpy(mom5).to(cuda)
    variants = [0, 1, 2] + ([3] if 64 < n <= 104 else []) + ([4] if n > 64 else [])
    try:
        for v in variants:
            api.tune_force("zgemm_f64.tile", v)
            got = api.run_contract_rho(d_prop, d_mom, engine="fp64").cpu().numpy()
            assert np.abs(got - ref).max() / np.abs(ref).max() <= 1e-12, v
    finally:
        api.tune_force("zgemm_f64.tile", -1)


@pytest.mark.gpu
def test_bounded_wait_runs_out_and_the_context_stays_usable(cuda):
    """Failure detection without a GPU fault: a device wait on an mbarrier that
    nothing arrives at gives up after 50 ms, the call reports CTR_ERR_TIMEOUT,
    and the next contraction on the same context is correct."""
    import ctypes
    import time
    from contractions_code_scattering_gb300._lib import lib
    s = torch.cuda.current_stream()
    t0 = time.perf_counter()
    rc = lib().ctr_wait_probe(50, ctypes.c_void_p(s.cuda_stream))
    dt = time.perf_counter() - t0
    assert rc == 5  # CTR_ERR_TIMEOUT
    assert b"timed out" in lib().ctr_last_error()
    assert 0.04 <= dt < 5.0
    assert lib().ctr_wait_probe(0, ctypes.c_void_p(s.cuda_stream)) != 0  # limits are checked
    nt, n = 3, 16
    prop, mom5 = _rho_inputs(nt, n, seed=505)
    ref = O.rho(prop, mom5)
    got = api.run_contract_rho(torch.from_numpy(prop).to(cuda), torch.from_numpy(mom5).to(cuda), engine="split")
    assert np.abs(got.cpu().numpy() - ref).max() / np.abs(ref).max() <= 1e-9
