"""Python host-side mirror of the reference's contraction launchers.

Each function takes device tensors (torch, complex128, contiguous, on the
current CUDA device) in the reference layouts and calls the C ABI of
libctr.so; the computation runs in the library's CUDA kernels.  Names and
argument meanings follow the reference's run_Contract* launchers
(include/contract.h:50-69) and Contract_* classes; errors raise CtrError
instead of terminating the process.
"""

import ctypes

import numpy as np

from ._lib import ENGINE_FP64, ENGINE_SPLIT, CtrError, check, lib

ENGINES = {"fp64": ENGINE_FP64, "split": ENGINE_SPLIT}


def _engine(e):
    if isinstance(e, int):
        return e
    try:
        return ENGINES[e]
    except KeyError:
        raise ValueError("engine must be one of %s" % list(ENGINES))


def _dev(t, name):
    import torch
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError("%s must be a CUDA tensor" % name)
    if t.dtype != torch.complex128:
        raise TypeError("%s must be complex128" % name)
    if not t.is_contiguous():
        raise ValueError("%s must be contiguous" % name)
    return ctypes.c_void_p(t.data_ptr())


def _stream(stream):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def _np_ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def device_init(device=0):
    check(lib().ctr_device_init(device))


def tables():
    """The diagram tables generated by the library, keyed by the reference's array names."""
    L = lib()
    out = {}
    s, lr, c = np.zeros((768, 4), np.int16), np.zeros((768, 2), np.int16), np.zeros((768, 2), np.float32)
    check(L.ctr_table_rho(_np_ptr(s), _np_ptr(lr), _np_ptr(c)))
    out.update(spinIndices_rho=s, lp_rp_rho=lr, coef_rho=c)
    s, ip, c = np.zeros((768, 6), np.int16), np.zeros((768,), np.int16), np.zeros((768, 2), np.float32)
    check(L.ctr_table_rhopi(_np_ptr(s), _np_ptr(ip), _np_ptr(c)))
    out.update(spinIndices_rhopi=s, ip_rhopi=ip, coef_rhopi=c)
    a = [np.zeros((256, 6), np.int16), np.zeros((256, 2), np.float32), np.zeros((256, 6), np.int16),
         np.zeros((256, 2), np.float32), np.zeros((256, 4), np.int16), np.zeros((256, 2), np.float32)]
    check(L.ctr_table_pipi(*[_np_ptr(x) for x in a]))
    out.update(spinIndices_pipi_square=a[0], coef_pipi_square=a[1], spinIndices_pipi_doubleTriangle=a[2],
               coef_pipi_doubleTriangle=a[3], spinIndices_pipi_doubleTriangle_hor=a[4],
               coef_pipi_doubleTriangle_hor=a[5])
    s, lr, c = np.zeros((64, 4), np.int16), np.zeros((64, 2), np.int16), np.zeros((64, 2), np.float32)
    check(L.ctr_table_sigma(_np_ptr(s), _np_ptr(lr), _np_ptr(c)))
    out.update(spinIndices_sigma=s, lp_rp_sigma=lr, coef_sigma=c)
    a = [np.zeros((16, 2), np.int16), np.zeros((16, 2), np.float32), np.zeros((128, 5), np.int16),
         np.zeros((128,), np.int16), np.zeros((128, 2), np.float32)]
    check(L.ctr_table_sigmapi(*[_np_ptr(x) for x in a]))
    out.update(spinIndices_sigmapi_hor_fish=a[0], coef_sigmapi_hor_fish=a[1], spinIndices_sigmapi_triangle=a[2],
               ip_sigmapi_triangle=a[3], coef_sigmapi_triangle=a[4])
    return out


def twosided(prop_rows, phi, rows, coef, out_index, nout, engine="fp64", tf_range=None, out=None, stream=None):
    """Generic two-sided contraction (include/ctr.h: ctr_twosided).

    prop_rows: [n_rows_held, Nt, 4, 4, N, N] tau rows for t_sink in tf_range;
    phi: [Nt, nphi, N, N]; rows: int16 [nrows, 6] = (a, b, c, d, L, R);
    coef: float32 [nrows, 2]; out_index: int32 [nrows].
    Returns out [n_rows_held, Nt, nout] complex128 (device)."""
    import torch
    nt, nev = phi.shape[0], phi.shape[-1]
    tf0, tf1 = tf_range if tf_range is not None else (0, nt)
    if out is None:
        out = torch.empty((tf1 - tf0, nt, nout), dtype=torch.complex128, device=phi.device)
    rows = np.ascontiguousarray(rows, np.int16)
    coef = np.ascontiguousarray(coef, np.float32)
    out_index = np.ascontiguousarray(out_index, np.int32)
    check(lib().ctr_twosided(_engine(engine), nev, nt, tf0, tf1, _dev(prop_rows, "prop_rows"), _dev(phi, "phi"),
                             phi.shape[1], rows.shape[0], _np_ptr(rows), _np_ptr(coef), _np_ptr(out_index), nout,
                             _dev(out, "out"), _stream(stream)))
    return out


def run_contract_rho(prop_rows, mom5, engine="fp64", tf_range=None, out=None, stream=None):
    """rho-rho for t_sink rows tf_range (run_ContractRho): corr [rows, Nt, 16, 3]."""
    import torch
    nt, nev = mom5.shape[0], mom5.shape[-1]
    tf0, tf1 = tf_range if tf_range is not None else (0, nt)
    if out is None:
        out = torch.empty((tf1 - tf0, nt, 16, 3), dtype=torch.complex128, device=mom5.device)
    check(lib().ctr_rho(_engine(engine), nev, nt, tf0, tf1, _dev(prop_rows, "prop_rows"), _dev(mom5, "mom5"),
                        _dev(out, "out"), _stream(stream)))
    return out


def run_contract_sigma(prop_rows, mom2, engine="fp64", tf_range=None, out=None, stream=None):
    """sigma-sigma one-fish for t_sink rows tf_range (run_ContractSigma): corr [rows, Nt, 4]."""
    import torch
    nt, nev = mom2.shape[0], mom2.shape[-1]
    tf0, tf1 = tf_range if tf_range is not None else (0, nt)
    if out is None:
        out = torch.empty((tf1 - tf0, nt, 4), dtype=torch.complex128, device=mom2.device)
    check(lib().ctr_sigma(_engine(engine), nev, nt, tf0, tf1, _dev(prop_rows, "prop_rows"), _dev(mom2, "mom2"),
                          _dev(out, "out"), _stream(stream)))
    return out


def prop_diag(prop):
    """tau(t,t) gathered on the device from the full perambulator [Nt,Nt,4,4,N,N]
    (LapH_prop::copyToDeviceExtraDiag, lib/contract.cpp:549-570)."""
    import torch
    nt = prop.shape[0]
    idx = torch.arange(nt, device=prop.device)
    return prop[idx, idx].contiguous()


def _rows(tf_range, nt):
    return tf_range if tf_range is not None else (0, nt)


def run_contract_rhopi(prop_rows, diag, p1, p2, mom5_p1p2, idir, engine="fp64", tf_range=None, out=None,
                       stream=None):
    """rho -> pi pi (run_ContractRhoPi): corr [rows, Nt, 4]."""
    import torch
    nt, nev = p1.shape[0], p1.shape[-1]
    tf0, tf1 = _rows(tf_range, nt)
    if out is None:
        out = torch.empty((tf1 - tf0, nt, 4), dtype=torch.complex128, device=p1.device)
    check(lib().ctr_rhopi(_engine(engine), nev, nt, tf0, tf1, idir, _dev(prop_rows, "prop_rows"), _dev(diag, "diag"),
                          _dev(p1, "p1"), _dev(p2, "p2"), _dev(mom5_p1p2, "mom5_p1p2"), _dev(out, "out"),
                          _stream(stream)))
    return out


def run_contract_pipi(prop_rows, diag, p1, p2, p3, p4, isospin, engine="fp64", tf_range=None, out=None,
                      stream=None):
    """pi pi -> pi pi (run_ContractPiPi / run_ContractPiPi_I0; isospin 1 or 0): corr [rows, Nt, 5]."""
    import torch
    nt, nev = p1.shape[0], p1.shape[-1]
    tf0, tf1 = _rows(tf_range, nt)
    if out is None:
        out = torch.empty((tf1 - tf0, nt, 5), dtype=torch.complex128, device=p1.device)
    check(lib().ctr_pipi(_engine(engine), nev, nt, tf0, tf1, isospin, _dev(prop_rows, "prop_rows"), _dev(diag, "diag"),
                         _dev(p1, "p1"), _dev(p2, "p2"), _dev(p3, "p3"), _dev(p4, "p4"), _dev(out, "out"),
                         _stream(stream)))
    return out


def run_contract_pipi_sets(prop_rows, diag, phi, sets, isospin, engine="fp64", tf_range=None, out=None, stream=None):
    """pi pi for many momentum sets in one call (include/ctr.h: ctr_pipi_sets).

    phi: [Nt, nphi, N, N] every elemental; sets: [nset, 4] indices of P1..P4 into
    phi's second axis.  Returns corr [nset, rows, Nt, 5] (device)."""
    import torch
    nt, nphi, nev = phi.shape[0], phi.shape[1], phi.shape[-1]
    sets = np.ascontiguousarray(np.asarray(sets, dtype=np.int32).reshape(-1, 4))
    tf0, tf1 = _rows(tf_range, nt)
    if out is None:
        out = torch.empty((len(sets), tf1 - tf0, nt, 5), dtype=torch.complex128, device=phi.device)
    check(lib().ctr_pipi_sets(_engine(engine), nev, nt, tf0, tf1, isospin, _dev(prop_rows, "prop_rows"),
                              _dev(diag, "diag"), _dev(phi, "phi"), nphi, len(sets), _np_ptr(sets), _dev(out, "out"),
                              _stream(stream)))
    return out


def run_contract_rhopi_sigmapi_sets(prop_rows, diag, phi, sets, mom5=None, mom2=None, engine="fp64", tf_range=None,
                                    rhopi=True, triangle=True, hor_fish=True, out=None, stream=None):
    """rho -> pi pi (3 polarisations) and sigma -> pi pi for many pion pairs in one call
    (include/ctr.h: ctr_rhopi_sigmapi_sets).  phi: [Nt, nphi, N, N]; sets: [nset, 2]
    indices of (P1, P2); mom5 [Nt, 5, N, N], mom2 [Nt, 2, N, N].  Returns a dict with
    'rhopi' [nset, 3, rows, Nt, 4], 'triangle' [nset, rows, Nt, 2], 'hor_fish' [nset, Nt]
    for the outputs requested (device); out: a dict of such tensors to fill instead."""
    import torch
    nt, nphi, nev = phi.shape[0], phi.shape[1], phi.shape[-1]
    sets = np.ascontiguousarray(np.asarray(sets, dtype=np.int32).reshape(-1, 2))
    ns = len(sets)
    tf0, tf1 = _rows(tf_range, nt)
    kw = dict(dtype=torch.complex128, device=phi.device)
    if out is None:
        out = {}
        if rhopi:
            out["rhopi"] = torch.empty((ns, 3, tf1 - tf0, nt, 4), **kw)
        if triangle:
            out["triangle"] = torch.empty((ns, tf1 - tf0, nt, 2), **kw)
        if hor_fish:
            out["hor_fish"] = torch.empty((ns, nt), **kw)
    opt = lambda t, name: _dev(t, name) if t is not None else None
    check(lib().ctr_rhopi_sigmapi_sets(_engine(engine), nev, nt, tf0, tf1,
                                       opt(prop_rows, "prop_rows") if (rhopi or triangle) else None, _dev(diag, "diag"),
                                       _dev(phi, "phi"), nphi, opt(mom5, "mom5"), opt(mom2, "mom2"), ns, _np_ptr(sets),
                                       opt(out.get("rhopi"), "rhopi"), opt(out.get("triangle"), "triangle"),
                                       opt(out.get("hor_fish"), "hor_fish"), _stream(stream)))
    return out


def run_contract_loop_unity(diag, mom, engine="fp64", out=None, stream=None):
    """Loop-unity (run_ContractLoopUnity): loop [Nt]."""
    import torch
    nt, nev = mom.shape[0], mom.shape[-1]
    if out is None:
        out = torch.empty((nt,), dtype=torch.complex128, device=mom.device)
    check(lib().ctr_loop_unity(_engine(engine), nev, nt, _dev(diag, "diag"), _dev(mom, "mom"), _dev(out, "out"),
                               _stream(stream)))
    return out


def run_contract_sigmapi(prop_rows, diag, p1, p2, mom2_p1p2, engine="fp64", tf_range=None, out=None, stream=None):
    """sigma -> pi pi (hor fish + triangle): (hor_fish [Nt], triangle [rows, Nt, 2]); out = (hf, tri) or None."""
    import torch
    nt, nev = p1.shape[0], p1.shape[-1]
    tf0, tf1 = _rows(tf_range, nt)
    if out is None:
        out = (torch.empty((nt,), dtype=torch.complex128, device=p1.device),
               torch.empty((tf1 - tf0, nt, 2), dtype=torch.complex128, device=p1.device))
    hf, tri = out
    check(lib().ctr_sigmapi(_engine(engine), nev, nt, tf0, tf1, _dev(prop_rows, "prop_rows"), _dev(diag, "diag"),
                            _dev(p1, "p1"), _dev(p2, "p2"), _dev(mom2_p1p2, "mom2_p1p2"), _dev(hf, "hor_fish"),
                            _dev(tri, "triangle"), _stream(stream)))
    return hf, tri


def zgemm_batched(x, y, engine="fp64", out=None, stream=None):
    """Block products out[b] = x[b] @ y[b] for device tensors [nb, N, N] complex128."""
    import torch
    nb, n = x.shape[0], x.shape[-1]
    if out is None:
        out = torch.empty_like(x)
    for t, nm in ((x, "x"), (y, "y"), (out, "out")):
        _dev(t, nm)
    stride = n * n * 16
    px = (ctypes.c_void_p * nb)(*[x.data_ptr() + b * stride for b in range(nb)])
    py = (ctypes.c_void_p * nb)(*[y.data_ptr() + b * stride for b in range(nb)])
    pc = (ctypes.c_void_p * nb)(*[out.data_ptr() + b * stride for b in range(nb)])
    check(lib().ctr_zgemm_batched(_engine(engine), n, nb, px, py, pc, _stream(stream)))
    return out


class Graph:
    """Library calls recorded once on a stream and replayed (include/ctr.h: ctr_graph_*).

        corr = torch.empty(...)           # outputs allocated before recording
        with api.Graph(stream) as g:      # records; nothing executes
            api.run_contract_rho(prop_rows, mom5, engine="split", out=corr, stream=stream)
        g.launch(stream)                  # replays; any number of times

    A replay reads the device tensors passed while recording (with the contents
    they hold at replay time) and writes the same outputs, so keep them alive
    and refill them in place.  Allocate every tensor before recording (pass
    out=): the stream is capturing while the block runs.  The split engine's recomputation of
    ill-conditioned entries runs between graph segments at every launch."""

    def __init__(self, stream=None):
        self._stream = stream
        self._g = None

    def __enter__(self):
        check(lib().ctr_graph_begin(_stream(self._stream)))
        return self

    def __exit__(self, exc_type, exc, tb):
        g = ctypes.c_void_p()
        rc = lib().ctr_graph_end(_stream(self._stream), ctypes.byref(g))
        if exc_type is None:
            check(rc)
            self._g = g
        return False

    def launch(self, stream=None):
        if self._g is None:
            raise CtrError(-1, "graph was not recorded")
        check(lib().ctr_graph_launch(self._g, _stream(stream if stream is not None else self._stream)))

    def info(self):
        """(segments, kernel nodes per replay, device bytes owned)."""
        ns, nk, nb = ctypes.c_int(), ctypes.c_longlong(), ctypes.c_longlong()
        check(lib().ctr_graph_info(self._g, ctypes.byref(ns), ctypes.byref(nk), ctypes.byref(nb)))
        return ns.value, nk.value, nb.value

    def close(self):
        if self._g is not None:
            lib().ctr_graph_destroy(self._g)
            self._g = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def tune_set_mode(mode):
    """0: cached choices or defaults; 1: measure keys met for the first time; 2: re-measure."""
    check(lib().ctr_tune_set_mode(int(mode)))


def tune_force(knob, value):
    """Pin a knob ("twosided.batch", "trace_rows", "slice_tau", "split_gemm.order", "zgemm_f64.tile") to a value; -1 releases it."""
    check(lib().ctr_tune_force(knob.encode(), int(value)))


def tune_report():
    """{"knob|shape": {"choice": c, "ms": [...]}} of the autotuner's table."""
    import json
    buf = ctypes.create_string_buffer(1 << 16)
    check(lib().ctr_tune_report(buf, len(buf)))
    return json.loads(buf.value.decode())


def tune_clear():
    lib().ctr_tune_clear()


def tune_save(path):
    check(lib().ctr_tune_save(str(path).encode()))


def tune_load(path):
    check(lib().ctr_tune_load(str(path).encode()))


def mma_schedule_probe(hp=False, nchunk=20000, stream=None):
    """The split GEMM's per-chunk MMA schedule by itself on every SM (include/ctr.h:
    ctr_mma_schedule_probe): returns (SM clocks per MMA, device BF16 TFLOP/s)."""
    cpm, tf = ctypes.c_double(), ctypes.c_double()
    check(lib().ctr_mma_schedule_probe(1 if hp else 0, int(nchunk), ctypes.byref(cpm), ctypes.byref(tf), _stream(stream)))
    return cpm.value, tf.value


def sync(stream=None):
    """Synchronise the stream and raise if a device-side wait of the split engine timed out."""
    check(lib().ctr_sync(_stream(stream)))


def source_average(corr, scale=1.0, stream=None):
    """dumpData's average over source times: [Nt, Nt, ...] -> [Nt, ...] (device)."""
    import torch
    nt = corr.shape[0]
    tail = tuple(corr.shape[2:])
    nc = int(np.prod(tail)) if tail else 1
    avg = torch.empty((nt,) + tail, dtype=torch.complex128, device=corr.device)
    check(lib().ctr_source_average(nt, nc, _dev(corr, "corr"), float(scale), _dev(avg, "avg"), _stream(stream)))
    return avg


def rho_rows_for_momenta(nmom, ico=0):
    """Two-sided rows of the rho two-point with op pair `ico` for `nmom`
    elementals stacked on the phi axis (one momentum each): returns
    (rows [nmom*48, 6], coef, out_index) with out index = p*3 + polarisation."""
    t = tables()
    spin, lprp, coef = t["spinIndices_rho"], t["lp_rp_rho"], t["coef_rho"]
    sel = np.arange(ico * 48, ico * 48 + 48)
    rows, cf, oi = [], [], []
    for p in range(nmom):
        for r in sel:
            s = spin[r]
            rows.append((s[0], s[1], s[2], s[3], p, p))
            cf.append(coef[r])
            oi.append(p * 3 + (r % 48) // 16)
    return np.array(rows, np.int16), np.array(cf, np.float32), np.array(oi, np.int32)


__all__ = ["CtrError", "device_init", "tables", "twosided", "run_contract_rho", "run_contract_sigma",
           "source_average", "rho_rows_for_momenta", "ENGINES"]


def split_levels(x, y, stream=None):
    """Diagnostics: raw tensor-core accumulators of the split product x @ y
    ([N,N] complex128 device tensors) -> float32 [8, N, N] (Re levels 0, 1, 2, >=3, then Im)."""
    import torch
    n = x.shape[-1]
    lv = torch.zeros((8, n, 128), dtype=torch.float32, device=x.device)
    check(lib().ctr_split_levels(n, _dev(x, "x"), _dev(y, "y"), ctypes.c_void_p(lv.data_ptr()), _stream(stream)))
    sync(stream)
    return lv[:, :, :n].transpose(1, 2)


# ------------------------------------------------------ distillation profile
FACTOR_TAU, FACTOR_PHI = 0, 1


class ctr_factor(ctypes.Structure):
    """One chain factor (include/ctr.h): tau(a, b)_{s1 s2} or diag(f) phi[a][b] diag(f)."""
    _fields_ = [("kind", ctypes.c_int32), ("dag", ctypes.c_int32), ("a", ctypes.c_int32), ("b", ctypes.c_int32),
                ("s1", ctypes.c_int32), ("s2", ctypes.c_int32)]


def _real(t, name):
    import torch
    if not isinstance(t, torch.Tensor) or not t.is_cuda or t.dtype != torch.float64 or not t.is_contiguous():
        raise TypeError("%s must be a contiguous float64 CUDA tensor" % name)
    return ctypes.c_void_p(t.data_ptr())


def apply_profile(f, phi, out=None, stream=None):
    """diag(f) phi[m] diag(f) for every matrix of phi [..., N, N] (device)."""
    import torch
    if out is None:
        out = torch.empty_like(phi)
    n = phi.shape[-1]
    check(lib().ctr_apply_profile(n, phi.numel() // (n * n), _real(f, "f"), _dev(phi, "phi"), _dev(out, "out"),
                                  _stream(stream)))
    return out


def chain_adjoint(prop, phi, f, chains, weights=None, values=True, grad=True, engine="fp64", stream=None):
    """Generic chain traces and their profile gradient (include/ctr.h: ctr_chain_adjoint).

    chains: list of lists of (kind, dag, a, b, s1, s2); weights: complex per chain.
    Returns (values [nchain] complex128 or None, grad [N] float64 or None)."""
    import torch
    nt, nev = prop.shape[0], prop.shape[-1]
    nphi = phi.shape[1] if phi is not None else 0
    off = np.zeros(len(chains) + 1, np.int32)
    flat = []
    for c, ch in enumerate(chains):
        off[c + 1] = off[c] + len(ch)
        flat += [ctr_factor(*fa) for fa in ch]
    fac = (ctr_factor * max(1, len(flat)))(*flat)
    w = None
    if weights is not None:
        w = np.ascontiguousarray(np.asarray(weights, np.complex128))
    vals = torch.zeros(len(chains), dtype=torch.complex128, device=prop.device) if values else None
    g = torch.zeros(nev, dtype=torch.float64, device=prop.device) if grad else None
    check(lib().ctr_chain_adjoint(_engine(engine), nev, nt, nphi, _dev(prop, "prop"), _dev(phi, "phi") if phi is not None else None,
                                  _real(f, "f"), len(chains), _np_ptr(off), ctypes.cast(fac, ctypes.c_void_p),
                                  _np_ptr(w) if w is not None else None,
                                  _dev(vals, "values") if vals is not None else None,
                                  _real(g, "grad") if g is not None else None, _stream(stream)))
    return vals, g


def rho_profile_vjp(prop, mom5, f, w, corr=True, grad=True, engine="fp64", stream=None):
    """rho-rho with profiled elementals: forward correlators [Nt, Nt, 48] of the entries
    with nonzero weight w [Nt, Nt, 48] (complex, device) and grad [N] = Re sum w dcorr/df."""
    import torch
    nt, nev = prop.shape[0], prop.shape[-1]
    c = torch.zeros((nt, nt, 48), dtype=torch.complex128, device=prop.device) if corr else None
    g = torch.zeros(nev, dtype=torch.float64, device=prop.device) if grad else None
    check(lib().ctr_rho_profile_vjp(_engine(engine), nev, nt, _dev(prop, "prop"), _dev(mom5, "mom5"), _real(f, "f"),
                                    _dev(w.contiguous(), "w"), _dev(c, "corr") if c is not None else None,
                                    _real(g, "grad") if g is not None else None, _stream(stream)))
    return c, g


def pipi_profile_vjp(prop, p1, p2, p3, p4, f, w, isospin, corr=True, grad=True, engine="fp64", stream=None):
    """pi pi with profiled elementals: forward correlators [Nt, Nt, 5] (isospin-weighted
    square, double triangle, star, fish, horizontal double triangle) of the pairs with
    nonzero weight w [Nt, Nt, 5] and grad [N] = Re sum w dcorr/df."""
    import torch
    nt, nev = prop.shape[0], prop.shape[-1]
    c = torch.zeros((nt, nt, 5), dtype=torch.complex128, device=prop.device) if corr else None
    g = torch.zeros(nev, dtype=torch.float64, device=prop.device) if grad else None
    check(lib().ctr_pipi_profile_vjp(_engine(engine), nev, nt, isospin, _dev(prop, "prop"), _dev(p1, "p1"), _dev(p2, "p2"),
                                     _dev(p3, "p3"), _dev(p4, "p4"), _real(f, "f"), _dev(w.contiguous(), "w"),
                                     _dev(c, "corr") if c is not None else None,
                                     _real(g, "grad") if g is not None else None, _stream(stream)))
    return c, g


class ctr_ztask(ctypes.Structure):
    """One multi-term block product (include/ctr.h)."""
    _fields_ = [("a", ctypes.c_void_p * 4), ("b", ctypes.c_void_p * 4), ("c", ctypes.c_void_p),
                ("wre", ctypes.c_float * 4), ("wim", ctypes.c_float * 4), ("nterm", ctypes.c_int),
                ("flags", ctypes.c_int)]


def zgemm_tasks(x, y, tasks, weights=None, a_dagger=False, b_dagger=False, engine="fp64", out=None, stream=None):
    """out[c] = sum_q w_q op(x[a_q]) op(y[b_q]) for tasks (a_list, b_list, c) on blocks of
    x, y [nb, N, N] (device complex128); weights per term (real), op = conjugate transpose
    where requested (include/ctr.h: ctr_zgemm_tasks)."""
    import torch
    n = x.shape[-1]
    _dev(x, "x")
    _dev(y, "y")
    nc = 1 + max(t[2] for t in tasks)
    if out is None:
        out = torch.zeros((nc, n, n), dtype=torch.complex128, device=x.device)
    stride = n * n * 16
    arr = (ctr_ztask * len(tasks))()
    for i, (al, bl, c) in enumerate(tasks):
        z = arr[i]
        z.nterm = len(al)
        flags = 0
        for q, (a, b) in enumerate(zip(al, bl)):
            z.a[q] = x.data_ptr() + a * stride
            z.b[q] = y.data_ptr() + b * stride
            z.wre[q] = 1.0 if weights is None else float(weights[q])
            flags |= (1 << q if a_dagger else 0) | (1 << (4 + q) if b_dagger else 0)
        z.flags = flags
        z.c = out.data_ptr() + c * stride
    check(lib().ctr_zgemm_tasks(_engine(engine), n, len(tasks), ctypes.cast(arr, ctypes.c_void_p), _stream(stream)))
    return out


def elementals(evec, moms, links=None, nops=None, out=None, stream=None):
    """Momentum elementals from Laplacian eigenvectors (include/ctr.h:
    ctr_elementals; the drivers' loops, tests/compute_rho.cpp:116-223).
    evec [nt, nev, nz, ny, nx, 3] and links [nt, nz, ny, nx, 3, 3, 3] are device
    complex128; moms is a list of integer 3-momenta.  Returns
    [nmom, nops, nt, nev, nev] (nops = 5 with links, else 1)."""
    import torch
    nt, nev, nz, ny, nx, nc = evec.shape
    if nc != 3:
        raise ValueError("evec must be [nt, nev, nz, ny, nx, 3]")
    _dev(evec, "evec")
    if nops is None:
        nops = 5 if links is not None else 1
    lp = None
    if links is not None:
        if tuple(links.shape) != (nt, nz, ny, nx, 3, 3, 3):
            raise ValueError("links must be [nt, nz, ny, nx, 3, 3, 3]")
        lp = _dev(links, "links")
    m = np.ascontiguousarray(np.asarray(moms, dtype=np.int32).reshape(-1, 3))
    if out is None:
        out = torch.empty((len(m), nops, nt, nev, nev), dtype=torch.complex128, device=evec.device)
    check(lib().ctr_elementals(nev, nt, nx, ny, nz, _dev(evec, "evec"), lp, len(m), _np_ptr(m), nops,
                               _dev(out, "out"), _stream(stream)))
    return out
