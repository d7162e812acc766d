"""The allocation-free rho entry point, ctr_rho_noalloc.

Callers that cannot allocate device memory at call time use it.  Examples are
components that hand the device memory budget to a fixed pool at start-up, and
code that must not trigger the device synchronisation cudaMalloc/cudaFree may
cause.  Its scratch is a fixed device array inside libctr.so, shared by every
call.  It must give the oracle's correlators (the reference's rho algorithm in
FP64) on repeated calls that reuse that shared array, and a call must not
change the device's free memory.  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest
import torch

from contractions_code_scattering_gb300 import synth
from contractions_code_scattering_gb300._lib import check, lib
from tests.parity import entrywise, rho_rows_abs

pytestmark = pytest.mark.gpu

TOL = 1e-12  # the plain FP64 engine's tolerance, per entry


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _entry():
    L = lib()
    L.ctr_rho_noalloc.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                  ctypes.c_void_p, ctypes.c_void_p]
    L.ctr_rho_noalloc_scratch_bytes.restype = ctypes.c_size_t
    return L


def test_noalloc_matches_oracle_on_calls_in_a_row(cuda):
    from oracle import pyoracle as O
    L = _entry()
    nt, nev = 3, 100
    prop = synth.make_prop(nt, nev, seed=77)
    rng = np.random.default_rng(78)
    mom5 = np.ascontiguousarray(np.stack([synth.make_phi_random(nt, nev, rng) for _ in range(5)], axis=1))
    d_prop = torch.from_numpy(prop).to(cuda)
    d_mom = torch.from_numpy(mom5).to(cuda)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    first = {}
    for tf in (1, 2, 1):  # calls in a row through the shared scratch; t_sink 1 twice
        rows, ref = O.rho_row(prop, mom5, tf)
        row = d_prop[tf].contiguous()
        out = torch.full((nt, 16, 3), complex(np.nan, np.nan), dtype=torch.complex128, device=cuda)
        check(L.ctr_rho_noalloc(nev, nt, tf, _ptr(row), _ptr(d_mom), _ptr(out), stream))
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        entrywise(got, ref, TOL, rho_rows_abs(rows), "t_sink %d" % tf)
        if tf in first:
            assert np.array_equal(got, first[tf]), "a repeated call gave different bits"
        first[tf] = got


def test_noalloc_call_leaves_free_memory_unchanged(cuda):
    L = _entry()
    nt, nev = 2, 64
    prop = synth.make_prop(nt, nev, seed=5)
    rng = np.random.default_rng(6)
    mom5 = np.ascontiguousarray(np.stack([synth.make_phi_random(nt, nev, rng) for _ in range(5)], axis=1))
    row = torch.from_numpy(prop[0]).to(cuda).contiguous()
    d_mom = torch.from_numpy(mom5).to(cuda)
    out = torch.empty((nt, 16, 3), dtype=torch.complex128, device=cuda)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    check(L.ctr_rho_noalloc(nev, nt, 0, _ptr(row), _ptr(d_mom), _ptr(out), stream))  # warm-up
    torch.cuda.synchronize()
    # free device memory is a device-wide figure: take the best of a few tries
    # so that an unrelated change elsewhere on the device does not decide it
    same = False
    for _ in range(3):
        free0, _ = torch.cuda.mem_get_info()
        check(L.ctr_rho_noalloc(nev, nt, 0, _ptr(row), _ptr(d_mom), _ptr(out), stream))
        torch.cuda.synchronize()
        free1, _ = torch.cuda.mem_get_info()
        if free1 == free0:
            same = True
            break
    assert same, "free device memory changed across a call (%d -> %d bytes)" % (free0, free1)


def test_noalloc_rejects_sizes_beyond_its_scratch(cuda):
    L = _entry()
    assert L.ctr_rho_noalloc_scratch_bytes() == 32 << 20
    buf = torch.zeros(16, dtype=torch.complex128, device=cuda)
    rc = L.ctr_rho_noalloc(128, 2, 0, _ptr(buf), _ptr(buf), _ptr(buf), None)
    assert rc == 1
    assert b"fixed maximum" in L.ctr_last_error()
