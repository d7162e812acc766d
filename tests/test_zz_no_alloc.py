"""The allocation-free rho entry point, ctr_rho_noalloc.

Callers that cannot allocate device memory at call time use it.  Examples are
components that hand the device memory budget to a fixed pool at start-up, and
code that must not trigger the device synchronisation cudaMalloc/cudaFree may
cause.  Its scratch is a fixed device array inside libctr.so.  It must give the
same correlators as ctr_rho (plain FP64 engine), and keep doing so on repeated
calls that reuse that shared array.  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest
import torch

from contractions_code_scattering_gb300 import api, synth
from contractions_code_scattering_gb300._lib import check, lib

pytestmark = pytest.mark.gpu

TOL = 1e-12  # the plain FP64 engine's tolerance


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def test_noalloc_matches_rho_on_two_calls(cuda):
    L = lib()
    L.ctr_rho_noalloc.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                  ctypes.c_void_p, ctypes.c_void_p]
    nt, nev = 3, 100
    prop = synth.make_prop(nt, nev, seed=77)
    rng = np.random.default_rng(78)
    mom5 = np.ascontiguousarray(np.stack([synth.make_phi_random(nt, nev, rng) for _ in range(5)], axis=1))
    d_prop = torch.from_numpy(prop).to(cuda)
    d_mom = torch.from_numpy(mom5).to(cuda)
    ref = api.run_contract_rho(d_prop, d_mom, engine="fp64").cpu().numpy()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for tf in (1, 2):  # two calls in a row, both through the shared scratch
        row = d_prop[tf].contiguous()
        out = torch.full((nt, 16, 3), complex(np.nan, np.nan), dtype=torch.complex128, device=cuda)
        check(L.ctr_rho_noalloc(nev, nt, tf, _ptr(row), _ptr(d_mom), _ptr(out), stream))
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        err = np.abs(got - ref[tf]).max() / np.abs(ref[tf]).max()
        assert err <= TOL, "t_sink %d: error %.3e" % (tf, err)


def test_noalloc_rejects_sizes_beyond_its_scratch(cuda):
    L = lib()
    L.ctr_rho_noalloc.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                  ctypes.c_void_p, ctypes.c_void_p]
    L.ctr_rho_noalloc_scratch_bytes.restype = ctypes.c_size_t
    assert L.ctr_rho_noalloc_scratch_bytes() == 32 << 20
    buf = torch.zeros(16, dtype=torch.complex128, device=cuda)
    rc = L.ctr_rho_noalloc(128, 2, 0, _ptr(buf), _ptr(buf), _ptr(buf), None)
    assert rc == 1
    assert b"fixed maximum" in L.ctr_last_error()
