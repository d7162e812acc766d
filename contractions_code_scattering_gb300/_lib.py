"""ctypes binding of libctr.so (the C ABI declared in include/ctr.h).

The library is loaded from the package directory.  If it is missing, importing
the binding fails loudly: there is no CPU or PyTorch fallback for the engine.
"""

import ctypes
import os

from . import _build

_LIB = None

CTR_OK = 0
ENGINE_FP64 = 0
ENGINE_SPLIT = 1


class CtrError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("ctr error %d: %s" % (code, msg))
        self.code = code


def lib(build_if_missing=True):
    """Load libctr.so (building it in-tree first if asked and absent)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise CtrError(-1, "libctr.so is not built (run __graft_entry__.build())")
        _build.build()
    L = ctypes.CDLL(path)
    vp, i, d = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    L.ctr_version.restype = i
    L.ctr_last_error.restype = ctypes.c_char_p
    L.ctr_error_string.restype = ctypes.c_char_p
    L.ctr_error_string.argtypes = [i]
    L.ctr_device_init.argtypes = [i]
    for name in ("ctr_table_rho", "ctr_table_rhopi", "ctr_table_sigma"):
        getattr(L, name).argtypes = [vp, vp, vp]
    L.ctr_table_pipi.argtypes = [vp] * 6
    L.ctr_table_sigmapi.argtypes = [vp] * 5
    L.ctr_twosided.argtypes = [i, i, i, i, i, vp, vp, i, i, vp, vp, vp, i, vp, vp]
    L.ctr_rho.argtypes = [i, i, i, i, i, vp, vp, vp, vp]
    L.ctr_sigma.argtypes = [i, i, i, i, i, vp, vp, vp, vp]
    L.ctr_source_average.argtypes = [i, i, vp, d, vp, vp]
    L.ctr_sync.argtypes = [vp]
    L.ctr_zgemm_batched.argtypes = [i, i, i, vp, vp, vp, vp]
    L.ctr_split_levels.argtypes = [i, vp, vp, vp, vp]
    L.ctr_rhopi.argtypes = [i, i, i, i, i, i, vp, vp, vp, vp, vp, vp, vp]
    L.ctr_pipi.argtypes = [i, i, i, i, i, i, vp, vp, vp, vp, vp, vp, vp, vp]
    L.ctr_pipi_sets.argtypes = [i, i, i, i, i, i, vp, vp, vp, i, i, vp, vp, vp]
    L.ctr_rhopi_sigmapi_sets.argtypes = [i, i, i, i, i, vp, vp, vp, i, vp, vp, i, vp, vp, vp, vp, vp]
    L.ctr_loop_unity.argtypes = [i, i, i, vp, vp, vp, vp]
    L.ctr_sigmapi.argtypes = [i, i, i, i, i, vp, vp, vp, vp, vp, vp, vp, vp]
    L.ctr_split_available.restype = i
    L.ctr_release_workspace.restype = None
    L.ctr_timing_enable.argtypes = [i]
    L.ctr_timing_enable.restype = None
    L.ctr_launch_count.restype = ctypes.c_longlong
    L.ctr_timing_report.argtypes = [ctypes.c_char_p, i]
    L.ctr_zgemm_tasks.argtypes = [i, i, i, vp, vp]
    L.ctr_elementals.argtypes = [i, i, i, i, i, vp, vp, i, vp, i, vp, vp]
    L.ctr_wait_probe.argtypes = [i, vp]
    L.ctr_mma_schedule_probe.argtypes = [i, i, ctypes.POINTER(d), ctypes.POINTER(d), vp]
    L.ctr_split_set_refine.argtypes = [d]
    L.ctr_split_refined.restype = ctypes.c_longlong
    L.ctr_split_flops.argtypes = [ctypes.POINTER(d), ctypes.POINTER(d), i]
    L.ctr_gram_flops.argtypes = [ctypes.POINTER(d), ctypes.POINTER(d), i]
    L.ctr_apply_profile.argtypes = [i, ctypes.c_longlong, vp, vp, vp, vp]
    L.ctr_chain_adjoint.argtypes = [i, i, i, i, vp, vp, vp, i, vp, vp, vp, vp, vp, vp]
    L.ctr_rho_profile_vjp.argtypes = [i, i, i, vp, vp, vp, vp, vp, vp, vp]
    L.ctr_pipi_profile_vjp.argtypes = [i, i, i, i, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp]
    L.ctr_graph_begin.argtypes = [vp]
    L.ctr_graph_end.argtypes = [vp, ctypes.POINTER(vp)]
    L.ctr_graph_launch.argtypes = [vp, vp]
    L.ctr_graph_info.argtypes = [vp, ctypes.POINTER(i), ctypes.POINTER(ctypes.c_longlong),
                                 ctypes.POINTER(ctypes.c_longlong)]
    L.ctr_graph_destroy.argtypes = [vp]
    L.ctr_graph_destroy.restype = None
    L.ctr_tune_set_mode.argtypes = [i]
    L.ctr_tune_force.argtypes = [ctypes.c_char_p, i]
    L.ctr_tune_report.argtypes = [ctypes.c_char_p, i]
    L.ctr_tune_clear.restype = None
    L.ctr_tune_save.argtypes = [ctypes.c_char_p]
    L.ctr_tune_load.argtypes = [ctypes.c_char_p]
    _LIB = L
    return L


def exported_functions():
    """Names of every function declared in include/*.h (for the ABI check)."""
    import re
    root = os.path.dirname(_build.PKG)
    names = []
    inc = os.path.join(root, "include")
    for f in sorted(os.listdir(inc)):
        if not f.endswith(".h"):
            continue
        txt = open(os.path.join(inc, f)).read()
        if 'extern "C"' not in txt:
            continue
        body = txt.split('extern "C"', 1)[1]
        names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(ctr_\w+)\s*\(", body, re.M)
    return sorted(set(names))


def check(rc):
    if rc != CTR_OK:
        L = lib()
        raise CtrError(rc, L.ctr_last_error().decode(errors="replace"))
    return rc


def timing_enable(on=True):
    lib().ctr_timing_enable(1 if on else 0)


def launch_count():
    return int(lib().ctr_launch_count())


def timing_report():
    """{kernel: (launches, timed_launches, total_ms)} since the last timing_enable()."""
    import json
    buf = ctypes.create_string_buffer(1 << 16)
    check(lib().ctr_timing_report(buf, len(buf)))
    return {k: tuple(v) for k, v in json.loads(buf.value.decode()).items()}


def split_flops(reset=False):
    """(executed BF16 MMA flops, complex block products) of the split engine's eager
    launches since the last reset (include/ctr.h: ctr_split_flops)."""
    a, b = ctypes.c_double(), ctypes.c_double()
    check(lib().ctr_split_flops(ctypes.byref(a), ctypes.byref(b), 1 if reset else 0))
    return a.value, b.value


def gram_flops(reset=False):
    """(executed BF16 MMA flops, closing traces) of the split engine's Gram-product
    trace launches since the last reset (include/ctr.h: ctr_gram_flops)."""
    a, b = ctypes.c_double(), ctypes.c_double()
    check(lib().ctr_gram_flops(ctypes.byref(a), ctypes.byref(b), 1 if reset else 0))
    return a.value, b.value
