"""Run the reference's own CUDA kernels (test infrastructure: pins the oracle).

The reference's device code (lib/contract_kernels_*.cu with the
lib/calculate_*_core.h bodies) is compiled, unmodified, from its sources into
cubins by ``oracle/build_ref.sh`` (outputs in oracle/_ref/, not committed).  This
module loads those cubins with the CUDA driver API through ctypes and drives
the kernels the way the reference's launchers do (grid 768/256/Nt*256 ...,
25x25 threads, texture objects over linear memory holding int4-viewed doubles,
tables in __constant__ memory), then applies the launchers' host reductions.
The reference hard-codes NSIZE = 100, so only Nev = 100 runs.

Only tests/golden/make_ref_fixtures.py uses this, to record the reference's
outputs as golden vectors; nothing on the product path does.
"""

import ctypes
import os
import struct

import numpy as np

from . import tables as T

_HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(_HERE, "_ref")
NSIZE = 100

_cu = None


def _driver():
    global _cu
    if _cu is None:
        _cu = ctypes.CDLL("libcuda.so.1")
    return _cu


def _ck(rc, what):
    if rc != 0:
        msg = ctypes.c_char_p()
        _driver().cuGetErrorString(rc, ctypes.byref(msg))
        raise RuntimeError("%s failed: %d %s" % (what, rc, msg.value))


def elf_function_names(path):
    """Names of the FUNC symbols in an ELF file built here (the cubin's kernel entry names)."""
    data = open(path, "rb").read()
    if data[:4] != b"\x7fELF" or data[4] != 2:
        raise ValueError("not an ELF64 file: %s" % path)
    shoff = struct.unpack_from("<Q", data, 0x28)[0]
    shentsize, shnum = struct.unpack_from("<HH", data, 0x3A)
    secs = [struct.unpack_from("<IIQQQQIIQQ", data, shoff + i * shentsize) for i in range(shnum)]
    names = []
    for s in secs:
        if s[1] == 2:  # SHT_SYMTAB
            off, size, link, entsize = s[4], s[5], s[6], s[9]
            stroff = secs[link][4]
            for k in range(size // entsize):
                st_name, st_info = struct.unpack_from("<IB", data, off + k * entsize)
                if (st_info & 0xF) == 2 and st_name:
                    end = data.index(b"\x00", stroff + st_name)
                    names.append(data[stroff + st_name:end].decode())
    return names


class _ResDesc(ctypes.Structure):
    _fields_ = [("resType", ctypes.c_int), ("pad0", ctypes.c_int), ("devPtr", ctypes.c_uint64),
                ("format", ctypes.c_int), ("numChannels", ctypes.c_uint), ("sizeInBytes", ctypes.c_size_t),
                ("reserved", ctypes.c_int * 26), ("flags", ctypes.c_uint), ("pad1", ctypes.c_uint)]


class _TexDesc(ctypes.Structure):
    _fields_ = [("addressMode", ctypes.c_int * 3), ("filterMode", ctypes.c_int), ("flags", ctypes.c_uint),
                ("maxAnisotropy", ctypes.c_uint), ("mipmapFilterMode", ctypes.c_int),
                ("mipmapLevelBias", ctypes.c_float), ("minMipmapLevelClamp", ctypes.c_float),
                ("maxMipmapLevelClamp", ctypes.c_float), ("borderColor", ctypes.c_float * 4),
                ("reserved", ctypes.c_int * 12)]


assert ctypes.sizeof(_ResDesc) == 144 and ctypes.sizeof(_TexDesc) == 104


class RefModule:
    """One reference cubin: kernels by (unmangled) name, __constant__ uploads, launches."""

    def __init__(self, cubin):
        import torch
        torch.cuda.init()
        torch.zeros(1, device="cuda")  # primary context current on this thread
        self.cu = _driver()
        self.mod = ctypes.c_void_p()
        _ck(self.cu.cuModuleLoad(ctypes.byref(self.mod), cubin.encode()), "cuModuleLoad(%s)" % cubin)
        self.names = elf_function_names(cubin)

    def kernel(self, needle):
        cands = [n for n in self.names if needle in n]
        if len(cands) != 1:
            raise KeyError("kernel %r: candidates %s" % (needle, cands))
        f = ctypes.c_void_p()
        _ck(self.cu.cuModuleGetFunction(ctypes.byref(f), self.mod, cands[0].encode()), "cuModuleGetFunction")
        return f

    def set_constant(self, name, arr):
        arr = np.ascontiguousarray(arr)
        dptr, size = ctypes.c_uint64(), ctypes.c_size_t()
        _ck(self.cu.cuModuleGetGlobal_v2(ctypes.byref(dptr), ctypes.byref(size), self.mod, name.encode()),
            "cuModuleGetGlobal(%s)" % name)
        if size.value != arr.nbytes:
            raise ValueError("%s: symbol %d bytes, table %d bytes" % (name, size.value, arr.nbytes))
        _ck(self.cu.cuMemcpyHtoD_v2(dptr, arr.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(arr.nbytes)),
            "cuMemcpyHtoD")

    def launch(self, f, grid, args):
        """args: list of ctypes values (pointers as c_uint64, textures as c_uint64, ints as c_int)."""
        ptrs = (ctypes.c_void_p * len(args))(*[ctypes.cast(ctypes.byref(a), ctypes.c_void_p) for a in args])
        _ck(self.cu.cuLaunchKernel(f, grid, 1, 1, 25, 25, 1, 0, None, ptrs, None), "cuLaunchKernel")

    def sync(self):
        _ck(self.cu.cuCtxSynchronize(), "cuCtxSynchronize")


def texture(t):
    """Texture object over a complex128 torch tensor, read as int4 (as Base::createTexObject does)."""
    cu = _driver()
    rd = _ResDesc()
    rd.resType = 0x02  # linear
    rd.devPtr = t.data_ptr()
    rd.format = 0x0A   # signed int32
    rd.numChannels = 4
    rd.sizeInBytes = t.numel() * 16
    td = _TexDesc()
    td.flags = 0x01    # read as integer
    tex = ctypes.c_uint64()
    _ck(cu.cuTexObjectCreate(ctypes.byref(tex), ctypes.byref(rd), ctypes.byref(td), None), "cuTexObjectCreate")
    return tex


def destroy_texture(tex):
    _driver().cuTexObjectDestroy(tex)


def _p(t):
    return ctypes.c_uint64(t.data_ptr())


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, np.complex128)).cuda()


def _f32(a):
    return np.ascontiguousarray(a, np.float32)


def _i16(a):
    return np.ascontiguousarray(a, np.int16)


def cubin(name):
    return os.path.join(REF_DIR, "contract_kernels_%s.cubin" % name)


# ---------------------------------------------------------------- diagrams
def rho(prop, mom5):
    """Contract_rho_rho::contractRho: rows [Nt(tf), Nt(ti), 768] and corr [tf, ti, 16, 3]."""
    import torch
    nt = prop.shape[0]
    m = RefModule(cubin("rho"))
    spin, lprp, coef = T.rho_tables()
    m.set_constant("c_spinIndices_rho", _i16(spin))
    m.set_constant("c_lp_rp_rho", _i16(lprp))
    m.set_constant("c_coef_rho", _f32(coef))
    k = m.kernel("calculate_rho_kernel_double")
    d_mom = _dev(mom5)
    tmom = texture(d_mom)
    rows = np.zeros((nt, nt, 768), np.complex128)
    tmp1 = torch.zeros(768 * NSIZE * NSIZE, dtype=torch.complex128, device="cuda")
    tmp2 = torch.zeros_like(tmp1)
    for tf in range(nt):
        d_row = _dev(prop[tf])
        tprop = texture(d_row)
        out = torch.zeros(nt * 768, dtype=torch.complex128, device="cuda")
        for ti in range(nt):
            m.launch(k, 768, [_p(out), tprop, tmom, ctypes.c_int(ti), ctypes.c_int(tf), _p(tmp1), _p(tmp2)])
        m.sync()
        rows[tf] = out.cpu().numpy().reshape(nt, 768)
        destroy_texture(tprop)
    destroy_texture(tmom)
    corr = rows.reshape(nt, nt, 16, 3, 16).sum(-1)
    return rows, corr


def sigma(prop, mom2):
    """Contract_sigma_sigma::contractSigma: rows [tf, ti, 64], corr [tf, ti, 4]."""
    import torch
    nt = prop.shape[0]
    m = RefModule(cubin("sigma"))
    spin, lprp, coef = T.sigma_tables()
    m.set_constant("c_spinIndices_sigma", _i16(spin))
    m.set_constant("c_lp_rp_sigma", _i16(lprp))
    m.set_constant("c_coef_sigma", _f32(coef))
    k = m.kernel("calculate_sigma_one_fish_kernel_double")
    d_mom = _dev(mom2)
    tmom = texture(d_mom)
    rows = np.zeros((nt, nt, 64), np.complex128)
    tmp1 = torch.zeros(nt * 64 * NSIZE * NSIZE, dtype=torch.complex128, device="cuda")
    tmp2 = torch.zeros_like(tmp1)
    for tf in range(nt):
        d_row = _dev(prop[tf])
        tprop = texture(d_row)
        out = torch.zeros(nt * 64, dtype=torch.complex128, device="cuda")
        m.launch(k, nt * 64, [_p(out), tprop, tmom, ctypes.c_int(tf), _p(tmp1), _p(tmp2)])
        m.sync()
        rows[tf] = out.cpu().numpy().reshape(nt, 64)
        destroy_texture(tprop)
    destroy_texture(tmom)
    return rows, rows.reshape(nt, nt, 4, 16).sum(-1)


def loop_unity(prop, mom):
    """Contract_loop_unity: rows [t, 4] and loop [t]."""
    import torch
    nt = prop.shape[0]
    m = RefModule(cubin("loop_unity"))
    k = m.kernel("calculate_loop_unity_kernel_double")
    d_diag = _dev(prop[np.arange(nt), np.arange(nt)])
    d_mom = _dev(mom)
    tdiag, tmom = texture(d_diag), texture(d_mom)
    out = torch.zeros(nt * 4, dtype=torch.complex128, device="cuda")
    tmp = torch.zeros(nt * 4 * NSIZE * NSIZE, dtype=torch.complex128, device="cuda")
    m.launch(k, nt * 4, [_p(out), tdiag, tmom, _p(tmp)])
    m.sync()
    rows = out.cpu().numpy().reshape(nt, 4)
    destroy_texture(tdiag)
    destroy_texture(tmom)
    return rows, rows.sum(-1)


def rhopi(prop, p1, p2, mom5_p1p2, idir):
    """Contract_rho_pipi::contractRhoPi: rows [tf, ti, 256], corr [tf, ti, 4]."""
    import torch
    nt = prop.shape[0]
    m = RefModule(cubin("rhopi"))
    spin, ip, coef = T.rhopi_tables()
    m.set_constant("c_spinIndices_rhopi", _i16(spin))
    m.set_constant("c_ip_rhopi", _i16(ip))
    m.set_constant("c_coef_rhopi", _f32(coef))
    k = m.kernel("calculate_rhopi_kernel_double")
    d_diag = _dev(prop[np.arange(nt), np.arange(nt)])
    d1, d2, d12 = _dev(p1), _dev(p2), _dev(mom5_p1p2)
    tdiag, t1, t2, t12 = texture(d_diag), texture(d1), texture(d2), texture(d12)
    rows = np.zeros((nt, nt, 256), np.complex128)
    tmp1 = torch.zeros(256 * NSIZE * NSIZE, dtype=torch.complex128, device="cuda")
    tmp2 = torch.zeros_like(tmp1)
    for tf in range(nt):
        d_row = _dev(prop[tf])
        tprop = texture(d_row)
        out = torch.zeros(nt * 256, dtype=torch.complex128, device="cuda")
        for ti in range(nt):
            m.launch(k, 256, [_p(out), tprop, tdiag, t1, t2, t12, ctypes.c_int(ti), ctypes.c_int(tf),
                              ctypes.c_int(idir), _p(tmp1), _p(tmp2)])
        m.sync()
        rows[tf] = out.cpu().numpy().reshape(nt, 256)
        destroy_texture(tprop)
    for t in (tdiag, t1, t2, t12):
        destroy_texture(t)
    return rows, rows.reshape(nt, nt, 4, 64).sum(-1)


def pipi(prop, p1, p2, p3, p4, iso):
    """Contract_pipi_pipi::contractPiPi (iso 1) / I0 (iso 0): per-diagram rows and corr [tf, ti, 5]."""
    import torch
    nt = prop.shape[0]
    m = RefModule(cubin("pipi"))
    t = T.pipi_tables()
    m.set_constant("c_spinIndices_pipi_square", _i16(t["spinIndices_pipi_square"]))
    m.set_constant("c_spinIndices_pipi_doubleTriangle", _i16(t["spinIndices_pipi_doubleTriangle"]))
    m.set_constant("c_spinIndices_pipi_doubleTriangle_hor", _i16(t["spinIndices_pipi_doubleTriangle_hor"]))
    m.set_constant("c_coef_pipi_square", _f32(t["coef_pipi_square"]))
    m.set_constant("c_coef_pipi_doubleTriangle", _f32(t["coef_pipi_doubleTriangle"]))
    m.set_constant("c_coef_pipi_doubleTriangle_hor", _f32(t["coef_pipi_doubleTriangle_hor"]))
    ksq = m.kernel("calculate_pipi_square_kernel_double")
    kdt = m.kernel("calculate_pipi_doubleTriangle_kernel_double")
    kdh = m.kernel("calculate_pipi_doubleTriangleHor_kernel_double")
    ksf = m.kernel("calculate_pipi_starfish_kernel_double")
    d_diag = _dev(prop[np.arange(nt), np.arange(nt)])
    dm = [_dev(x) for x in (p1, p2, p3, p4)]
    tdiag = texture(d_diag)
    tm = [texture(x) for x in dm]
    tmp1 = torch.zeros(nt * 256 * NSIZE * NSIZE, dtype=torch.complex128, device="cuda")
    tmp2 = torch.zeros_like(tmp1)
    res = {k: np.zeros((nt, nt) + s, np.complex128) for k, s in
           (("square", (256,)), ("dtri", (256,)), ("dtri_hor", (256,)), ("star", (2, 16)), ("fish", (2, 16)))}
    for tf in range(nt):
        d_row = _dev(prop[tf])
        tprop = texture(d_row)
        o = {k: torch.zeros(nt * 256, dtype=torch.complex128, device="cuda") for k in ("square", "dtri", "dtri_hor")}
        o["star"] = torch.zeros(2 * nt * 16, dtype=torch.complex128, device="cuda")
        o["fish"] = torch.zeros(2 * nt * 16, dtype=torch.complex128, device="cuda")
        tfc = ctypes.c_int(tf)
        m.launch(ksq, nt * 256, [_p(o["square"]), tprop, tdiag] + tm + [tfc, _p(tmp1), _p(tmp2)])
        m.launch(kdt, nt * 256, [_p(o["dtri"]), tprop, tdiag] + tm + [tfc, _p(tmp1), _p(tmp2)])
        if iso == 0:
            m.launch(kdh, nt * 256, [_p(o["dtri_hor"]), tprop] + tm + [tfc, _p(tmp1), _p(tmp2)])
        m.launch(ksf, nt * 16, [_p(o["star"]), tprop] + tm + [tfc, _p(tmp1), _p(tmp2)])
        m.launch(ksf, nt * 16, [_p(o["fish"]), tprop, tm[0], tm[1], tm[3], tm[2], tfc, _p(tmp1), _p(tmp2)])
        m.sync()
        for k in ("square", "dtri", "dtri_hor"):
            res[k][tf] = o[k].cpu().numpy().reshape(nt, 256)
        for k in ("star", "fish"):
            res[k][tf] = o[k].cpu().numpy().reshape(2, nt, 16).transpose(1, 0, 2)
        destroy_texture(tprop)
    for x in [tdiag] + tm:
        destroy_texture(x)
    sq, dt, dh = res["square"].sum(-1), res["dtri"].sum(-1), res["dtri_hor"].sum(-1)
    st = res["star"].sum(-1)
    fi = res["fish"].sum(-1)
    star, fish = st[..., 0] * st[..., 1], fi[..., 0] * fi[..., 1]
    corr = np.zeros((nt, nt, 5), np.complex128)
    if iso == 1:   # lib/contract_kernels_pipi.cu:288-303
        corr[..., 0], corr[..., 1], corr[..., 2], corr[..., 3] = -2 * sq, 2 * dt, -star, fish
    else:          # lib/contract_kernels_pipi.cu:463-478
        corr[..., 0], corr[..., 1], corr[..., 2], corr[..., 3], corr[..., 4] = (
            -sq / 3, -dt / 3, star, fish, -5 * dh / 3)
    res["corr"] = corr
    return res


def sigmapi(prop, p1, p2, mom2_p1p2):
    """Contract_sigma_pipi::contractSigmaPi: hor-fish rows [t,16] / corr [t]; triangle rows [tf,ti,128] / corr [tf,ti,2]."""
    import torch
    nt = prop.shape[0]
    m = RefModule(cubin("sigmapi"))
    t = T.sigmapi_tables()
    m.set_constant("c_spinIndices_sigmapi_hor_fish", _i16(t["spinIndices_sigmapi_hor_fish"]))
    m.set_constant("c_coef_sigmapi_hor_fish", _f32(t["coef_sigmapi_hor_fish"]))
    m.set_constant("c_spinIndices_sigmapi_triangle", _i16(t["spinIndices_sigmapi_triangle"]))
    m.set_constant("c_ip_sigmapi_triangle", _i16(t["ip_sigmapi_triangle"]))
    m.set_constant("c_coef_sigmapi_triangle", _f32(t["coef_sigmapi_triangle"]))
    khf = m.kernel("calculate_sigmapi_hor_fish_kernel_double")
    ktr = m.kernel("calculate_sigmapi_triangle_kernel_double")
    d_diag = _dev(prop[np.arange(nt), np.arange(nt)])
    d1, d2, d12 = _dev(p1), _dev(p2), _dev(mom2_p1p2)
    tdiag, t1, t2, t12 = texture(d_diag), texture(d1), texture(d2), texture(d12)
    tmp1 = torch.zeros(nt * 128 * NSIZE * NSIZE, dtype=torch.complex128, device="cuda")
    tmp2 = torch.zeros_like(tmp1)
    out = torch.zeros(nt * 16, dtype=torch.complex128, device="cuda")
    m.launch(khf, nt * 16, [_p(out), tdiag, t1, t2, _p(tmp1), _p(tmp2)])
    m.sync()
    hf_rows = out.cpu().numpy().reshape(nt, 16)
    tri_rows = np.zeros((nt, nt, 128), np.complex128)
    for tf in range(nt):
        d_row = _dev(prop[tf])
        tprop = texture(d_row)
        o = torch.zeros(nt * 128, dtype=torch.complex128, device="cuda")
        m.launch(ktr, nt * 128, [_p(o), tprop, tdiag, t1, t2, t12, ctypes.c_int(tf), _p(tmp1), _p(tmp2)])
        m.sync()
        tri_rows[tf] = o.cpu().numpy().reshape(nt, 128)
        destroy_texture(tprop)
    for x in (tdiag, t1, t2, t12):
        destroy_texture(x)
    return dict(hor_fish_rows=hf_rows, hor_fish=hf_rows.sum(-1), triangle_rows=tri_rows,
                triangle=tri_rows.reshape(nt, nt, 2, 64).sum(-1))
