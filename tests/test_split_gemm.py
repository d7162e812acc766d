"""The split-precision tensor-core GEMM (BF16 slices, tcgen05, float-float
recombination) against numpy complex128 products.

Tolerance: each operand keeps 45 bits below its row/column scale (5 balanced
base-512 digits, rounded), levels 0-2 of the slice products accumulate exactly,
level >= 3 and the dropped slice pairs are ~2^-44 of the result.  The bound
tested is 1e-11 relative to max|C|, two orders of magnitude inside the 1e-9
correlator tolerance."""
import numpy as np
import pytest
import torch

from contractions_code_scattering_gb300 import api

pytestmark = pytest.mark.gpu

TOL = 1e-11


def _rand(rng, shape, scale=1.0):
    return (rng.normal(size=shape) + 1j * rng.normal(size=shape)) * scale


def _check(x, y, cuda, engine="split", tol=TOL):
    got = api.zgemm_batched(torch.from_numpy(x).to(cuda), torch.from_numpy(y).to(cuda), engine=engine)
    api.sync()
    ref = np.einsum("bij,bjk->bik", x, y)
    err = np.abs(got.cpu().numpy() - ref).max() / np.abs(ref).max()
    assert err <= tol, "split GEMM error %.3e > %.1e" % (err, tol)
    return err


@pytest.mark.parametrize("n", [100, 16, 37, 80, 81, 128, 1])
def test_split_gemm_random(cuda, n):
    rng = np.random.default_rng(n)
    _check(_rand(rng, (3, n, n)), _rand(rng, (3, n, n)), cuda)


def test_split_gemm_identity_is_exact(cuda):
    n = 100
    eye = np.eye(n, dtype=np.complex128)[None]
    rng = np.random.default_rng(1)
    # values with <= 40 significant bits are reproduced exactly
    y = np.round(_rand(rng, (1, n, n)) * 2 ** 20) / 2 ** 20
    got = api.zgemm_batched(torch.from_numpy(eye).to(cuda), torch.from_numpy(y).to(cuda), engine="split")
    api.sync()
    assert np.array_equal(got.cpu().numpy(), y)


def test_split_gemm_row_and_column_scales(cuda):
    """Rows of X and columns of Y spanning 1e-12 .. 1e3: per-row/column power-of-two scaling."""
    n = 100
    rng = np.random.default_rng(2)
    x = _rand(rng, (2, n, n)) * np.logspace(-12, 3, n)[None, :, None]
    y = _rand(rng, (2, n, n)) * np.logspace(3, -12, n)[None, None, :]
    got = api.zgemm_batched(torch.from_numpy(x).to(cuda), torch.from_numpy(y).to(cuda), engine="split")
    api.sync()
    ref = np.einsum("bij,bjk->bik", x, y)
    # entry-wise relative error against the scale of the entry's row and column
    scale = np.abs(x).max(axis=2)[:, :, None] * np.abs(y).max(axis=1)[:, None, :] * n
    assert (np.abs(got.cpu().numpy() - ref) / scale).max() < 1e-11


def test_split_gemm_zero_and_sparse(cuda):
    n = 64
    x = np.zeros((2, n, n), np.complex128)
    y = np.zeros((2, n, n), np.complex128)
    x[1, 3, 5] = 2.5 - 1j
    y[1, 5, 7] = -0.75j
    got = api.zgemm_batched(torch.from_numpy(x).to(cuda), torch.from_numpy(y).to(cuda), engine="split").cpu().numpy()
    api.sync()
    assert np.array_equal(got[0], np.zeros((n, n)))
    ref = np.einsum("bij,bjk->bik", x, y)
    assert np.array_equal(got[1], ref[1])


def test_fp64_engine_gemm(cuda):
    rng = np.random.default_rng(3)
    _check(_rand(rng, (2, 100, 100)), _rand(rng, (2, 100, 100)), cuda, engine="fp64", tol=1e-14)


def _emulate_slices(X, axis, nslice=5):
    """Exact emulation of the slicer: per-row (axis=1) or per-column (axis=0)
    power-of-two scale 2^E, balanced base-512 digits of the 63-bit fixed-point
    magnitude |x|/2^E (digit s at bit 55-9s, rounded at the last digit)."""
    re, im = X.real, X.imag
    er = np.where(re != 0, np.frexp(re)[1], -30000)
    ei = np.where(im != 0, np.frexp(im)[1], -30000)
    e = np.maximum(er, ei).max(axis=axis, keepdims=True)
    E = np.where(e < -1000, 0, e)
    shift = [55 - 9 * s for s in range(nslice)]
    offset = (1 << (shift[-1] - 1)) + sum(256 << shift[s] for s in range(1, nslice))

    def cut(a):
        U = np.floor(np.abs(a) * np.ldexp(1.0, 63 - E)).astype(np.uint64)
        W = U + np.uint64(offset)
        out = []
        for s in range(nslice):
            if s == 0:
                d = (W >> np.uint64(55)).astype(np.int64)
            else:
                d = ((W >> np.uint64(shift[s])) & np.uint64(511)).astype(np.int64) - 256
            assert np.abs(d).max() <= 256
            out.append(np.sign(a) * d.astype(np.float64) * 2.0 ** (shift[s] - 63))
        return out
    return cut(re), cut(im)


def test_slice_emulation_reconstructs():
    """CPU check of the digit arithmetic the slicer uses: the digits sum back to
    |x|/2^E within 2^-45 (round to nearest at the last digit)."""
    rng = np.random.default_rng(5)
    x = _rand(rng, (40, 40)) * np.logspace(-8, 2, 40)[:, None]
    (xr, xi) = _emulate_slices(x, 1)
    E = np.maximum(np.frexp(np.abs(x.real))[1], np.frexp(np.abs(x.imag))[1]).max(axis=1, keepdims=True)
    err = np.abs(sum(xr) * np.ldexp(1.0, E) - x.real) / np.ldexp(1.0, E)
    assert err.max() <= 2.0 ** -45
    err = np.abs(sum(xi) * np.ldexp(1.0, E) - x.imag) / np.ldexp(1.0, E)
    assert err.max() <= 2.0 ** -45


def test_tensor_core_accumulation_levels(cuda):
    """Levels 0, 1, 2 are sums of < 2^24 integer units: the FP32 tensor-core
    accumulation must reproduce them exactly; level >= 3 to ~2^-17 of its size."""
    n = 100
    rng = np.random.default_rng(11)
    x, y = _rand(rng, (n, n)), _rand(rng, (n, n))
    lv = api.split_levels(torch.from_numpy(x).to(cuda), torch.from_numpy(y).to(cuda)).cpu().numpy().astype(np.float64)
    (xr, xi), (yr, yi) = _emulate_slices(x, 1), _emulate_slices(y, 0)
    exact = np.zeros((8, n, n))
    for i in range(5):
        for j in range(5 - i):
            l = min(i + j, 3)
            exact[l] += xr[i] @ yr[j] - xi[i] @ yi[j]
            exact[4 + l] += xr[i] @ yi[j] + xi[i] @ yr[j]
    report = []
    for a in range(8):
        d = np.abs(lv[a] - exact[a])
        report.append("acc%d: max|diff| %.3e (max|exact| %.3e, mismatches %d)" % (a, d.max(), np.abs(exact[a]).max(), (d > 0).sum()))
    print("\n".join(report))
    for a in (0, 1, 2, 4, 5, 6):
        assert np.array_equal(lv[a], exact[a]), report[a]
    # level >= 3 is ~2^-27 of the result; the tensor core truncates its small
    # addends (measured ~2^-18 of the level), i.e. ~2^-45 of the result
    for a in (3, 7):
        assert np.abs(lv[a] - exact[a]).max() <= 2.0 ** -16 * np.abs(exact[a]).max(), report[a]


def test_mma_schedule_probe(cuda):
    """The split GEMMs' MMA schedules issued alone (ctr_mma_schedule_probe): the
    standard one at the full tensor rate (64 clocks per M128 N128 K16 MMA), the
    high-precision one bound by its shared-memory operand reads (~56 clocks per
    M128 N96 K16 MMA); loose bounds, since only the order of magnitude is checked."""
    cpm, tf = api.mma_schedule_probe(False, 200)
    assert 60.0 <= cpm <= 90.0 and tf > 500.0, (cpm, tf)
    cpm, tf = api.mma_schedule_probe(True, 200)
    assert 44.0 <= cpm <= 80.0 and tf > 400.0, (cpm, tf)
