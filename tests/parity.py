"""Per-entry parity gate shared by the tests.

Every correlator entry is checked on its own:

    |got - ref| <= tol * |ref| + FLOOR * rows_abs

where ``rows_abs`` is the sum of the magnitudes of the spin rows (or trace
products) the entry is summed from, as the oracle computes them.  The second
term is the FP64 rounding floor of a cancelling entry: two correct FP64
evaluations in different orders differ by up to ~1e-13 of each row (measured:
the oracle against the reference's own kernels, per row, at Nev=100), so an
entry whose rows cancel to 1e-5 of their magnitudes cannot agree to better than
~1e-8 relative whatever the engine.  FLOOR = 2^-44 (5.7e-14) keeps that term
below 1e-12 of the entry wherever the rows do not cancel (they sum to a few
times the entry's magnitude), so there the gate is the plain relative one.
"""

import numpy as np

FLOOR = 2.0 ** -44


def entrywise(got, ref, tol, rows_abs=None, what="", floor=FLOOR):
    """Assert the gate for every entry; return the statistics (worst relative
    error, how many entries needed the floor).  `floor` replaces 2^-44 where two
    split-engine results are compared with each other: their float-float traces
    carry ~2^-44 of the rows' magnitudes each."""
    got = np.asarray(got)
    ref = np.asarray(ref)
    assert got.shape == ref.shape, (what, got.shape, ref.shape)
    assert np.all(np.isfinite(got)), "%s: non-finite entries" % what
    err = np.abs(got - ref)
    mag = np.abs(ref)
    bound = tol * mag
    if rows_abs is not None:
        rows_abs = np.broadcast_to(np.asarray(rows_abs, dtype=np.float64), ref.shape)
        bound = bound + floor * rows_abs
    bad = err > bound
    rel = err / np.maximum(mag, 1e-300)
    stats = {"entries": int(ref.size), "max_rel": float(rel.max()) if ref.size else 0.0,
             "needed_floor": int(np.count_nonzero(err > tol * mag))}
    if np.any(bad):
        i = np.unravel_index(int(np.argmax(err - bound)), ref.shape)
        raise AssertionError("%s: %d of %d entries outside |err| <= %.1e |ref| + %.2e rows_abs; worst at %s: got %r "
                             "ref %r (rel %.3e, rows_abs %.3e)"
                             % (what, int(bad.sum()), ref.size, tol, floor, tuple(int(x) for x in i), got[i], ref[i],
                                rel[i],
                                float(rows_abs[i]) if rows_abs is not None else 0.0))
    return stats


def rho_rows_abs(rows):
    """rows [..., 768] (oracle rho rows) -> the per-entry row magnitudes [..., 16, 3]
    (output o = row // 16, lib/contract_kernels_rho.cu:108-116)."""
    a = np.abs(np.asarray(rows))
    return a.reshape(a.shape[:-1] + (48, 16)).sum(-1).reshape(a.shape[:-1] + (16, 3))


def _group_abs(rows, per):
    a = np.abs(np.asarray(rows))
    return a.reshape(a.shape[:-1] + (a.shape[-1] // per, per)).sum(-1)


def sigma_rows_abs(rows):
    """sigma rows [..., 64] -> [..., 4]: 16 spin rows per (lp, rp) (lib/contract_kernels_sigma.cu)."""
    return _group_abs(rows, 16)


def rhopi_rows_abs(rows):
    """rho -> pi pi rows [..., 256] of one idir -> [..., 4]: 64 rows per rho operator."""
    return _group_abs(rows, 64)


def triangle_rows_abs(rows):
    """sigma -> pi pi triangle rows [..., 128] -> [..., 2]: 64 rows per operator."""
    return _group_abs(rows, 64)


def sum_rows_abs(rows):
    """Rows [..., k] that all sum into one entry (hor-fish [Nt, 16], loop [Nt, 4])."""
    return np.abs(np.asarray(rows)).sum(-1)


def pipi_rows_abs(d, iso):
    """The oracle's pi pi row dict (pyoracle.pipi_row) -> [Nt, 5] with the isospin weights of
    lib/contract_kernels_pipi.cu:288-303 (I=1) and :463-478 (I=0); star and fish are
    products of two spin sums, so their magnitude is the product of the two row sums."""
    sq, dt = sum_rows_abs(d["square"]), sum_rows_abs(d["dtri"])
    star = sum_rows_abs(d["star"][0]) * sum_rows_abs(d["star"][1])
    fish = sum_rows_abs(d["fish"][0]) * sum_rows_abs(d["fish"][1])
    if iso == 1:
        return np.stack([2 * sq, 2 * dt, star, fish, np.zeros_like(sq)], axis=-1)
    return np.stack([sq / 3, dt / 3, star, fish, 5 * sum_rows_abs(d["dtri_hor"]) / 3], axis=-1)
