"""Seeded synthetic perambulators and elementals.

The reference reads perambulators and builds elementals from lattice files
(tests/compute_rho.cpp:100-225) that are not available here; these generators
stand in for them with the shapes and value distributions the workloads name:

* tau(t1,t2) for t1 >= t2: 16 spin blocks of Nev x Nev entries, complex
  Gaussian with E|z|^2 = 1/Nev, times exp(-decay*|t1-t2|).  The time diagonal is
  gamma5-symmetrised and the other half is filled by gamma5-hermiticity,
  tau(t2,t1) = g5 tau(t1,t2)^dagger g5, i.e. block (a,b) = g5_a g5_b
  (block (b,a) of tau(t1,t2))^dagger with g5 = diag(1,1,-1,-1).
* Phi(0,t) = (G + G^dagger)/2 with G complex Gaussian N(0,1/Nev).
* Phi(p,t) for one member of each +-p pair: real N(0,1/Nev) entries times a
  uniform phase e^{i theta}; Phi(-p,t) = Phi(p,t)^dagger.

Arrays are complex128 in the reference layouts: tau [Nt,Nt,4,4,N,N],
Phi [Nt,N,N].  ``backend="torch"`` builds them on a CUDA device with a seeded
torch generator (used for production sizes); ``"numpy"`` on the host.
"""

import itertools

import numpy as np

G5 = np.array([1.0, 1.0, -1.0, -1.0])


def momenta(max_p2):
    """All integer momenta with |p|^2 <= max_p2, ordered by |p|^2 then lexicographically."""
    r = int(np.floor(np.sqrt(max_p2)))
    ps = [p for p in itertools.product(range(-r, r + 1), repeat=3) if sum(c * c for c in p) <= max_p2]
    return sorted(ps, key=lambda p: (sum(c * c for c in p), p))


def _canonical(p):
    """True for the representative of a +-p pair (first non-zero component > 0)."""
    for c in p:
        if c != 0:
            return c > 0
    return True


def _gamma5_adjoint_np(blocks):
    # blocks [4,4,N,N] -> g5 blocks^dagger g5 in the 4N x 4N sense
    out = np.conj(np.transpose(blocks, (1, 0, 3, 2)))
    return out * (G5[:, None, None, None] * G5[None, :, None, None])


def make_prop(nt, nev, seed, decay=0.35, backend="numpy", device="cuda"):
    if backend == "torch":
        return _make_prop_torch(nt, nev, seed, decay, device)
    rng = np.random.default_rng(seed)
    tau = np.zeros((nt, nt, 4, 4, nev, nev), np.complex128)
    sd = np.sqrt(0.5 / nev)
    for t1 in range(nt):
        for t2 in range(t1 + 1):
            x = (rng.normal(0.0, sd, (4, 4, nev, nev)) + 1j * rng.normal(0.0, sd, (4, 4, nev, nev)))
            x *= np.exp(-decay * abs(t1 - t2))
            if t1 == t2:
                x = 0.5 * (x + _gamma5_adjoint_np(x))
            tau[t1, t2] = x
    for t1 in range(nt):
        for t2 in range(t1 + 1, nt):
            tau[t1, t2] = _gamma5_adjoint_np(tau[t2, t1])
    return tau


def _make_prop_torch(nt, nev, seed, decay, device):
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    sd = float(np.sqrt(0.5 / nev))
    tau = torch.empty((nt, nt, 4, 4, nev, nev), dtype=torch.complex128, device=device)
    g5 = torch.tensor(G5, dtype=torch.float64, device=device)
    sign = (g5[:, None] * g5[None, :])[:, :, None, None]
    for t1 in range(nt):
        n = t1 + 1
        re = torch.randn((n, 4, 4, nev, nev), generator=g, dtype=torch.float64, device=device) * sd
        im = torch.randn((n, 4, 4, nev, nev), generator=g, dtype=torch.float64, device=device) * sd
        x = torch.complex(re, im)
        dist = torch.arange(t1, -1, -1, device=device, dtype=torch.float64)  # t2 = 0..t1 -> |t1-t2|
        x *= torch.exp(-decay * dist)[:, None, None, None, None]
        diag = x[t1]
        x[t1] = 0.5 * (diag + torch.conj(diag.permute(1, 0, 3, 2)) * sign)
        tau[t1, : t1 + 1] = x
    for t1 in range(nt - 1):
        # tau[t1, t2] for t2 > t1 from tau[t2, t1]
        src = tau[t1 + 1:, t1]
        tau[t1, t1 + 1:] = torch.conj(src.permute(0, 2, 1, 4, 3)) * sign
    return tau


def make_phi_hermitian(nt, nev, seed):
    rng = np.random.default_rng(seed)
    sd = np.sqrt(0.5 / nev)
    g = rng.normal(0.0, sd, (nt, nev, nev)) + 1j * rng.normal(0.0, sd, (nt, nev, nev))
    return 0.5 * (g + np.conj(np.transpose(g, (0, 2, 1))))


def make_phi_random(nt, nev, rng):
    mag = rng.normal(0.0, np.sqrt(1.0 / nev), (nt, nev, nev))
    th = rng.uniform(0.0, 2 * np.pi, (nt, nev, nev))
    return mag * np.exp(1j * th)


def make_phi_momenta(nt, nev, moms, seed):
    """{p: Phi(p) [Nt,N,N]} for every p in moms, with Phi(-p) = Phi(p)^dagger and
    Phi(0) Hermitian."""
    rng = np.random.default_rng(seed)
    out = {}
    for p in sorted(set(moms) | {tuple(-c for c in q) for q in moms}, key=lambda p: (sum(c * c for c in p), p)):
        if p in out:
            continue
        if all(c == 0 for c in p):
            sd = np.sqrt(0.5 / nev)
            g = rng.normal(0.0, sd, (nt, nev, nev)) + 1j * rng.normal(0.0, sd, (nt, nev, nev))
            out[p] = 0.5 * (g + np.conj(np.transpose(g, (0, 2, 1))))
            continue
        rep = p if _canonical(p) else tuple(-c for c in p)
        neg = tuple(-c for c in rep)
        ph = make_phi_random(nt, nev, rng)
        out[rep] = ph
        out[neg] = np.conj(np.transpose(ph, (0, 2, 1)))
    return {p: out[p] for p in moms}


def make_phi_momenta_torch(nt, nev, moms, seed, device="cuda"):
    """Device version of make_phi_momenta: returns [Nt, len(moms), N, N] complex128."""
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    sd = float(np.sqrt(1.0 / nev))
    cache = {}
    out = torch.empty((nt, len(moms), nev, nev), dtype=torch.complex128, device=device)
    for k, p in enumerate(moms):
        if all(c == 0 for c in p):
            if p not in cache:
                re = torch.randn((nt, nev, nev), generator=g, dtype=torch.float64, device=device) * sd * np.sqrt(0.5)
                im = torch.randn((nt, nev, nev), generator=g, dtype=torch.float64, device=device) * sd * np.sqrt(0.5)
                x = torch.complex(re, im)
                cache[p] = 0.5 * (x + torch.conj(x.transpose(1, 2)))
            out[:, k] = cache[p]
            continue
        rep = p if _canonical(p) else tuple(-c for c in p)
        if rep not in cache:
            mag = torch.randn((nt, nev, nev), generator=g, dtype=torch.float64, device=device) * sd
            th = torch.rand((nt, nev, nev), generator=g, dtype=torch.float64, device=device) * (2 * np.pi)
            cache[rep] = torch.polar(mag.abs(), th) * torch.sign(mag)
        out[:, k] = cache[rep] if rep == p else torch.conj(cache[rep].transpose(1, 2))
    return out


def mom_stack(phis, order):
    """Stack {key: [Nt,N,N]} into [Nt, len(order), N, N] (the op/momentum axis second)."""
    return np.ascontiguousarray(np.stack([phis[k] for k in order], axis=1))


# ------------------------------------------------ eigenvectors and gauge links
# The elemental construction (tests/compute_rho.cpp:116-201) reads Laplacian
# eigenvectors and a smeared gauge configuration from lattice files; these stand
# in for them: per time slice, nev orthonormal colour-vector fields (the Q factor
# of a complex Gaussian matrix over sites x colours) and SU(3) links (the
# phase-fixed Q factor of a complex Gaussian 3 x 3 matrix, divided by a cube
# root of its determinant).  Layouts: evec [nt, nev, nz, ny, nx, 3] (colour
# fastest), links [nt, nz, ny, nx, 3 directions, 3, 3].

def make_eigvecs(nt, nev, nx, ny, nz, seed, backend="numpy", device="cuda"):
    """Built on the host (LAPACK QR) for both backends, so the seeded data are
    the same; backend "torch" returns them on the device."""
    K = 3 * nx * ny * nz
    rng = np.random.default_rng(seed)
    out = np.empty((nt, nev, nz, ny, nx, 3), np.complex128)
    for t in range(nt):
        G = rng.normal(size=(K, nev)) + 1j * rng.normal(size=(K, nev))
        Q, _ = np.linalg.qr(G)
        out[t] = Q.T.reshape(nev, nz, ny, nx, 3)
    if backend == "torch":
        import torch
        return torch.from_numpy(out).to(device)
    return out


def _su3(G):
    """SU(3) matrices from complex Gaussian [..., 3, 3]."""
    Q, R = np.linalg.qr(G)
    d = np.diagonal(R, axis1=-2, axis2=-1)
    Q = Q * (d / abs(d))[..., None, :]
    det = np.linalg.det(Q)
    return Q / (det ** (1.0 / 3.0))[..., None, None]


def make_links(nt, nx, ny, nz, seed, backend="numpy", device="cuda"):
    """Built on the host for both backends (as make_eigvecs)."""
    shape = (nt, nz, ny, nx, 3, 3, 3)
    rng = np.random.default_rng(seed)
    G = rng.normal(size=shape) + 1j * rng.normal(size=shape)
    out = np.ascontiguousarray(_su3(G))
    if backend == "torch":
        import torch
        return torch.from_numpy(out).to(device)
    return out
