"""Seeded initial states of the shipped workloads.

All randomness comes from splitmix64 (S. Vigna's public-domain generator,
also the seeding step of xoshiro), so the same seed gives the same state on
any machine — unlike the ``srand(time(NULL))``/``rand()`` of the reference's
drivers (examples/pearson-3d-main.cpp:164, examples/pearson-2d-main.cpp:13-33).
"""
from __future__ import annotations

import numpy as np

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed: int, n: int, offset: int = 0) -> np.ndarray:
    """The n outputs following state `seed` (+ offset draws), as uint64."""
    with np.errstate(over="ignore"):
        i = np.arange(offset + 1, offset + n + 1, dtype=np.uint64)
        z = np.uint64(seed & 0xFFFFFFFFFFFFFFFF) + i * _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def uniform(seed: int, n: int, offset: int = 0) -> np.ndarray:
    """n doubles uniform in [0, 1) (53-bit)."""
    return (splitmix64(seed, n, offset) >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)


def diffusion_2d(nx: int, ny: int, seed: int = 1) -> np.ndarray:
    """Uniform [0,1) density, the 2D diffusion workload's initial state."""
    return uniform(seed, nx * ny).reshape(nx, ny)


def gray_scott_3d(nx: int, ny: int, nz: int, seed: int = 1, ncubes: int = 8, side: int = 16,
                  dtype=np.float64):
    """U=1, V=0, plus `ncubes` cubes of side `side` at seeded positions (periodic
    wrap) where U = 0.5 and V = 0.25, each with +-1% uniform noise."""
    U = np.ones((nx, ny, nz), dtype=np.float64)
    V = np.zeros((nx, ny, nz), dtype=np.float64)
    pos = splitmix64(seed, 3 * ncubes)
    s = min(side, nx, ny, nz)
    draws = 3 * ncubes
    for c in range(ncubes):
        x0 = int(pos[3 * c] % np.uint64(nx))
        y0 = int(pos[3 * c + 1] % np.uint64(ny))
        z0 = int(pos[3 * c + 2] % np.uint64(nz))
        ix = (x0 + np.arange(s)) % nx
        iy = (y0 + np.arange(s)) % ny
        iz = (z0 + np.arange(s)) % nz
        r = uniform(seed, 2 * s ** 3, offset=draws).reshape(2, s, s, s)
        draws += 2 * s ** 3
        U[np.ix_(ix, iy, iz)] = 0.5 * (1.0 + 0.01 * (2.0 * r[0] - 1.0))
        V[np.ix_(ix, iy, iz)] = 0.25 * (1.0 + 0.01 * (2.0 * r[1] - 1.0))
    return U.astype(dtype), V.astype(dtype)


def gray_scott_2d_square(nx: int, ny: int, seed: int = 1, dtype=np.float64, frac: float = 0.2):
    """The 2D Gray-Scott start of examples/pearson-2d-main.cpp:16-33 scaled to
    the grid: U=1, V=0 with one seeded square (side frac*N) set to
    U = 0.5 + 0.01 r, V = 0.25 + 0.01 r."""
    U = np.ones((nx, ny), dtype=np.float64)
    V = np.zeros((nx, ny), dtype=np.float64)
    p = splitmix64(seed, 2)
    sx, sy = max(1, int(frac * nx)), max(1, int(frac * ny))
    x0, y0 = int(p[0] % np.uint64(nx)), int(p[1] % np.uint64(ny))
    ix = (x0 + np.arange(sx)) % nx
    iy = (y0 + np.arange(sy)) % ny
    r = uniform(seed, 2 * sx * sy, offset=2).reshape(2, sx, sy)
    U[np.ix_(ix, iy)] = 0.5 + 0.01 * r[0]
    V[np.ix_(ix, iy)] = 0.25 + 0.01 * r[1]
    return U.astype(dtype), V.astype(dtype)


ENSEMBLE_SIZES = (64, 128, 256, 512, 1024)


def gs2d_ensemble(n_inst: int = 512, seed: int = 1, sizes=ENSEMBLE_SIZES,
                  F_range=(0.02, 0.06), k_range=(0.05, 0.07)):
    """The batched 2D Gray-Scott workload: instance sizes drawn uniformly from
    `sizes`, F ~ U[F_range], k ~ U[k_range] (seeded).  Returns (sizes, F, k)."""
    r = uniform(seed, 3 * n_inst).reshape(3, n_inst)
    sz = [int(sizes[min(int(x * len(sizes)), len(sizes) - 1)]) for x in r[0]]
    F = F_range[0] + (F_range[1] - F_range[0]) * r[1]
    k = k_range[0] + (k_range[1] - k_range[0]) * r[2]
    return sz, F, k


def gs2d_ensemble_state(sizes, seed: int = 1, dtype=np.float32):
    """Flat U, V of an ensemble: instance i is gray_scott_2d_square(n_i, n_i,
    seed + i) laid out back to back."""
    us, vs = [], []
    for i, n in enumerate(sizes):
        u, v = gray_scott_2d_square(n, n, seed=seed * 100003 + i)
        us.append(u.reshape(-1))
        vs.append(v.reshape(-1))
    return np.concatenate(us).astype(dtype), np.concatenate(vs).astype(dtype)


MHD_FIELDS = ("dens", "vx", "vy", "vz", "Bx", "By", "Bz", "s", "Psi")


def _random_modes(n: int, seed: int, kmax: float, offset: int) -> np.ndarray:
    """A real periodic field on [0,1)^3 (n^3 grid) made of all Fourier modes
    with 0 < |k| <= kmax (integer wavenumbers), unit amplitude and seeded
    random phases, normalised to unit rms."""
    k = np.fft.fftfreq(n, 1.0 / n)
    kx, ky, kz = np.meshgrid(k, k, k[: n // 2 + 1], indexing="ij")
    kk = np.sqrt(kx ** 2 + ky ** 2 + kz ** 2)
    mask = (kk > 0) & (kk <= kmax)
    spec = np.zeros(kk.shape, dtype=np.complex128)
    m = int(mask.sum())
    ph = uniform(seed, m, offset=offset) * 2.0 * np.pi
    spec[mask] = np.exp(1j * ph)
    f = np.fft.irfftn(spec, s=(n, n, n), axes=(0, 1, 2))
    return f / np.sqrt(np.mean(f ** 2))


def _d4(a: np.ndarray, axis: int, n: int) -> np.ndarray:
    """The 4th-order central difference of 3d-mhd-rk4.fmr:13-15 (dx = 1/n)."""
    r = lambda s: np.roll(a, -s, axis)  # noqa: E731  (value at i+s)
    return (((r(-2) + 8.0 * r(1)) - 8.0 * r(-1)) - r(2)) / (12.0 * (1.0 / n))


def mhd_3d(n: int, seed: int = 1, amp: float = 1e-2, kmax: float = 4.0):
    """Initial state of the 3D MHD workload: rho = 1, p = 1 (dens = 0, s = 0
    for the linearised EOS p = dens0 + dens + 0.4 s of 3d-mhd-rk4.fmr:94),
    Psi = 0, velocity and magnetic perturbations of rms amplitude `amp` with
    random phases over wavenumbers 0 < |k| <= kmax.  B is the discrete curl of
    a random vector potential taken with the program's own 4th-order
    difference, so its discrete divergence vanishes (up to rounding).
    Returns the 9 fields as float64 arrays [n][n][n]."""
    v = [amp * _random_modes(n, seed, kmax, offset=1000003 * c) for c in range(3)]
    A = [_random_modes(n, seed + 7, kmax, offset=1000003 * (c + 3)) for c in range(3)]
    B = [_d4(A[2], 1, n) - _d4(A[1], 2, n),
         _d4(A[0], 2, n) - _d4(A[2], 0, n),
         _d4(A[1], 0, n) - _d4(A[0], 1, n)]
    rms = np.sqrt(np.mean(B[0] ** 2 + B[1] ** 2 + B[2] ** 2) / 3.0)
    B = [amp * b / rms for b in B]
    z = np.zeros((n, n, n))
    return [z.copy(), v[0], v[1], v[2], B[0], B[1], B[2], z.copy(), z.copy()]
