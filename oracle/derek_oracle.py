"""CPU FP64 oracle for the DEReK plane-wave Kohn-Sham hot path.

TEST INFRASTRUCTURE ONLY.  This module is the checker the GPU library is
compared against; nothing in the shipped library imports it.  Only the tests,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may use it.

What it restates, and from where (paths are inside the DEReK source tree):

* FFT grid sizing          Source/basis.f90:87-95 (k_cut, std and fine sizes)
* smooth-size rounding     Source/basis.f90:257-309 (basis_prime_fact, 13-smooth)
* reciprocal cell          Source/io.f90:1954 (inv_cell = transpose(2 pi cell^-1))
* lattice lengths          Source/io.f90:1956-1966 (norms of the columns of cell)
* centred G enumeration    Source/basis.f90:125-149 (x outer, z inner)
* real-space grid          Source/basis.f90:156-188 (frac = i/n, i = 1..n)
* Monkhorst-Pack k-points  Source/io.f90:2016-2031 (k = n d - (1 + d)/2)
* FFT sign / layout        Source/fft.f90:204-212, 260-291 (dir=+1 forward e^{-i},
                           dir=-1 backward e^{+i}, neither normalised, flat
                           index (ix*ny + iy)*nz + iz)
* jellium potential        Source/pot.f90:131-136 (diag = 0.5 Ne / N_fine;
                           V = (V11 + V22)/2 as in Source/xsf.f90:44-45)
* nbands                   Source/io.f90:316 (n_electrons + conduction_bands)
* LDA exchange/correlation libxc 6.2.2 vendored in ExLib/libxc:
                           maple/util.mpl:39-97 (LDA_X_FACTOR, RS_FACTOR),
                           maple/lda_exc/lda_c_pw.mpl:18-45 (PW92, id 12),
                           src/lda_c_pw.c:41-50 (parameters),
                           src/work_lda_inc.c:50-56 (density threshold 1e-15)

Everything the reference never implemented (its SCF loop, density, V.psi and
overlap routines are stubs: Source/electronic.f90:135-167,
Source/density.f90:101-130, Source/pot.f90:344-382, Source/wave.f90:929-1036)
is textbook plane-wave DFT, written out below: kinetic 1/2|k+G|^2, Hartree
4 pi n(G)/|G|^2 with G=0 dropped, Fermi-Dirac occupations with bisection for
the Fermi level, Pulay (DIIS) density mixing with optional Kerker
preconditioning, and the Kohn-Sham total and free energies.

Units are Hartree atomic units throughout.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

TWO_PI = 2.0 * math.pi
FOUR_PI = 4.0 * math.pi
DENS_THRESHOLD = 1e-15  # libxc lda_x.c:63 / lda_c_pw.c:130


# --------------------------------------------------------------------------
# Grid sizing and reciprocal-space tables
# --------------------------------------------------------------------------

def prime_fact_round(n: int, primes=(2, 3, 5, 7, 11, 13), max_cycles: int = 100) -> int:
    """Smallest m >= n whose prime factors all lie in ``primes``.

    Restates basis_prime_fact (Source/basis.f90:257-309): strip every listed
    prime from N repeatedly; if nothing else remains N is accepted, otherwise
    N is incremented (at most ``max_cycles`` times).
    """
    for _ in range(max_cycles):
        m = n
        changed = True
        while changed:
            changed = False
            for p in primes:
                if m % p == 0:
                    m //= p
                    changed = True
        if m == 1:
            return n
        n += 1
    return n


def smooth23_round(n: int) -> int:
    """Smallest m >= n of the form 2^a 3^b (the {2,3}-smooth grid policy)."""
    return prime_fact_round(n, primes=(2, 3), max_cycles=1 << 20)


def lattice_lengths(cell: np.ndarray) -> np.ndarray:
    """|a|,|b|,|c| as the norms of the columns of cell (Source/io.f90:1956-1966)."""
    cell = np.asarray(cell, dtype=np.float64)
    return np.sqrt((cell ** 2).sum(axis=0))


def inv_cell(cell: np.ndarray) -> np.ndarray:
    """transpose(2 pi * inverse(cell)) (Source/io.f90:1954).

    G = inv_cell @ (i, j, k) for integer Miller indices (Source/basis.f90:130-131).
    """
    return np.ascontiguousarray((TWO_PI * np.linalg.inv(np.asarray(cell, dtype=np.float64))).T)


def cell_volume(cell: np.ndarray) -> float:
    return float(abs(np.linalg.det(np.asarray(cell, dtype=np.float64))))


def grid_sizes(cell, ecut: float, g_fine_scale: float = 2.0, policy: str = "reference"):
    """Standard and fine FFT grid sizes (Source/basis.f90:87-105).

    policy "reference": round the fine grid to {2,3,5,7,11,13}-smooth sizes as
    the reference; policy "smooth23": round it to {2,3}-smooth sizes.  The
    standard box is always rounded by the reference rule.
    Returns (n_std[3], n_fine[3]) as int tuples.
    """
    k_cut = math.sqrt(2.0 * ecut)
    lengths = lattice_lengths(cell)
    std = [math.ceil(k_cut * L / math.pi) for L in lengths]
    fine = [math.ceil(g_fine_scale * k_cut * L / math.pi) for L in lengths]
    rnd = prime_fact_round if policy == "reference" else smooth23_round
    # the standard box defines the G list, so it always follows the reference rule
    return tuple(prime_fact_round(n) for n in std), tuple(rnd(n) for n in fine)


def centred_range(n: int) -> np.ndarray:
    """Miller range -n/2 .. n - n/2 - 1 with Fortran integer division (basis.f90:126)."""
    return np.arange(-(n // 2), n - n // 2, dtype=np.int64)


def miller_box(n_std) -> np.ndarray:
    """Centred Miller indices of the standard box, x outermost, z innermost
    (Source/basis.f90:125-135).  Row ig-1 holds grid_points(ig,:) / inv_cell."""
    rx, ry, rz = (centred_range(n) for n in n_std)
    mx, my, mz = np.meshgrid(rx, ry, rz, indexing="ij")
    return np.stack([mx.ravel(), my.ravel(), mz.ravel()], axis=1)


def mp_kpoints(grid) -> np.ndarray:
    """Monkhorst-Pack list in fractional reciprocal coordinates
    (Source/io.f90:2016-2031): k_i = n d - (1 + d)/2, d = 1/N_i, n = 1..N_i,
    x outermost, z innermost."""
    out = []
    d = [1.0 / g for g in grid]
    for a in range(1, grid[0] + 1):
        for b in range(1, grid[1] + 1):
            for c in range(1, grid[2] + 1):
                out.append([a * d[0] - (1.0 + d[0]) / 2,
                            b * d[1] - (1.0 + d[1]) / 2,
                            c * d[2] - (1.0 + d[2]) / 2])
    return np.array(out, dtype=np.float64)


def gsphere(cell, ecut: float, kfrac, n_std, inv_cell_given=None):
    """Plane-wave sphere for one k-point.

    The sphere is the ordered subsequence of the reference's standard-box
    G list (Source/basis.f90:125-135) with 1/2 |k+G|^2 <= ecut.  Returns
    (box_rows, miller, kinetic): 0-based row numbers into the box list, the
    Miller indices (Npw,3) and 1/2|k+G|^2 (Npw,).
    """
    B = inv_cell(cell) if inv_cell_given is None else np.asarray(inv_cell_given, dtype=np.float64)
    m = miller_box(n_std)
    kq = m.astype(np.float64) + np.asarray(kfrac, dtype=np.float64)[None, :]
    # G_i = inv_cell(i,1) q1 + inv_cell(i,2) q2 + inv_cell(i,3) q3, summed left to
    # right without fused multiply-adds (the order of Fortran's matmul loop)
    g = [(B[i, 0] * kq[:, 0] + B[i, 1] * kq[:, 1]) + B[i, 2] * kq[:, 2] for i in range(3)]
    kin = 0.5 * ((g[0] * g[0] + g[1] * g[1]) + g[2] * g[2])
    rows = np.nonzero(kin <= ecut)[0]
    return rows.astype(np.int64), m[rows], kin[rows]


def fft_flat_index(miller: np.ndarray, n_fine) -> np.ndarray:
    """Flat z-fastest index (ix*ny + iy)*nz + iz of Miller indices wrapped
    into the fine FFT box (Source/fft.f90:260,273 layout)."""
    n1, n2, n3 = n_fine
    ix = np.mod(miller[:, 0], n1)
    iy = np.mod(miller[:, 1], n2)
    iz = np.mod(miller[:, 2], n3)
    return (ix * n2 + iy) * n3 + iz


def fft_miller(n: int) -> np.ndarray:
    """Miller index of each FFT index 0..n-1 under the reference's centred
    convention: i for i < n - n/2, else i - n (basis.f90:126 range)."""
    i = np.arange(n, dtype=np.int64)
    return np.where(i < n - n // 2, i, i - n)


def gvec_sq_grid(cell, n_fine) -> np.ndarray:
    """|G|^2 on the fine FFT box (n1,n2,n3)."""
    B = inv_cell(cell)
    m1, m2, m3 = (fft_miller(n) for n in n_fine)
    M = np.stack(np.meshgrid(m1, m2, m3, indexing="ij"), axis=-1).astype(np.float64)
    G = M @ B.T
    return (G * G).sum(axis=-1)


def real_frac_points(n_fine) -> np.ndarray:
    """Fractional coordinates of the reference's real grid, frac = i/n with
    i = 1..n (Source/basis.f90:156-188), z-fastest flat order, shape (N,3)."""
    f = [np.arange(1, n + 1, dtype=np.float64) / n for n in n_fine]
    fx, fy, fz = np.meshgrid(*f, indexing="ij")
    return np.stack([fx.ravel(), fy.ravel(), fz.ravel()], axis=1)


# --------------------------------------------------------------------------
# External potential
# --------------------------------------------------------------------------

def vext_jellium_wells(cell, n_fine, n_electrons: float, wells) -> np.ndarray:
    """Jellium constant plus attractive Gaussian wells on the fine grid.

    The constant follows the reference's 'jelly' case (Source/pot.f90:133-134:
    each diagonal entry 0.5 Ne / N_fine, so V = (V11+V22)/2 = 0.5 Ne / N_fine).
    Each well i (fractional centre c_i, depth U_i > 0, width w_i) subtracts
    U_i exp(-|r - R_i|^2 / (2 w_i^2)) using the minimum-image distance.  The
    reference parses such wells (Source/io.f90:1888-1922) but sets them to
    zero (Source/pot.f90:165-166); this is the intended form.
    Points are sampled at the reference's real grid (frac = i/n, i = 1..n).
    Returns V(r) as a flat float64 array in z-fastest order.
    """
    cell = np.asarray(cell, dtype=np.float64)
    N = int(np.prod(n_fine))
    frac = real_frac_points(n_fine)
    v = np.full(N, 0.5 * n_electrons / N, dtype=np.float64)
    for (cx, cy, cz, depth, width) in np.asarray(wells, dtype=np.float64).reshape(-1, 5):
        d = frac - np.array([cx, cy, cz])[None, :]
        d -= np.rint(d)
        r = d @ cell.T
        r2 = (r * r).sum(axis=1)
        v -= depth * np.exp(-r2 / (2.0 * width * width))
    return v


def random_wells(rng: np.random.Generator, count: int,
                 depth=(1.0, 3.0), width=(0.8, 1.5)) -> np.ndarray:
    """Seeded wells: rows (cx, cy, cz, depth, width), centres fractional U[0,1)."""
    c = rng.random((count, 3))
    d = rng.uniform(depth[0], depth[1], count)
    w = rng.uniform(width[0], width[1], count)
    return np.concatenate([c, d[:, None], w[:, None]], axis=1)


# --------------------------------------------------------------------------
# FFT with the reference's conventions
# --------------------------------------------------------------------------

def fft3d(flat: np.ndarray, n_fine, direction: int) -> np.ndarray:
    """3D c2c DFT of a z-fastest flat array, unnormalised both ways.

    direction=+1 is FFTW_FORWARD (exponent -i), direction=-1 FFTW_BACKWARD
    (exponent +i), Source/fft.f90:264-284.  numpy.fft stands in for FFTW.
    """
    a = np.asarray(flat, dtype=np.complex128).reshape(n_fine)
    if direction == 1:
        out = np.fft.fftn(a)
    elif direction == -1:
        out = np.fft.ifftn(a) * a.size
    else:
        raise ValueError("direction must be +1 or -1")
    return out.ravel()


# --------------------------------------------------------------------------
# LDA exchange-correlation (Slater + Perdew-Wang 92), spin-unpolarised
# --------------------------------------------------------------------------

PW92 = dict(a=0.031091, alpha1=0.21370, beta1=7.5957, beta2=3.5876,
            beta3=1.6382, beta4=0.49294, p=1.0)


def lda_x_c(rho: np.ndarray):
    """(eps_x, v_x, eps_c, v_c) for spin-unpolarised densities.

    Exchange: eps_x = -(3/4)(3/pi)^{1/3} n^{1/3} (maple/util.mpl:58,86-94 with
    zeta=0), v_x = 4/3 eps_x.  Correlation: PW92 G(rs) of
    maple/lda_exc/lda_c_pw.mpl:34-37 with the first parameter column of
    src/lda_c_pw.c:41-50 (zeta = 0 kills the spin-stiffness terms),
    v_c = eps_c - rs/3 d eps_c/d rs.  rs = (3/(4 pi n))^{1/3}.
    Densities below 1e-15 give zeros (src/work_lda_inc.c:50); exchange is also
    screened when n/2 <= 1e-15 (maple/util.mpl:102).
    """
    rho = np.asarray(rho, dtype=np.float64)
    out = [np.zeros_like(rho) for _ in range(4)]
    mask = rho >= DENS_THRESHOLD
    n = np.maximum(rho[mask], DENS_THRESHOLD)
    ex = -0.75 * (3.0 / math.pi) ** (1.0 / 3.0) * np.cbrt(n)
    xmask = (0.5 * n) > DENS_THRESHOLD
    ex = np.where(xmask, ex, 0.0)
    vx = 4.0 / 3.0 * ex
    rs = (3.0 / (FOUR_PI * n)) ** (1.0 / 3.0)
    P = PW92
    srs = np.sqrt(rs)
    q0 = -2.0 * P["a"] * (1.0 + P["alpha1"] * rs)
    q1 = 2.0 * P["a"] * (P["beta1"] * srs + P["beta2"] * rs + P["beta3"] * rs * srs
                         + P["beta4"] * rs ** (P["p"] + 1.0))
    dq1 = P["a"] * (P["beta1"] / srs + 2.0 * P["beta2"] + 3.0 * P["beta3"] * srs
                    + 2.0 * (P["p"] + 1.0) * P["beta4"] * rs ** P["p"])
    lg = np.log(1.0 + 1.0 / q1)  # libxc evaluates log(1 + x), not log1p
    ec = q0 * lg
    dec = -2.0 * P["a"] * P["alpha1"] * lg - q0 * dq1 / (q1 * q1 + q1)
    vc = ec - rs / 3.0 * dec
    for o, v in zip(out, (ex, vx, ec, vc)):
        o[mask] = v
    return tuple(out)


# PW92 parameter columns of src/lda_c_pw.c:41-50: eps_c(rs, 0), eps_c(rs, 1)
# and -alpha_c(rs); fz20 = f''(0)
PW92_POL = dict(a=(0.031091, 0.015545, 0.016887), alpha1=(0.21370, 0.20548, 0.11125),
                beta1=(7.5957, 14.1189, 10.357), beta2=(3.5876, 6.1977, 3.6231),
                beta3=(1.6382, 3.3662, 0.88026), beta4=(0.49294, 0.62517, 0.49671), fz20=1.709921)
ZETA_THRESHOLD = np.finfo(np.float64).eps   # libxc's default zeta threshold


def _pw_g(k: int, rs: np.ndarray):
    """G_k(rs) of maple/lda_exc/lda_c_pw.mpl:34-37 (equation 10 of Perdew and
    Wang 1992) and dG_k/drs for parameter column k."""
    P = PW92_POL
    a, al = P["a"][k], P["alpha1"][k]
    srs = np.sqrt(rs)
    q0 = -2.0 * a * (1.0 + al * rs)
    q1 = 2.0 * a * (P["beta1"][k] * srs + P["beta2"][k] * rs + P["beta3"][k] * rs * srs + P["beta4"][k] * rs * rs)
    dq1 = a * (P["beta1"][k] / srs + 2.0 * P["beta2"][k] + 3.0 * P["beta3"][k] * srs + 4.0 * P["beta4"][k] * rs)
    lg = np.log(1.0 + 1.0 / q1)
    return q0 * lg, -2.0 * a * al * lg - q0 * dq1 / (q1 * q1 + q1)


def lda_pol(rhoa: np.ndarray, rhob: np.ndarray):
    """Spin-polarised LDA_X + LDA_C_PW: (eps_x, v_x (n, 2), eps_c, v_c (n, 2)).

    Follows libxc 6.2.2: each spin density is raised to the density
    threshold and points with rhoa + rhob below it give zeros
    (src/work_lda_inc.c:48-55); zeta is kept 1e-16 inside [-1, 1] (z_thr,
    maple/util.mpl:77-82); an exchange channel with n_s <= threshold is
    screened (maple/util.mpl:101-110).  Exchange per channel is
    -(3/8)(3/pi)^{1/3} (2 n_s)^{4/3} / n, v_x,s = -(6 n_s / pi)^{1/3}.
    Correlation: eps_c = G1 + z^4 f(z) (G2 - G1 + G3/fz20) - f(z) G3/fz20
    (maple/lda_exc/lda_c_pw.mpl:42-44), f(z) = ((1+z)^{4/3} + (1-z)^{4/3} - 2)
    / (2^{4/3} - 2); v_c,s = eps_c - rs/3 d eps_c/drs -/+ (z -/+ 1) d eps_c/dz.
    """
    ra = np.asarray(rhoa, dtype=np.float64)
    rb = np.asarray(rhob, dtype=np.float64)
    n_pts = ra.shape[0]
    ex = np.zeros(n_pts)
    ec = np.zeros(n_pts)
    vx = np.zeros((n_pts, 2))
    vc = np.zeros((n_pts, 2))
    mask = (ra + rb) >= DENS_THRESHOLD
    na = np.maximum(ra[mask], DENS_THRESHOLD)
    nb = np.maximum(rb[mask], DENS_THRESHOLD)
    n = na + nb
    zt = ZETA_THRESHOLD
    # 1 +/- zeta as 2 n_s / n: no cancellation next to full polarisation
    opz = 2.0 * na / n
    omz = 2.0 * nb / n
    opz, omz = np.where(opz <= zt, zt, np.where(omz <= zt, 2.0 - zt, opz)), \
        np.where(omz <= zt, zt, np.where(opz <= zt, 2.0 - zt, omz))
    z = opz - 1.0
    cx = -0.75 * (3.0 / math.pi) ** (1.0 / 3.0)
    e_x = np.zeros_like(n)
    for ns, sign, col in ((na, 1.0, 0), (nb, -1.0, 1)):
        live = ns > DENS_THRESHOLD
        opz_s = opz if sign > 0 else omz
        e_x += np.where(live, 0.5 * cx * np.cbrt(n) * opz_s ** (4.0 / 3.0), 0.0)
        vx_s = np.where(live, -np.cbrt(6.0 * ns / math.pi), 0.0)
        tmp = np.zeros(n_pts)
        tmp[mask] = vx_s
        vx[:, col] = tmp
    ex[mask] = e_x
    rs = (3.0 / (FOUR_PI * n)) ** (1.0 / 3.0)
    g1, d1 = _pw_g(0, rs)
    g2, d2 = _pw_g(1, rs)
    g3, d3 = _pw_g(2, rs)
    fz20 = PW92_POL["fz20"]
    den = 2.0 ** (4.0 / 3.0) - 2.0
    fz = (opz ** (4.0 / 3.0) + omz ** (4.0 / 3.0) - 2.0) / den
    dfz = (4.0 / 3.0) * (np.cbrt(opz) - np.cbrt(omz)) / den
    z4 = z ** 4
    e_c = g1 + z4 * fz * (g2 - g1 + g3 / fz20) - fz * g3 / fz20
    de_rs = d1 + z4 * fz * (d2 - d1 + d3 / fz20) - fz * d3 / fz20
    de_z = (4.0 * z ** 3 * fz + z4 * dfz) * (g2 - g1 + g3 / fz20) - dfz * g3 / fz20
    base = e_c - rs / 3.0 * de_rs
    ec[mask] = e_c
    tmp = np.zeros(n_pts)
    tmp[mask] = base + omz * de_z
    vc[:, 0] = tmp
    tmp = np.zeros(n_pts)
    tmp[mask] = base - opz * de_z
    vc[:, 1] = tmp
    return ex, vx, ec, vc


def lda_exc_vxc(rho: np.ndarray):
    ex, vx, ec, vc = lda_x_c(rho)
    return ex + ec, vx + vc


# --------------------------------------------------------------------------
# Deterministic start vectors (same hash as the GPU library)
# --------------------------------------------------------------------------

MASK64 = (1 << 64) - 1


def splitmix64(x: np.ndarray) -> np.ndarray:
    x = (x + np.uint64(0x9E3779B97F4A7C15)) & np.uint64(MASK64)
    z = x
    z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & np.uint64(MASK64)
    z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & np.uint64(MASK64)
    return z ^ (z >> np.uint64(31))


def start_wavefunctions(seed: int, sys_index: int, k_index: int, nbands: int, npw: int) -> np.ndarray:
    """Real start coefficients r - 0.5 per (band, G) like wave_initialise_wfn
    (Source/wave.f90:873-886), drawn from a counter hash instead of the
    Fortran generator so every implementation produces the same numbers.
    Returns (nbands, npw) complex128."""
    with np.errstate(over="ignore"):
        b = np.arange(nbands, dtype=np.uint64)[:, None]
        g = np.arange(npw, dtype=np.uint64)[None, :]
        key = (np.uint64(seed) * np.uint64(0x100000001B3)
               ^ (np.uint64(sys_index) << np.uint64(40))
               ^ (np.uint64(k_index) << np.uint64(24)))
        ctr = (key + b * np.uint64(1 << 20) + g) & np.uint64(MASK64)
        h = splitmix64(ctr)
    u = (h >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    return (u - 0.5).astype(np.complex128)


# --------------------------------------------------------------------------
# System description
# --------------------------------------------------------------------------

@dataclass
class System:
    cell: np.ndarray
    ecut: float
    n_fine: tuple
    n_std: tuple
    kpts: np.ndarray            # (nk,3) fractional
    wk: np.ndarray              # (nk,) weights summing to 1
    nbands: int
    nelec: float
    kT: float
    vext: np.ndarray            # flat (N,)
    wells: np.ndarray = field(default_factory=lambda: np.zeros((0, 5)))

    @property
    def nr(self) -> int:
        return int(np.prod(self.n_fine))

    @property
    def volume(self) -> float:
        return cell_volume(self.cell)


def make_system(L: float, ecut: float, nelec: float, nbands: int, wells,
                kgrid=(1, 1, 1), kpts=None, kT: float = 0.01,
                policy: str = "smooth23", g_fine_scale: float = 2.0) -> System:
    """Cubic-cell system with the jellium + wells potential."""
    cell = np.eye(3) * float(L)
    n_std, n_fine = grid_sizes(cell, ecut, g_fine_scale, policy)
    if kpts is None:
        kpts = mp_kpoints(kgrid)
    kpts = np.asarray(kpts, dtype=np.float64).reshape(-1, 3)
    wk = np.full(len(kpts), 1.0 / len(kpts))
    wells = np.asarray(wells, dtype=np.float64).reshape(-1, 5)
    vext = vext_jellium_wells(cell, n_fine, nelec, wells)
    return System(cell, ecut, tuple(n_fine), tuple(n_std), kpts, wk, nbands,
                  float(nelec), float(kT), vext, wells)


# --------------------------------------------------------------------------
# Hamiltonian pieces
# --------------------------------------------------------------------------

class KBasis:
    """Sphere data of one k-point: Miller indices, FFT indices, kinetic."""

    def __init__(self, sys: System, ik: int):
        rows, mil, kin = gsphere(sys.cell, sys.ecut, sys.kpts[ik], sys.n_std)
        self.rows = rows
        self.miller = mil
        self.kinetic = kin
        self.fidx = fft_flat_index(mil, sys.n_fine)
        self.npw = len(rows)


def apply_h(sys: System, kb: KBasis, vloc: np.ndarray, psi: np.ndarray) -> np.ndarray:
    """H psi for psi of shape (nb, npw): 1/2|k+G|^2 psi + (1/N) F[V F^-1 psi].

    F^-1 is the reference's unnormalised backward transform (dir=-1) and F the
    forward one (dir=+1); the 1/N restores the DFT normalisation.
    """
    N = sys.nr
    out = np.empty_like(psi)
    box = np.zeros(N, dtype=np.complex128)
    for b in range(psi.shape[0]):
        box[:] = 0
        box[kb.fidx] = psi[b]
        r = fft3d(box, sys.n_fine, -1)
        r *= vloc
        g = fft3d(r, sys.n_fine, 1)
        out[b] = kb.kinetic * psi[b] + g[kb.fidx] / N
    return out


def apply_h_block(sys: System, kb: KBasis, vloc: np.ndarray, psi: np.ndarray,
                  chunk: int = 16, workers=None) -> np.ndarray:
    """apply_h for a block psi (nb, npw), the bands of a chunk transformed
    together by scipy.fft (norm="forward": the backward transform is the
    reference's unnormalised dir=-1, the forward one carries the 1/N).  Same
    arithmetic as apply_h, batched for the large grids."""
    import scipy.fft as sfft
    nf = tuple(int(x) for x in sys.n_fine)
    v = vloc.reshape(nf)
    out = np.empty_like(psi)
    for b0 in range(0, psi.shape[0], chunk):
        p = psi[b0:b0 + chunk]
        box = np.zeros((p.shape[0], sys.nr), dtype=np.complex128)
        box[:, kb.fidx] = p
        r = sfft.ifftn(box.reshape((-1,) + nf), axes=(1, 2, 3), norm="forward", workers=workers)
        r *= v
        g = sfft.fftn(r, axes=(1, 2, 3), norm="forward", workers=workers)
        out[b0:b0 + chunk] = kb.kinetic * p + g.reshape(p.shape[0], -1)[:, kb.fidx]
    return out


def _orthonormalise(X: np.ndarray) -> np.ndarray:
    """Rows of X made orthonormal: S = conj(X) X^T = L L^H, X <- conj(L)^-1 X."""
    import scipy.linalg as sla
    S = X.conj() @ X.T
    L = np.linalg.cholesky(0.5 * (S + S.conj().T))
    return sla.solve_triangular(L.conj(), X, lower=True)


def _rayleigh_ritz(sys, kb, vloc, X, workers):
    X = _orthonormalise(X)
    HX = apply_h_block(sys, kb, vloc, X, workers=workers)
    Hs = X.conj() @ HX.T
    w, U = np.linalg.eigh(0.5 * (Hs + Hs.conj().T))
    return w, U.T @ X, U.T @ HX


def eigensolve_filtered(sys: System, kb: KBasis, vloc: np.ndarray, X: np.ndarray, nconv: int,
                        tol: float = 1e-9, degree: int = 12, max_pass: int = 400, workers=None,
                        ntight: int = None, tail_tol: float = 1e-7, fixed_passes: int = None):
    """Lowest eigenpairs of H(k) by Chebyshev-filtered subspace iteration with
    Rayleigh-Ritz (Zhou, Saad, Tiago, Chelikowsky, J. Comput. Phys. 219
    (2006) 172), in FP64.  X (m, npw) is the start block (m > nconv buffer
    rows speed up the lowest nconv).  Iterates until the residual norms
    |H x - eps x| of the lowest nconv Ritz pairs are below tol (with ntight
    given: the lowest ntight below tol and the rest below max(tol, tail_tol),
    for empty bands whose eigenvalue error, of order residual^2 / gap, stays
    far below the parity tolerance); returns (eps (m,), X (m, npw)
    orthonormal Ritz vectors, passes); with fixed_passes, exactly that many
    filter passes and no convergence test.  The filter damps
    [eps_top, b] with b = ecut + max V, an upper bound of the spectrum
    (kinetic <= ecut on the sphere, <psi|V|psi> <= max V |psi|^2)."""
    b = sys.ecut + float(vloc.max()) + 0.1
    w, X, HX = _rayleigh_ritz(sys, kb, vloc, X, workers)
    for p in range(max_pass if fixed_passes is None else fixed_passes + 1):
        if fixed_passes is not None:
            if p == fixed_passes:
                return w, X, p
        else:
            R = np.linalg.norm(HX[:nconv] - w[:nconv, None] * X[:nconv], axis=1)
            nt = nconv if ntight is None else max(1, min(ntight, nconv))
            if float(np.max(R[:nt])) < tol and (nt == nconv or float(np.max(R[nt:])) < max(tol, tail_tol)):
                return w, X, p
        a, a0 = float(w[-1]), float(w[0])
        e, c = 0.5 * (b - a), 0.5 * (b + a)
        sigma = e / (a0 - c)
        s1 = sigma
        Y = (HX - c * X) * (s1 / e)
        Xp = X
        for _ in range(1, degree):
            s2 = 1.0 / (2.0 / s1 - sigma)
            Yn = (2.0 * s2 / e) * (apply_h_block(sys, kb, vloc, Y, workers=workers) - c * Y) - (sigma * s2) * Xp
            Xp, Y, sigma = Y, Yn, s2
        w, X, HX = _rayleigh_ritz(sys, kb, vloc, Y, workers)
    raise RuntimeError(f"eigensolve_filtered: no convergence to {tol} in {max_pass} passes")


def dense_h(sys: System, kb: KBasis, vloc: np.ndarray) -> np.ndarray:
    """Dense Npw x Npw Hamiltonian: T + V(G - G') with V(G) = F[V]/N."""
    vG = fft3d(vloc.astype(np.complex128), sys.n_fine, 1).reshape(sys.n_fine) / sys.nr
    d = kb.miller[:, None, :] - kb.miller[None, :, :]
    n1, n2, n3 = sys.n_fine
    H = vG[np.mod(d[..., 0], n1), np.mod(d[..., 1], n2), np.mod(d[..., 2], n3)]
    H[np.diag_indices_from(H)] += kb.kinetic
    return H


def band_density(sys: System, kb: KBasis, psi: np.ndarray, weights: np.ndarray) -> np.ndarray:
    """sum_b weights[b] |psi_b(r)|^2 / Omega with psi_b(r) = F^-1[c_b]."""
    N = sys.nr
    rho = np.zeros(N, dtype=np.float64)
    box = np.zeros(N, dtype=np.complex128)
    for b in range(psi.shape[0]):
        if weights[b] == 0.0:
            continue
        box[:] = 0
        box[kb.fidx] = psi[b]
        r = fft3d(box, sys.n_fine, -1)
        rho += weights[b] * (r.real ** 2 + r.imag ** 2)
    return rho / sys.volume


def band_density_block(sys: System, kb: KBasis, psi: np.ndarray, weights: np.ndarray,
                       chunk: int = 16, workers=None) -> np.ndarray:
    """band_density with the bands of a chunk transformed together (scipy.fft)."""
    import scipy.fft as sfft
    nf = tuple(int(x) for x in sys.n_fine)
    rho = np.zeros(sys.nr, dtype=np.float64)
    occ = np.nonzero(np.asarray(weights) != 0.0)[0]
    for c0 in range(0, len(occ), chunk):
        sel = occ[c0:c0 + chunk]
        box = np.zeros((len(sel), sys.nr), dtype=np.complex128)
        box[:, kb.fidx] = psi[sel]
        r = sfft.ifftn(box.reshape((-1,) + nf), axes=(1, 2, 3), norm="forward", workers=workers)
        r = r.reshape(len(sel), -1)
        rho += np.einsum("b,bn->n", np.asarray(weights)[sel], r.real ** 2 + r.imag ** 2)
    return rho / sys.volume


# --------------------------------------------------------------------------
# Non-collinear spinors: coeff(gvec, band, 1:2) (Source/wave.f90:30,164), the
# 2x2 nc_pot (Source/pot.f90:33) and den%spin(nr, 3) (Source/density.f90:64).
# The reference leaves the products on them as stubs; these are their
# definitions, reducing to apply_h / band_density per component when nc_pot
# is diag(V, V).
# --------------------------------------------------------------------------

MU_B = 0.5   # Bohr magneton in atomic units (Source/constants.f90:102)


def nc_from_fields(v: np.ndarray, b: np.ndarray) -> np.ndarray:
    """nc_pot[n, i, j] = V I + mu_B sigma.B, the form whose components
    Source/xsf.f90:44-51 reads back; b has shape (3, nr)."""
    bx, by, bz = b
    nc = np.empty((len(v), 2, 2), dtype=np.complex128)
    nc[:, 0, 0] = v + MU_B * bz
    nc[:, 1, 1] = v - MU_B * bz
    nc[:, 0, 1] = MU_B * (bx - 1j * by)
    nc[:, 1, 0] = MU_B * (bx + 1j * by)
    return nc


def nc_components(nc: np.ndarray):
    """(V, Bx, By, Bz) of nc_pot as Source/xsf.f90:44-51 computes them."""
    v = (nc[:, 0, 0] + nc[:, 1, 1]) / 2.0
    bx = (nc[:, 0, 1] + nc[:, 1, 0]) / (MU_B * 2.0)
    by = (nc[:, 0, 1] - nc[:, 1, 0]) / (-MU_B * 2j)
    bz = (nc[:, 0, 0] - nc[:, 1, 1]) / (2.0 * MU_B)
    return v, bx, by, bz


def apply_h_spinor(sys: System, kb: KBasis, nc: np.ndarray, psi: np.ndarray) -> np.ndarray:
    """H psi for spinor psi of shape (2, nb, npw):
    (H psi)_s = 1/2|k+G|^2 psi_s + (1/N) F[sum_s' nc[:, s, s'] F^-1 psi_s']."""
    N = sys.nr
    out = np.empty_like(psi)
    box = np.zeros(N, dtype=np.complex128)
    for b in range(psi.shape[1]):
        r = []
        for sp in range(2):
            box[:] = 0
            box[kb.fidx] = psi[sp, b]
            r.append(fft3d(box, sys.n_fine, -1))
        for sp in range(2):
            w = nc[:, sp, 0] * r[0] + nc[:, sp, 1] * r[1]
            g = fft3d(w, sys.n_fine, 1)
            out[sp, b] = kb.kinetic * psi[sp, b] + g[kb.fidx] / N
    return out


def dense_h_spinor(sys: System, kb: KBasis, nc: np.ndarray) -> np.ndarray:
    """Dense 2 Npw x 2 Npw spinor Hamiltonian, blocks (s, s') of Npw rows:
    T delta_ss' + V_ss'(G - G') with V_ss'(G) = F[nc[:, s, s']] / N.  Row
    s * Npw + g holds spinor s of plane wave g (apply_h_spinor's layout)."""
    n1, n2, n3 = sys.n_fine
    d = kb.miller[:, None, :] - kb.miller[None, :, :]
    ix = (np.mod(d[..., 0], n1), np.mod(d[..., 1], n2), np.mod(d[..., 2], n3))
    npw = kb.npw
    H = np.zeros((2 * npw, 2 * npw), dtype=np.complex128)
    for a in range(2):
        for b in range(2):
            vG = fft3d(np.ascontiguousarray(nc[:, a, b]), sys.n_fine, 1).reshape(sys.n_fine) / sys.nr
            H[a * npw:(a + 1) * npw, b * npw:(b + 1) * npw] = vG[ix]
    H[np.diag_indices_from(H)] += np.concatenate([kb.kinetic, kb.kinetic])
    return H


def spinor_density(sys: System, kb: KBasis, psi: np.ndarray, weights: np.ndarray):
    """(n, m) with n = sum_b w_b (|u|^2 + |d|^2) / Omega and
    m = sum_b w_b psi^H sigma psi / Omega, shape (3, nr)."""
    N = sys.nr
    n = np.zeros(N)
    m = np.zeros((3, N))
    box = np.zeros(N, dtype=np.complex128)
    for b in range(psi.shape[1]):
        if weights[b] == 0.0:
            continue
        r = []
        for sp in range(2):
            box[:] = 0
            box[kb.fidx] = psi[sp, b]
            r.append(fft3d(box, sys.n_fine, -1))
        u, d = r
        ud = np.conj(u) * d
        n += weights[b] * (np.abs(u) ** 2 + np.abs(d) ** 2)
        m[0] += weights[b] * 2.0 * ud.real
        m[1] += weights[b] * 2.0 * ud.imag
        m[2] += weights[b] * (np.abs(u) ** 2 - np.abs(d) ** 2)
    return n / sys.volume, m / sys.volume


def hartree(sys: System, rho: np.ndarray):
    """(V_H(r), E_H): V_H(G) = 4 pi n(G)/|G|^2 with G = 0 dropped,
    n(G) = F[n]/N, E_H = Omega/2 sum_G 4 pi |n(G)|^2/|G|^2."""
    g2 = gvec_sq_grid(sys.cell, sys.n_fine).ravel()
    nG = fft3d(rho.astype(np.complex128), sys.n_fine, 1) / sys.nr
    with np.errstate(divide="ignore", invalid="ignore"):
        kern = np.where(g2 > 0, FOUR_PI / np.where(g2 > 0, g2, 1.0), 0.0)
    vG = kern * nG
    eh = 0.5 * sys.volume * float(np.sum(kern * (nG.real ** 2 + nG.imag ** 2)))
    vh = fft3d(vG, sys.n_fine, -1).real
    return vh, eh


def fermi_occupations(eigs: np.ndarray, wk: np.ndarray, nelec: float, kT: float, tol: float = 1e-14,
                      g: float = 2.0):
    """Fermi-Dirac occupations f in [0, g] (g = 2 for spin-degenerate bands,
    1 for spinor bands) with the Fermi level found by bisection so that
    sum_k w_k sum_n f_nk = Ne.  Returns (f, mu, entropy) where entropy
    S = -g sum w f~ ln f~ + (1-f~) ln(1-f~), f~ = f/g, so that the free
    energy is E - kT S."""
    lo = float(eigs.min()) - 50.0 * kT - 1.0
    hi = float(eigs.max()) + 50.0 * kT + 1.0

    def count(mu):
        x = np.clip((eigs - mu) / kT, -200.0, 200.0)
        f = g / (1.0 + np.exp(x))
        return float((wk[:, None] * f).sum())

    for _ in range(200):
        mid = 0.5 * (lo + hi)
        if count(mid) < nelec:
            lo = mid
        else:
            hi = mid
        if hi - lo < tol:
            break
    mu = 0.5 * (lo + hi)
    x = np.clip((eigs - mu) / kT, -200.0, 200.0)
    ft = 1.0 / (1.0 + np.exp(x))
    with np.errstate(divide="ignore", invalid="ignore"):
        s = np.where((ft > 0) & (ft < 1), ft * np.log(ft) + (1 - ft) * np.log1p(-ft), 0.0)
    entropy = -g * float((wk[:, None] * s).sum())
    return g * ft, mu, entropy


class PulayMixer:
    """Pulay (DIIS) density mixing with optional Kerker preconditioning.

    Residual R = n_out - n_in.  Coefficients c minimise |sum c_i R_i|^2 (plain
    r-space dot) subject to sum c_i = 1; the next input density is
    sum c_i n_in_i + P[sum c_i R_i] with P = alpha (q0 = 0) or
    alpha G^2/(G^2 + q0^2) applied in reciprocal space (Kerker).
    """

    def __init__(self, sys: System, alpha: float = 0.3, history: int = 8, q0: float = 0.0):
        self.sys = sys
        self.alpha = alpha
        self.history = history
        self.q0 = q0
        self.nin: list = []
        self.res: list = []
        if q0 > 0:
            g2 = gvec_sq_grid(sys.cell, sys.n_fine).ravel()
            self.kerker = g2 / (g2 + q0 * q0)
        else:
            self.kerker = None

    def precondition(self, r: np.ndarray) -> np.ndarray:
        if self.kerker is None:
            return self.alpha * r
        rG = fft3d(r.astype(np.complex128), self.sys.n_fine, 1)
        rG *= self.alpha * self.kerker
        return fft3d(rG, self.sys.n_fine, -1).real / self.sys.nr

    def mix(self, nin: np.ndarray, nout: np.ndarray) -> np.ndarray:
        self.nin.append(nin.copy())
        self.res.append(nout - nin)
        if len(self.nin) > self.history:
            self.nin.pop(0)
            self.res.pop(0)
        m = len(self.res)
        A = np.empty((m + 1, m + 1))
        for i in range(m):
            for j in range(m):
                A[i, j] = float(np.dot(self.res[i], self.res[j]))
        A[m, :m] = 1.0
        A[:m, m] = 1.0
        A[m, m] = 0.0
        rhs = np.zeros(m + 1)
        rhs[m] = 1.0
        c = np.linalg.lstsq(A, rhs, rcond=None)[0][:m]
        n_opt = sum(ci * ni for ci, ni in zip(c, self.nin))
        r_opt = sum(ci * ri for ci, ri in zip(c, self.res))
        return n_opt + self.precondition(r_opt)


@dataclass
class ScfResult:
    converged: bool
    iterations: int
    energy: float           # Kohn-Sham total energy of the output density
    free_energy: float      # energy - kT * entropy
    efermi: float
    eigenvalues: np.ndarray  # (nk, nb)
    occupations: np.ndarray  # (nk, nb)
    density: np.ndarray      # output density of the last iteration, flat
    history: list


def scf(sys: System, max_scf: int = 100, etol: float = 1e-10, alpha: float = 0.3,
        history: int = 8, q0: float = 0.0, solver: str = "dense", verbose: bool = False,
        rtol: float = None, buffer: int = 8, eig_tol: float = 1e-9, workers=None,
        nin0: np.ndarray = None, blocks0: list = None, keep: dict = None,
        passes: int = None) -> ScfResult:
    """Self-consistent field loop (the intended electronic_scf,
    Source/electronic.f90:86-175: iterate until |E - E_prev| < etol).

    Each iteration diagonalises H[n_in] (solver "dense": scipy eigh of the
    Npw x Npw matrix; "filtered": eigensolve_filtered warm-started from the
    previous iteration's Ritz vectors with `buffer` extra rows, residual
    norms below min(1e-4, 0.01 max|n_out - n_in|) and at least eig_tol, for
    spheres too large for a dense matrix), fills bands with Fermi-Dirac
    occupations, forms n_out, evaluates the energies of n_out and mixes.
    Start density: uniform Ne/Omega, or nin0; the filtered solver starts
    from blocks0 when given (a previous run's keep["blocks"]: a warm start
    for nearby parameters).  With rtol set, convergence also needs
    max|n_out - n_in| < rtol.  With `passes` the filtered solver runs that
    many filter passes per iteration instead of converging each eigenproblem
    (the subspace then converges together with the density, as in
    Chebyshev-filtered SCF); once the SCF test passes, the last iteration's
    eigenproblem is solved to eig_tol and that iteration's occupations,
    output density and energies are recomputed from it, so the result is the
    same fixed point the converged-per-iteration solver reaches.
    """
    import scipy.linalg as sla

    kbs = [KBasis(sys, ik) for ik in range(len(sys.kpts))]
    blocks = None
    if solver == "filtered":
        m = sys.nbands + buffer
        blocks = []
        for kb in kbs:
            # start: the m lowest-kinetic plane waves plus a small seeded perturbation
            X = np.zeros((m, kb.npw), dtype=np.complex128)
            X[np.arange(m), np.argsort(kb.kinetic, kind="stable")[:m]] = 1.0
            X += 1e-3 * start_wavefunctions(7, 0, len(blocks), m, kb.npw)
            blocks.append(X)
        if blocks0 is not None:
            blocks = [np.array(b) for b in blocks0]
    elif solver != "dense":
        raise ValueError(f"unknown solver {solver}")
    resid = 1.0
    omega = sys.volume
    N = sys.nr
    dv = omega / N
    nin = np.full(N, sys.nelec / omega) if nin0 is None else np.array(nin0, dtype=np.float64)
    mixer = PulayMixer(sys, alpha=alpha, history=history, q0=q0)
    e_prev = None
    hist = []
    result = None
    def evaluate(nin, vhxc, vloc, exact):
        eigs = np.zeros((len(kbs), sys.nbands))
        vecs = []
        for ik, kb in enumerate(kbs):
            if blocks is None:
                H = dense_h(sys, kb, vloc)
                w, v = sla.eigh(H, subset_by_index=[0, sys.nbands - 1], driver="evr")
                eigs[ik] = w
                vecs.append(v.T.copy())
            else:
                tol = eig_tol if exact else max(eig_tol, min(1e-4, 0.01 * resid))
                # bands below mu + 40 kT of the previous iteration carry the
                # density and energy: those converge to tol, empty ones to 1e-7
                nt = None if result is None else int(np.sum(result.eigenvalues[ik] < result.efermi + 40 * sys.kT)) + 1
                w, X, _ = eigensolve_filtered(sys, kb, vloc, blocks[ik], sys.nbands, tol=tol,
                                              workers=workers, ntight=nt,
                                              fixed_passes=None if exact else passes)
                blocks[ik] = X
                eigs[ik] = w[:sys.nbands]
                vecs.append(X[:sys.nbands])
        f, mu, ent = fermi_occupations(eigs, sys.wk, sys.nelec, sys.kT)
        nout = np.zeros(N)
        for ik, kb in enumerate(kbs):
            if blocks is None:
                nout += sys.wk[ik] * band_density(sys, kb, vecs[ik], f[ik])
            else:
                nout += sys.wk[ik] * band_density_block(sys, kb, vecs[ik], f[ik], workers=workers)
        eband = float((sys.wk[:, None] * f * eigs).sum())
        _, eh = hartree(sys, nout)
        exc_eps, _ = lda_exc_vxc(nout)
        exc = dv * float(np.dot(nout, exc_eps))
        e_dc = dv * float(np.dot(vhxc, nout))
        energy = eband - e_dc + eh + exc
        return eigs, f, mu, ent, nout, energy, energy - sys.kT * ent

    for it in range(1, max_scf + 1):
        vh, _ = hartree(sys, nin)
        _, vxc = lda_exc_vxc(nin)
        vhxc = vh + vxc
        vloc = sys.vext + vhxc
        eigs, f, mu, ent, nout, energy, free = evaluate(nin, vhxc, vloc, False)
        resid = float(np.max(np.abs(nout - nin)))
        hist.append((it, energy, free, mu, resid))
        if verbose:
            print(f"scf {it:3d} E={energy:.12f} F={free:.12f} mu={mu:.8f} |R|={resid:.2e}")
        result = ScfResult(False, it, energy, free, mu, eigs, f, nout, hist)
        if keep is not None and blocks is not None:
            keep["blocks"] = blocks
        if e_prev is not None and abs(free - e_prev) < etol and (rtol is None or resid < rtol):
            if blocks is not None and passes is not None:
                # the last iteration's eigenproblem solved to eig_tol
                eigs, f, mu, ent, nout, energy, free = evaluate(nin, vhxc, vloc, True)
                resid = float(np.max(np.abs(nout - nin)))
                hist.append((it, energy, free, mu, resid))
                if verbose:
                    print(f"exact {it:3d} E={energy:.12f} F={free:.12f} mu={mu:.8f} |R|={resid:.2e}")
                result = ScfResult(False, it, energy, free, mu, eigs, f, nout, hist)
            result.converged = True
            break
        e_prev = free
        nin = mixer.mix(nin, nout)
    return result


# --------------------------------------------------------------------------
# Non-collinear SCF (spinor bands, nspinor = 2)
# --------------------------------------------------------------------------

def xc_noncollinear(n: np.ndarray, m: np.ndarray):
    """(eps_xc, vbar, b) of the spin-polarised LDA on the local spin
    densities (n +/- |m|)/2: V_xc = vbar I + b.sigma with vbar = (v_up +
    v_down)/2 and b = (v_up - v_down)/2 m/|m| (b = 0 where m = 0)."""
    am = np.linalg.norm(m, axis=0)
    ex, vx, ec, vc = lda_pol(0.5 * (n + am), 0.5 * (n - am))
    va, vb = vx[:, 0] + vc[:, 0], vx[:, 1] + vc[:, 1]
    with np.errstate(divide="ignore", invalid="ignore"):
        sc = np.where(am > 0.0, 0.5 * (va - vb) / am, 0.0)
    return ex + ec, 0.5 * (va + vb), sc[None, :] * m


@dataclass
class SpinorScfResult:
    converged: bool
    iterations: int
    energy: float
    free_energy: float
    efermi: float
    eigenvalues: np.ndarray   # (nk, nb)
    occupations: np.ndarray   # (nk, nb), f in [0, 1]
    density: np.ndarray       # n_out
    magnetisation: np.ndarray  # m_out, (3, nr)
    history: list


def scf_spinor(sys: System, nc_ext: np.ndarray, max_scf: int = 100, etol: float = 1e-10,
               alpha: float = 0.3, history: int = 8, start_m: np.ndarray = None,
               verbose: bool = False, rtol: float = None) -> SpinorScfResult:
    """Non-collinear SCF in an external 2x2 potential nc_ext (nr, 2, 2).

    Each iteration diagonalises the dense spinor Hamiltonian of
    nc = nc_ext + (V_H[n_in] + vbar) I + b.sigma exactly, fills spinor bands
    (one electron each) with Fermi-Dirac occupations, forms n_out and m_out,
    evaluates E = sum w f eps - int (V_Hxc n_out + b.m_out) + E_H[n_out] +
    E_xc[n_out, m_out] and mixes (n, m) with Pulay on the stacked vector
    (plain dot, alpha, no Kerker).  Start: uniform n, m = start_m or 0.
    With rtol set, convergence also needs max|(n, m)_out - (n, m)_in| < rtol.
    """
    import scipy.linalg as sla

    kbs = [KBasis(sys, ik) for ik in range(len(sys.kpts))]
    N = sys.nr
    dv = sys.volume / N
    nin = np.full(N, sys.nelec / sys.volume)
    min_ = np.zeros((3, N)) if start_m is None else np.array(start_m, dtype=np.float64).reshape(3, N)
    mixer = PulayMixer(sys, alpha=alpha, history=history, q0=0.0)
    e_prev, hist, result = None, [], None
    for it in range(1, max_scf + 1):
        vh, _ = hartree(sys, nin)
        _, vbar, b = xc_noncollinear(nin, min_)
        vhxc = vh + vbar
        nc = np.array(nc_ext, dtype=np.complex128, copy=True)
        nc[:, 0, 0] += vhxc + b[2]
        nc[:, 1, 1] += vhxc - b[2]
        nc[:, 0, 1] += b[0] - 1j * b[1]
        nc[:, 1, 0] += b[0] + 1j * b[1]
        eigs = np.zeros((len(kbs), sys.nbands))
        vecs = []
        for ik, kb in enumerate(kbs):
            w, v = sla.eigh(dense_h_spinor(sys, kb, nc), subset_by_index=[0, sys.nbands - 1], driver="evr")
            eigs[ik] = w
            vecs.append(v.T.reshape(sys.nbands, 2, kb.npw).transpose(1, 0, 2).copy())
        f, mu, ent = fermi_occupations(eigs, sys.wk, sys.nelec, sys.kT, g=1.0)
        nout = np.zeros(N)
        mout = np.zeros((3, N))
        for ik, kb in enumerate(kbs):
            n_k, m_k = spinor_density(sys, kb, vecs[ik], f[ik])
            nout += sys.wk[ik] * n_k
            mout += sys.wk[ik] * m_k
        eband = float((sys.wk[:, None] * f * eigs).sum())
        _, eh = hartree(sys, nout)
        e_out, _, _ = xc_noncollinear(nout, mout)
        exc = dv * float(np.dot(nout, e_out))
        e_dc = dv * (float(np.dot(vhxc, nout)) + float(np.sum(b * mout)))
        energy = eband - e_dc + eh + exc
        free = energy - sys.kT * ent
        resid = max(float(np.max(np.abs(nout - nin))), float(np.max(np.abs(mout - min_))))
        hist.append((it, energy, free, mu, resid))
        if verbose:
            print(f"scf {it:3d} E={energy:.12f} F={free:.12f} mu={mu:.8f} |R|={resid:.2e}")
        result = SpinorScfResult(False, it, energy, free, mu, eigs, f, nout, mout, hist)
        if e_prev is not None and abs(free - e_prev) < etol and (rtol is None or resid < rtol):
            result.converged = True
            break
        e_prev = free
        x = mixer.mix(np.concatenate([nin, min_.ravel()]), np.concatenate([nout, mout.ravel()]))
        nin, min_ = x[:N], x[N:].reshape(3, N)
    return result


def external_nc_pot(p: dict, n_fine) -> np.ndarray:
    """nc_pot (nr, 2, 2) of pot_external_pot (Source/pot.f90:128-166) for
    the preset kinds, from a parameter dict as read_info returns it, with
    mu_B sigma.B of a uniform ext_bfield added.  A point-by-point loop over
    the reference's real grid (small grids only)."""
    n1, n2, n3 = n_fine
    nr = n1 * n2 * n3
    nc = np.zeros((nr, 2, 2), dtype=np.complex128)
    kind = p["external_pot"]
    half_w = [w / 2.0 for w in p["finite_barrier_width"]]
    g = p["periodic_pot_grid"]
    for ix in range(n1):
        for iy in range(n2):
            for iz in range(n3):
                r = (ix * n2 + iy) * n3 + iz
                fr = ((ix + 1) / n1, (iy + 1) / n2, (iz + 1) / n3)
                if kind == "jelly":
                    v = 0.5 * p["n_electrons"] / nr
                elif kind == "finite_barrier":
                    inside = all(abs(fr[a] - 0.5) < half_w[a] for a in range(3))
                    v = 0.5 * p["finite_barrier_height"] if inside else 0.0
                elif kind == "periodic_pot":
                    x = fr[0]
                    v = 0.5 * p["periodic_pot_amp"] * math.sin(2 * math.pi * g[0] * x) * \
                        math.sin(2 * math.pi * g[1] * x) * math.sin(2 * math.pi * g[2] * x)
                else:
                    v = 0.0
                nc[r, 0, 0] = nc[r, 1, 1] = v
    bx, by, bz = p["ext_bfield"]
    nc[:, 0, 0] += MU_B * bz
    nc[:, 1, 1] -= MU_B * bz
    nc[:, 0, 1] += MU_B * (bx - 1j * by)
    nc[:, 1, 0] += MU_B * (bx + 1j * by)
    return nc
