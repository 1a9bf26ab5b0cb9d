"""Synthetic RVE inputs for the named workloads.

No public dataset is involved: microstructures are periodic Voronoi tessellations of
seeded uniform points, orientations are Haar-random on SO(3) (Shoemake's subgroup
algorithm), converted to the Kocks angles the reference's orientation files carry
(src/mm10_a.f:1287-1345 convention).  Loading follows the reference's `.in` loading
semantics (src/inlod.f:57-63, src/inlodcase.f): BC_all(:, step) accumulates the
per-step increments and adds 1 on the diagonal of prescribed F components.
"""
from dataclasses import dataclass

import numpy as np

# MTS parameters (h_type 2) and the Ma-Roters-Raabe constants c1..c6 (h_type 7) at the
# reference's crystal defaults (initialize_new_crystal, src/mod_crystals.f:257-285); Voce
# crystals carry them unread.
MTS_DEFAULTS = dict(
    tau_a=0.0, tau_hat_y=-1.0, G_0_y=-1.0, p_y=0.5, q_y=2.0, tau_hat_v=-1.0, G_0_v=-1.0,
    p_v=0.5, q_v=2.0, eps_dot_0_v=1.0e10, burgers=2.87e-7, boltzman=1.3806e-20,
    mu_0=69000.0 / 2.0 / 1.33, D_0=0.0, T_0=294.0,
    u1=0.0, u2=0.0, u3=0.0, u4=0.0, u5=0.0, u6=0.0,
)

# Material of the named workloads (MPa, s): FCC {111}<110>, anisotropic type-3
# elasticity C11=C33=168.4, C12=C13=121.4, C44=C55=75.4 GPa, Voce hardening.
FCC_VOCE = dict(
    slip_type=1, elastic_type=3, e=0.0, nu=0.0, mu=0.0,
    C11=168400.0, C12=121400.0, C13=121400.0, C33=168400.0, C44=75400.0, C55=75400.0,
    h_type=1, harden_n=20.0, tau_y=50.0, tau_v=100.0, theta_0=400.0, voce_m=1.0,
    gamma_bar=1.0e-3, iD_v=0.0, alter_mode=1,
    atol=1.0e-10, atol1=1.0e-10, rtol=1.0e-10, rtol1=1.0e-10, miter=30,
    exact_j22=1, **MTS_DEFAULTS,
)

# The reference's example deck's crystal (examples/test_mm10.in): BCC with 48 slip
# systems, isotropic elasticity, Voce hardening (the deck's `harden_n 5,48` read as 5.48),
# the reference's own d(R2)/d(tau) (exact_j22 = 0).
BCC48_DECK = dict(
    slip_type=8, elastic_type=1, e=200000.0, nu=0.3, mu=0.0,
    C11=0.0, C12=0.0, C13=0.0, C33=0.0, C44=0.0, C55=0.0,
    h_type=1, harden_n=5.48, tau_y=205.0, tau_v=5000.0, theta_0=0.01, voce_m=1.0,
    gamma_bar=4.0e-5, iD_v=0.0, alter_mode=1,
    atol=1.0e-10, atol1=1.0e-10, rtol=1.0e-10, rtol1=1.0e-10, miter=30,
    exact_j22=0, **MTS_DEFAULTS,
)

# An HCP crystal (slip_type 9, hcp6: basal and prismatic <a> systems) with anisotropic
# type-3 elasticity of titanium's order (C11 = 162.4, C12 = 92.0, C13 = 69.0, C33 = 180.7,
# C44 = C55 = 46.7 GPa; the reference's type 3 sets C66 = C55) and Voce hardening.
HCP_VOCE = dict(
    FCC_VOCE, slip_type=9,
    C11=162400.0, C12=92000.0, C13=69000.0, C33=180700.0, C44=46700.0, C55=46700.0,
    tau_y=120.0, tau_v=200.0, theta_0=800.0,
)

# The material entry of a non-crystal material: not read by the crystal path (the
# bilinear Mises properties go through Solver.set_mises).
NOT_A_CRYSTAL = dict(FCC_VOCE, slip_type=0)


def single(x):
    """A deck value as the reference holds material properties: single precision (matprp
    is `real`, src/mod_fft.f:20), widened to double."""
    return float(np.float32(x))


# The two bilinear Mises materials of the reference's example deck (examples/test_mm01.in):
# (e, nu, yld_pt, tan_e, beta), single-precision values.
MM01_DECK = [
    dict(e=single(12000.0), nu=single(0.3), yld_pt=single(100.0), tan_e=single(1000.0),
         beta=single(0.5)),
    dict(e=single(24000.0), nu=single(0.3), yld_pt=single(200.0), tan_e=single(1000.0),
         beta=single(0.5)),
]

# An FCC crystal with MTS hardening (h_type 2): the workloads' elasticity, thermally
# activated thresholds tau_y(rate, T) and tau_v(rate, T) (MPa, mm, mJ/K), rate exponent 20.
MTS_FCC = dict(
    FCC_VOCE, h_type=2, harden_n=20.0, theta_0=2000.0, voce_m=1.0, alter_mode=0,
    tau_a=20.0, tau_hat_y=200.0, G_0_y=0.5, p_y=0.5, q_y=2.0,
    tau_hat_v=300.0, G_0_v=0.5, p_v=0.5, q_v=2.0, eps_dot_0_v=1.0e7, gamma_bar=1.0e7,
    burgers=2.5e-7, boltzman=1.3806e-20, mu_0=75400.0, D_0=0.0, T_0=294.0,
)

# An FCC crystal with Ma-Roters-Raabe hardening (h_type 7; N, mm, s, MPa): the workloads'
# elasticity, twelve dislocation densities starting at 1e6 / mm^2, thermally activated
# glide over the passing stress (Q_slip = 3e-16 N mm, 73 kT at 297 K; attack frequency
# 1e10 / s) with p = 1, q = 2 (with p < 1 the reference's fract**p is NaN wherever the
# resolved shear is below the passing stress), storage c4 = 0.01, athermal annihilation
# c5 = 5, dipole formation c6 = 1, thermal annihilation c7 = 0.01 (Q_bulk = 2.4e-16 N mm,
# exponent c8 = 0.3); exact local Jacobian.  The local solve fails for 5 % of random
# orientations under strain increments of 5e-3 (the slip increment jumps where the
# reference switches to its linear extrapolation, fract = 1, and the law is stiff).
MRR_FCC = dict(
    FCC_VOCE, h_type=7, exact_j22=1, alter_mode=0,
    tau_a=2.4e-16, G_0_v=3.0e-16, G_0_y=1.0e10, p_v=1.0, q_v=2.0,
    tau_hat_y=0.01, tau_hat_v=0.3, burgers=2.5e-7, boltzman=1.3806e-20, mu_0=75400.0,
    theta_0=1.0e6, u1=0.5, u2=0.1, u3=1.0, u4=0.01, u5=5.0, u6=1.0,
)

# An FCC crystal with ORNL hardening (h_type 4): MRR_FCC's densities and hardening
# constants, the shear modulus softened at 297 K (D_0 = 3000 MPa, T_0 = 200 K), slip at
# 0.1 rho_a v_s (c2 b) with v_s = 1e5 mm/s and c2 = 10, passing stress c1 mu b sqrt(rho_P),
# cutting stress c3 mu / mu_0 with c3 = 150 MPa, Q_slip = 3e-16 N mm, p = 0.5 (1 below the
# passing stress), q = 2.
ORNL_FCC = dict(
    MRR_FCC, h_type=4, G_0_y=1.0e5, G_0_v=3.0e-16, p_v=0.5, q_v=2.0, D_0=3000.0, T_0=200.0,
    u2=10.0, u3=150.0,
)

# component order of 9-vectors: 11,12,13,21,22,23,31,32,33
COMP = ["xx", "xy", "xz", "yx", "yy", "yz", "zx", "zy", "zz"]


def haar_quaternions(n, rng):
    """Uniform random unit quaternions (w, x, y, z) by Shoemake's method."""
    u1, u2, u3 = rng.random(n), rng.random(n), rng.random(n)
    a, b = np.sqrt(1.0 - u1), np.sqrt(u1)
    q = np.stack([b * np.cos(2 * np.pi * u3), a * np.sin(2 * np.pi * u2),
                  a * np.cos(2 * np.pi * u2), b * np.sin(2 * np.pi * u3)], axis=1)
    return q


def quat_to_matrix(q):
    w, x, y, z = q.T
    R = np.empty((len(q), 3, 3))
    R[:, 0, 0] = 1 - 2 * (y * y + z * z)
    R[:, 0, 1] = 2 * (x * y - w * z)
    R[:, 0, 2] = 2 * (x * z + w * y)
    R[:, 1, 0] = 2 * (x * y + w * z)
    R[:, 1, 1] = 1 - 2 * (x * x + z * z)
    R[:, 1, 2] = 2 * (y * z - w * x)
    R[:, 2, 0] = 2 * (x * z - w * y)
    R[:, 2, 1] = 2 * (y * z + w * x)
    R[:, 2, 2] = 1 - 2 * (x * x + y * y)
    return R


def kocks_matrix(ang_deg):
    """Rotation built from Kocks angles (psi, theta, phi) in degrees, the formula of
    mm10_rotation_matrix (src/mm10_a.f:1287-1345)."""
    a = np.radians(np.atleast_2d(ang_deg))
    psi, th, phi = a[:, 0], a[:, 1], a[:, 2]
    s, c = np.sin, np.cos
    r = np.empty((len(a), 3, 3))
    r[:, 0, 0] = -s(psi) * s(phi) - c(psi) * c(phi) * c(th)
    r[:, 0, 1] = c(psi) * s(phi) - s(psi) * c(phi) * c(th)
    r[:, 0, 2] = c(phi) * s(th)
    r[:, 1, 0] = s(psi) * c(phi) - c(psi) * s(phi) * c(th)
    r[:, 1, 1] = -c(psi) * c(phi) - s(psi) * s(phi) * c(th)
    r[:, 1, 2] = s(phi) * s(th)
    r[:, 2, 0] = c(psi) * s(th)
    r[:, 2, 1] = s(psi) * s(th)
    r[:, 2, 2] = c(th)
    return r


def matrix_to_kocks(R):
    """Inverse of kocks_matrix (the extraction of mm10_update_euler_angles,
    src/mm10_a.f:1171-1222), angles in degrees."""
    psi = np.arctan2(R[:, 2, 1], R[:, 2, 0])
    phi = np.arctan2(R[:, 1, 2], R[:, 0, 2])
    th = np.arccos(np.clip(R[:, 2, 2], -1.0, 1.0))
    return np.degrees(np.stack([psi, th, phi], axis=1))


def quat_to_kocks(q):
    return matrix_to_kocks(quat_to_matrix(q))


def periodic_voronoi(N, ngrains, rng):
    """Grain id (0-based) per voxel of an N^3 periodic Voronoi tessellation.  Voxel
    v = a + N*b + N*N*c sits at x = ((c+0.5)/N, (b+0.5)/N, (a+0.5)/N) (tensor index 1
    pairs with the slowest memory axis, src/FFT_init.f:310-318)."""
    seeds = rng.random((ngrains, 3))
    g = (np.arange(N) + 0.5) / N
    xc, xb, xa = np.meshgrid(g, g, g, indexing="ij")  # c slowest, a fastest
    pts = np.stack([xc.ravel(), xb.ravel(), xa.ravel()], axis=1)
    try:
        from scipy.spatial import cKDTree
        tree = cKDTree(seeds, boxsize=1.0)
        _, idx = tree.query(pts)
        return idx.astype(np.int64)
    except ImportError:  # pragma: no cover - scipy missing on a host
        best = np.full(len(pts), np.inf)
        idx = np.zeros(len(pts), dtype=np.int64)
        for k, s in enumerate(seeds):
            d = pts - s
            d -= np.round(d)
            r2 = (d * d).sum(1)
            m = r2 < best
            best[m] = r2[m]
            idx[m] = k
        return idx


@dataclass
class RVE:
    N: int
    grains: np.ndarray      # (N3,) 0-based grain id
    kocks: np.ndarray       # (3, N3) Kocks angles in degrees (column-major (N3,3))
    mat_list: np.ndarray    # (N3,) 1-based crystal number
    crystals: list          # crystal dicts
    quats: np.ndarray       # (ngrains, 4)


def make_rve(N, ngrains, seed, crystal=None):
    rng = np.random.default_rng(seed)
    grains = periodic_voronoi(N, ngrains, rng)
    q = haar_quaternions(ngrains, rng)
    ang = quat_to_kocks(q)                      # (ngrains, 3)
    kocks = np.ascontiguousarray(ang[grains].T)  # (3, N3)
    crystal = dict(crystal or FCC_VOCE)
    return RVE(N=N, grains=grains, kocks=kocks,
               mat_list=np.ones(N ** 3, dtype=np.int32), crystals=[crystal], quats=q)


@dataclass
class Loading:
    BC_all: np.ndarray   # (nstep, 9)
    isNBC: np.ndarray    # (9,) int
    name: str


def _accumulate(incr, isNBC, nstep):
    """BC_all as inlod builds it (src/inlod.f:57-63) for constant per-step increments."""
    mults = np.ones(nstep)
    bc = np.cumsum(np.outer(mults, incr), axis=0)
    for d in (0, 4, 8):
        if not isNBC[d]:
            bc[:, d] += 1.0
    return bc


def uniaxial_tension(total_strain, nstep):
    """F_xx prescribed; F_xy = F_xz = F_yz = 0 prescribed to suppress the rigid rotation
    about the load axis; the other five P components held at zero."""
    isNBC = np.array([0, 0, 0, 1, 1, 0, 1, 1, 1], dtype=np.int32)
    incr = np.zeros(9)
    incr[0] = total_strain / nstep
    return Loading(_accumulate(incr, isNBC, nstep), isNBC, "uniaxial_tension")


def cyclic_uniaxial(amplitude, cycles, nstep):
    """Uniaxial tension/compression cycles between +-amplitude in F_xx (boundary
    conditions of uniaxial_tension): each cycle climbs to +amplitude, falls to -amplitude
    and returns to zero in nstep / cycles equal increments."""
    isNBC = np.array([0, 0, 0, 1, 1, 0, 1, 1, 1], dtype=np.int32)
    per = nstep // cycles
    q = per // 4
    de = amplitude / q
    signs = np.concatenate([np.full(q, 1.0), np.full(2 * q, -1.0), np.full(per - 3 * q, 1.0)])
    incr = np.zeros((nstep, 9))
    incr[:, 0] = de * np.tile(signs, cycles)[:nstep]
    bc = np.cumsum(incr, axis=0)
    for d in (0, 4, 8):
        if not isNBC[d]:
            bc[:, d] += 1.0
    return Loading(bc, isNBC, "cyclic_uniaxial")


def plane_strain_compression(total_strain, nstep):
    """F_zz decreasing, F_yy = 1, F_xy = F_xz = F_yz = 0 prescribed; P_xx, P_yx, P_zx,
    P_zy held at zero."""
    isNBC = np.array([1, 0, 0, 1, 0, 0, 1, 1, 0], dtype=np.int32)
    incr = np.zeros(9)
    incr[8] = -total_strain / nstep
    return Loading(_accumulate(incr, isNBC, nstep), isNBC, "plane_strain_compression")


def uniaxial_strain(direction, total_strain, nstep):
    """Fully prescribed F = I + eps n (x) n (a random tensile direction cannot be
    written with the deck's per-component keywords, src/inlodcase.f)."""
    n = np.asarray(direction, dtype=np.float64)
    n = n / np.linalg.norm(n)
    isNBC = np.zeros(9, dtype=np.int32)
    incr = (total_strain / nstep) * np.outer(n, n).ravel()
    return Loading(_accumulate(incr, isNBC, nstep), isNBC, "uniaxial_strain")


def prescribed_stretch(diag_total, nstep):
    """Every F component prescribed: F = I + diag(diag_total) s / nstep at step s (the
    example deck's `strains F_xx .. F_yy .. F_zz ..` loading with zero shears)."""
    isNBC = np.zeros(9, dtype=np.int32)
    incr = np.zeros(9)
    incr[[0, 4, 8]] = np.asarray(diag_total, dtype=np.float64) / nstep
    return Loading(_accumulate(incr, isNBC, nstep), isNBC, "prescribed_stretch")
