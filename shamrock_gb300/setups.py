"""Seeded synthetic particle sets for the SPH hot path.

These stand in for the reference's setup generators and benchmark inputs (no
dataset is involved): every generator is deterministic given its seed.

- ``sedov_taylor``: FCC lattice of 4*n^3 equal-mass particles in the periodic
  unit cube, rho = 1, u = 1e-5, total energy E added uniformly to the internal
  energy of the particles within r < r_inj * a of the centre (a = 1/n), optional
  Gaussian position jitter sigma * a.
- ``clustered_box``: half the particles uniform in the unit cube, half in a
  Gaussian clump, both sampled from jittered lattices (the clump by radial stretch
  mapping), v ~ N(0, 0.1^2), u ~ U[0.5, 1.5].
- ``sound_wave``: simple cubic lattice of 64^3 = 2^18 particles filling the periodic
  unit cube, with a 1e-4 sin(2 pi x) density perturbation applied by a position
  remap and the matching travelling-wave velocity (an FCC lattice cannot hold exactly 2^18 sites in a cube: 4*40^3 < 2^18, and
  trimming 4*41^3 leaves a void slab whose collapse swamps the wave).

h is initialised to hfact * (m / rho)^(1/3) with the local density estimate of
the generator (hfact = 1.2 for M4).
"""

import numpy as np

HFACT_M4 = 1.2


def fcc_lattice(n, box_min=(0.0, 0.0, 0.0), box_max=(1.0, 1.0, 1.0)):
    """4*n^3 positions of a cubic FCC lattice filling the box, in i-j-k-basis order.

    Lattice sites sit at ((i, j, k) + basis + 1/4) * a so that no particle lies on a
    box face."""
    bmin = np.asarray(box_min, float)
    a = (np.asarray(box_max, float) - bmin) / n
    basis = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]]) + 0.25
    idx = np.stack(np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij"), -1)
    idx = idx.reshape(-1, 1, 3).astype(float)
    pos = (idx + basis[None, :, :]).reshape(-1, 3) * a + bmin
    return pos


def sedov_taylor(n_cells, jitter=0.0, seed=1, E=1.0, u0=1e-5, r_inj=2.0, gamma=5.0 / 3.0):
    pos = fcc_lattice(n_cells)
    N = pos.shape[0]
    a = 1.0 / n_cells
    if jitter > 0:
        rng = np.random.default_rng(seed)
        pos = pos + rng.normal(0.0, jitter * a, size=pos.shape)
        pos = np.mod(pos, 1.0)
    pmass = 1.0 / N
    u = np.full(N, u0)
    r = np.linalg.norm(pos - 0.5, axis=1)
    inj = r < r_inj * a
    n_inj = int(inj.sum())
    if n_inj:
        u[inj] += E / (pmass * n_inj)
    h = np.full(N, HFACT_M4 * (pmass / 1.0) ** (1.0 / 3.0))
    return dict(pos=pos, vel=np.zeros((N, 3)), h=h, u=u, pmass=pmass, gamma=gamma,
                box_min=(0.0, 0.0, 0.0), box_max=(1.0, 1.0, 1.0), periodic=True,
                n_inject=n_inj)


def _chi3_radius_table(n=4096, rmax=8.0):
    """Radius of a 3-D standard normal vector against its cumulative probability
    P(r) = erf(r / sqrt 2) - sqrt(2 / pi) r exp(-r^2 / 2), tabulated for inversion."""
    from math import erf

    r = np.linspace(0.0, rmax, n)
    P = np.array([erf(x / np.sqrt(2.0)) for x in r]) - np.sqrt(2.0 / np.pi) * r * np.exp(-0.5 * r * r)
    return P, r


def _jittered_lattice(n_side, rng, jitter):
    g = (np.arange(n_side) + 0.5) / n_side
    i, j, k = np.meshgrid(g, g, g, indexing="ij")
    pos = np.stack([i.ravel(), j.ravel(), k.ravel()], 1)
    return pos + (jitter / n_side) * rng.standard_normal(pos.shape)


def clustered_box(N, seed=12345, sigma=0.05, gamma=5.0 / 3.0, jitter=0.1, literal=False):
    """Half the particles uniform in the unit cube, half in a Gaussian clump of width sigma
    at the centre; v ~ N(0, 0.1^2) per component, u ~ U[0.5, 1.5].

    Both halves are sampled from jittered cubic lattices (jitter 0.1 of the spacing),
    not as independent random points: the uniform half is a lattice over the cube with
    sites removed at random down to N/2; the clump is a lattice ball mapped radially so
    that its mass profile is the Gaussian's (stretch mapping).  Independent random
    points put some pairs far closer than the mean spacing; for such a particle the
    density sum is dominated by close pairs, Omega < 0, and the h-rho Newton step of
    IterateSmoothingLengthDensity moves h away from the root every iteration (h then
    grows by the sub-cycle limit until it spans the box).  Lattice sampling keeps the
    same density field without near-coincident pairs.

    literal: both halves as independent random points instead (uniform in the cube; the
    clump N(0.5, sigma^2) per coordinate, clipped into the box), the configuration as
    stated, which exercises the h iteration's non-convergence and restart path."""
    rng = np.random.default_rng(seed)
    n1 = N // 2
    n2 = N - n1
    if literal:
        p1 = rng.uniform(0.0, 1.0, size=(n1, 3))
        p2 = np.clip(rng.normal(0.5, sigma, size=(n2, 3)), 1e-9, 1.0 - 1e-9)
        return _clustered_fields(np.concatenate([p1, p2]), rng, N, sigma, gamma)
    # uniform half: smallest cubic lattice with >= n1 sites, random sites removed
    ns = int(np.ceil(n1 ** (1.0 / 3.0)))
    p1 = _jittered_lattice(ns, rng, jitter)
    p1 = np.mod(p1[rng.permutation(len(p1))[:n1]], 1.0)
    # clump: lattice ball of radius 1 with n2 sites (closest to the centre), stretched
    nb = int(np.ceil((n2 * 6.0 / np.pi) ** (1.0 / 3.0))) + 2
    q = _jittered_lattice(nb, rng, jitter) * 2.0 - 1.0
    rq = np.linalg.norm(q, axis=1)
    keep = np.argsort(rq, kind="stable")[:n2]
    q, rq = q[keep], rq[keep]
    u_frac = (rq / rq.max()) ** 3 * (1.0 - 1e-9)  # uniform ball: mass fraction r^3
    P, rt = _chi3_radius_table()
    r_new = sigma * np.interp(u_frac, P, rt)
    dirs = q / np.maximum(rq, 1e-300)[:, None]
    p2 = np.clip(0.5 + dirs * r_new[:, None], 1e-9, 1.0 - 1e-9)
    return _clustered_fields(np.concatenate([p1, p2]), rng, N, sigma, gamma)


def _clustered_fields(pos, rng, N, sigma, gamma):
    vel = rng.normal(0.0, 0.1, size=(N, 3))
    u = rng.uniform(0.5, 1.5, size=N)
    pmass = 1.0 / N
    # local density estimate of the two populations
    rho_uniform = 0.5
    r = pos - 0.5
    rho_clump = 0.5 * np.exp(-0.5 * np.sum(r * r, 1) / sigma**2) / ((2 * np.pi) ** 1.5 * sigma**3)
    rho = np.maximum(rho_uniform + rho_clump, 1e-3)
    h = HFACT_M4 * (pmass / rho) ** (1.0 / 3.0)
    return dict(pos=pos, vel=vel, h=h, u=u, pmass=pmass, gamma=gamma,
                box_min=(0.0, 0.0, 0.0), box_max=(1.0, 1.0, 1.0), periodic=True)


def sound_wave(n_side=64, amp=1e-4, gamma=1.0001, cs=1.0, travelling=True, noise=1e-4,
               seed=12345):
    """n_side^3 particles on a simple cubic lattice (sites at (i + 1/2) / n_side), then
    rho = 1 + amp sin(2 pi x) by the first-order remap x -> x + amp/(2 pi) cos(2 pi x)
    (the displacement's derivative is -amp sin(2 pi x), so the spacing shrinks where
    sin > 0);
    P = cs^2 / gamma at rho = 1 (u = P / ((gamma - 1) rho)).  travelling: the acoustic
    wave's own velocity v_x = amp cs sin(2 pi x) (a wave moving in +x); else at rest.
    noise: seeded perturbations, velocity N(0, (noise cs)^2) per component and u relative
    N(0, noise^2).  They break the lattice's exact plane symmetry, which otherwise keeps
    pairs of one plane exactly at zero relative velocity and zero pressure difference:
    on the viscosity switch max(-rho v_sig w / 2, 0) and the |P_a - P_b|^(1/2)
    conductivity speed, where the step has no derivative."""
    g = (np.arange(n_side) + 0.5) / n_side
    i, j, k = np.meshgrid(g, g, g, indexing="ij")
    pos = np.stack([i.ravel(), j.ravel(), k.ravel()], 1)
    N = pos.shape[0]
    x = pos[:, 0]
    pos[:, 0] = np.mod(x + amp / (2 * np.pi) * np.cos(2 * np.pi * x), 1.0)
    pmass = 1.0 / N
    rho = 1.0 + amp * np.sin(2 * np.pi * pos[:, 0])
    P0 = cs * cs / gamma
    u = np.full(N, P0 / ((gamma - 1.0) * 1.0))
    h = HFACT_M4 * (pmass / rho) ** (1.0 / 3.0)
    vel = np.zeros((N, 3))
    if travelling:
        vel[:, 0] = amp * cs * np.sin(2 * np.pi * pos[:, 0])
    if noise:
        rng = np.random.default_rng(seed)
        vel += noise * cs * rng.standard_normal((N, 3))
        u = u * (1.0 + noise * rng.standard_normal(N))
    return dict(pos=pos, vel=vel, h=h, u=u, pmass=pmass, gamma=gamma,
                box_min=(0.0, 0.0, 0.0), box_max=(1.0, 1.0, 1.0), periodic=True)

def keplerian_disc(N, seed=12345, r_in=0.1, r_out=1.0, HoR=0.05, q=0.25, M=1.0, G=1.0,
                   disc_mass=1e-3, jitter=0.1):
    """Gas disc around a central point mass M at the origin: cylindrical radius r in
    [r_in, r_out] with surface density Sigma ~ 1/r, locally isothermal sound speed
    c_s = cs0 r^-q (r in units of r0 = 1) with cs0 = HoR so that H/R = HoR at r = 1,
    vertical Gaussian of height H = c_s / Omega_K, Keplerian azimuthal velocity.

    Sampling: a jittered lattice in (u_r, u_phi, u_z) in [0, 1]^3 mapped by the inverse
    cumulative distributions (r uniform for Sigma ~ 1/r, phi uniform, z = H Phi^-1(u_z)),
    with lattice counts that make the spacing nearly isotropic at mid radius, so no pair
    starts much closer than the local spacing (see clustered_box)."""
    from scipy.special import ndtri

    rng = np.random.default_rng(seed)
    cs0 = HoR
    rm = 0.5 * (r_in + r_out)
    Hm = cs0 * rm ** (1.5 - q)
    dr_span, dphi_span, dz_span = r_out - r_in, 2 * np.pi * rm, 5.0 * Hm
    # n_r : n_phi : n_z in proportion to the spans, product >= N
    scale = (N / (dr_span * dphi_span * dz_span)) ** (1.0 / 3.0)
    n1 = max(2, int(np.ceil(dr_span * scale)))
    n2 = max(4, int(np.ceil(dphi_span * scale)))
    n3 = max(2, int(np.ceil(dz_span * scale)))
    while n1 * n2 * n3 < N:
        n3 += 1
    g1, g2, g3 = ((np.arange(k) + 0.5) / k for k in (n1, n2, n3))
    a, b, c = np.meshgrid(g1, g2, g3, indexing="ij")
    u = np.stack([a.ravel(), b.ravel(), c.ravel()], 1)
    u += (jitter / np.array([n1, n2, n3])) * rng.standard_normal(u.shape)
    u = u[rng.permutation(len(u))[:N]]
    u[:, 0] = np.clip(u[:, 0], 0.0, 1.0)
    u[:, 1] = np.mod(u[:, 1], 1.0)
    u[:, 2] = np.clip(u[:, 2], 1e-4, 1.0 - 1e-4)
    r = r_in + u[:, 0] * dr_span
    phi = 2 * np.pi * u[:, 1]
    cs_r = cs0 * r ** (-q)
    H = cs_r / np.sqrt(G * M / r**3)
    z = H * ndtri(u[:, 2])
    pos = np.stack([r * np.cos(phi), r * np.sin(phi), z], 1)
    vk = np.sqrt(G * M / r)
    vel = np.stack([-vk * np.sin(phi), vk * np.cos(phi), np.zeros(N)], 1)
    pmass = disc_mass / N
    sigma = disc_mass / (2 * np.pi * dr_span * r)
    rho = sigma * np.exp(-0.5 * (z / H) ** 2) / (np.sqrt(2 * np.pi) * H)
    h = HFACT_M4 * (pmass / rho) ** (1.0 / 3.0)
    Rsph = np.linalg.norm(pos, axis=1)
    u_int = 1.5 * (cs0 * Rsph ** (-q)) ** 2
    return dict(pos=pos, vel=vel, h=h, u=u_int, pmass=pmass, gamma=5.0 / 3.0, cs0=cs0, q=q,
                r0=1.0, M=M, G=G, periodic=False,
                box_min=tuple(pos.min(0) - 1e-3), box_max=tuple(pos.max(0) + 1e-3))


def _hcp_index_bounds(dr, bmin, bmax):
    """Integer lattice bounds of LatticeHCP::get_box_index_bounds (shammath/crystalLattice.hpp:
    145-170): coordinates divided by the lattice steps, truncated toward zero, widened by 1."""
    steps = np.array([2.0, np.sqrt(3.0), 2 * np.sqrt(6.0) / 3])
    cmin = (np.asarray(bmin, float) / steps) / dr
    cmax = (np.asarray(bmax, float) / steps) / dr
    return np.trunc(cmin).astype(np.int64) - 1, np.trunc(cmax).astype(np.int64) + 1


def _hcp_points(dr, i, j, k):
    """LatticeHCP::generator (crystalLattice.hpp:68-79)."""
    return dr * np.stack([2 * i + (np.abs(j + k) % 2),
                          np.sqrt(3.0) * (j + (1.0 / 3.0) * (np.abs(k) % 2)),
                          2 * np.sqrt(6.0) * k / 3], 1)


def homogeneous_box(n_target=1 << 25, bmin=(-0.6, -0.6, -0.6), bmax=(0.6, 0.6, 0.6), rho=1.0,
                    u_inj=1.0):
    """The reference's SPH throughput benchmark (examples/benchmarks/sph_homogeneous_benchmark.py):
    an HCP lattice of about n_target particles filling the periodic box that the lattice
    closes exactly (LatticeHCP::get_ideal_hcp_box), density rho, u = 0 except a central
    injection u_inj W(r, 16 dr) (Model::add_kernel_value), h = dr as the lattice generator
    sets it.  With n_target = 2^25 this gives 33,848,064 particles, the count of the
    reference's published single-GPU runs."""
    bmin = np.asarray(bmin, float)
    bmax = np.asarray(bmax, float)
    vol = float(np.prod(bmax - bmin))
    dr = (0.74 * (vol / n_target) / ((4.0 / 3.0) * 3.1416)) ** (1.0 / 3.0)
    # ideal periodic box (crystalLattice.hpp:172-202, 387-401)
    cmin, cmax = _hcp_index_bounds(dr, bmin, bmax)
    if cmax[0] - cmin[0] < 2:
        cmax[0] += 1
    if (cmax[1] + cmin[1]) % 2 != 0:
        cmax[1] += 1
    if (cmax[2] + cmin[2]) % 2 != 0:
        cmax[2] += 1
    lo = np.array([2.0 * cmin[0], np.sqrt(3.0) * cmin[1], 2 * np.sqrt(6.0) * cmin[2] / 3]) * dr
    hi = np.array([2.0 * cmax[0], np.sqrt(3.0) * cmax[1], 2 * np.sqrt(6.0) * cmax[2] / 3]) * dr
    # lattice sites inside [lo, hi) (GeneratorLatticeHCP.hpp:51-110, Patch.hpp:209-214)
    gmin, gmax = _hcp_index_bounds(dr, lo, hi)
    parts = []
    ii = np.arange(gmin[0], gmax[0])
    jj = np.arange(gmin[1], gmax[1])
    for k in range(gmin[2], gmax[2]):
        i, j = np.meshgrid(ii, jj, indexing="ij")
        i, j = i.ravel(), j.ravel()
        p = _hcp_points(dr, i, j, np.full_like(i, k))
        keep = np.all((p >= lo) & (p < hi), axis=1)
        parts.append(p[keep])
    pos = np.concatenate(parts)
    n = len(pos)
    pmass = rho * float(np.prod(hi - lo)) / n
    r = np.linalg.norm(pos, axis=1)
    h_inj = 16 * dr
    q = r / h_inj
    f = np.where(q < 1, 0.25 * (2 - q) ** 3 - (1 - q) ** 3, np.where(q < 2, 0.25 * (2 - q) ** 3, 0.0))
    u = u_inj * f / (np.pi * h_inj ** 3)
    return dict(pos=pos, vel=np.zeros_like(pos), h=np.full(n, dr), u=u, pmass=pmass,
                gamma=5.0 / 3.0, box_min=tuple(lo), box_max=tuple(hi), dr=dr)
