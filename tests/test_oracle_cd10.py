"""CPU checks of the oracle's varying-viscosity (Cullen & Dehnen 2010) restatement.

The reference's tests hold no vectors for the velocity-gradient operators, so the
oracle is checked against properties those operators have by construction:
  - the linearly corrected gradient G(f) = R^-1 D(f) (DiffOperatorDtDivv.cpp) is exact
    for a linear field: with v = M x and a = 0 every particle gets d(div v)/dt =
    -tr(M M), whatever the particle arrangement (R is symmetric for radial kernels);
  - the SPH estimates div v and curl v (DiffOperator.cpp) of a linear field approach
    tr(M) and minus the curl of M x inside a uniform lattice;
  - the switch update (UpdateViscosity.cpp) follows its closed form particle by particle.
"""

import numpy as np
import pytest

from oracle import oracle as O


def _cfg(pmass, bmin, bmax, periodic):
    oc = O.OrcConfig(gamma=5.0 / 3.0, pmass=pmass, alpha_u=1.0, alpha_AV=0.0, beta_AV=2.0,
                     cfl_cour=0.3, cfl_force=0.3, cfl_mult_stiffness=2.0, htol_up_coarse=1.1,
                     htol_up_fine=1.1, epsilon_h=1e-6, h_iter_per_subcycles=50,
                     h_max_subcycles=100, tree_reduction_level=3, periodic=periodic,
                     av_kind=1, alpha_min=0.0, alpha_max=1.0, sigma_decay=0.1)
    oc.bmin[:] = list(bmin)
    oc.bmax[:] = list(bmax)
    return oc


def _lattice(n_side, jitter, seed):
    rng = np.random.default_rng(seed)
    g = (np.arange(n_side) + 0.5) / n_side
    pos = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    pos = pos + jitter / n_side * rng.uniform(-0.5, 0.5, pos.shape)
    h = np.full(len(pos), 1.2 / n_side)
    return pos, h


@pytest.mark.parametrize("jitter", [0.0, 0.3])
def test_dtdivv_exact_for_linear_velocity(jitter):
    """Free boundary, v = M x, a = 0: d(div v)/dt = -tr(M^2) at every particle."""
    pos, h = _lattice(10, jitter, 3)
    n = len(h)
    rng = np.random.default_rng(7)
    M = 0.1 * rng.standard_normal((3, 3))
    vel = pos @ M.T
    u = np.full(n, 1.0)
    sim = O.Sim(_cfg(1.0 / n, pos.min(0) - 0.01, pos.max(0) + 0.01, 0), pos, vel, h, u)
    sim.evolve_once()  # dt = 0: positions stay, derivatives were zero
    av = sim.get_av()
    expect = -np.trace(M @ M)
    err = np.abs(av["dtdivv"] - expect) / abs(expect)
    assert err.max() < 1e-9, err.max()


def test_sph_divv_curlv_of_linear_field_in_periodic_lattice():
    """Uniform periodic lattice, v = M x: the SPH estimates of div v and curl v at interior particles are close to tr(M) and
    to minus the curl of M x: the reference's curl operator sums -1/(Omega rho) m v_ab x
    grad W (DiffOperator.cpp:236-240), the opposite sign of the usual estimate, which the
    switch does not see (it uses |curl v|^2)."""
    pos, h = _lattice(12, 0.0, 1)
    n = len(h)
    M = np.array([[0.02, -0.05, 0.01], [0.05, 0.03, -0.02], [-0.01, 0.02, 0.01]])
    # interior particles only see neighbours inside the box, so periodic wrap is harmless
    # for a check restricted to them
    vel = pos @ M.T
    sim = O.Sim(_cfg(1.0 / n, (0, 0, 0), (1, 1, 1), 1), pos, vel, h, np.ones(n))
    sim.evolve_once()
    av = sim.get_av()
    inner = np.all((pos > 0.25) & (pos < 0.75), axis=1)
    curl = np.array([M[2, 1] - M[1, 2], M[0, 2] - M[2, 0], M[1, 0] - M[0, 1]])
    assert np.allclose(av["divv"][inner], np.trace(M), rtol=2e-2, atol=1e-4)
    assert np.allclose(av["curlv"][inner], -curl[None, :], rtol=2e-2, atol=1e-4)


def test_cd10_update_closed_form():
    """The switch update against its closed form, from the quantities the oracle
    returns (alpha before = 0.2, stored sound speed 0.7, dt of the second step)."""
    pos, h = _lattice(8, 0.2, 5)
    n = len(h)
    rng = np.random.default_rng(11)
    vel = 0.05 * rng.standard_normal((n, 3))
    sim = O.Sim(_cfg(1.0 / n, (0, 0, 0), (1, 1, 1), 1), pos, vel, h, np.full(n, 1.0))
    sim.set_av(alpha=np.full(n, 0.2), soundspeed=np.full(n, 0.7))
    sim.evolve_once()  # dt = 0 step
    before = sim.get_av()
    h_b = sim.get()["hpart"]
    _, dt, _ = sim.get_time()
    sim.evolve_once()
    av = sim.get_av()
    cs = before["soundspeed"]
    hh = sim.get()["hpart"]  # h of the second step (the update uses the current h)
    fact = dt * cs * 0.1 / hh
    fac = np.maximum(-av["divv"], 0) ** 2
    tr = np.sum(av["curlv"] ** 2, axis=1)
    bal = np.where(fac + tr > np.finfo(float).eps, fac / np.where(fac + tr > 0, fac + tr, 1), 1.0)
    A = bal * np.maximum(-av["dtdivv"], 0)
    loc = np.minimum(10 * hh * hh * A / cs ** 2, 1.0)
    new = (before["alpha_AV"] + loc * fact) / (1 + fact)
    new = np.where(loc > before["alpha_AV"], loc, new)
    assert dt > 0 and np.all(np.isfinite(h_b))
    assert np.allclose(av["alpha_AV"], new, rtol=1e-12, atol=1e-15)


def test_mm97_update_closed_form():
    """The Morris & Monaghan (1997) update against its closed form."""
    pos, h = _lattice(8, 0.2, 9)
    n = len(h)
    rng = np.random.default_rng(13)
    vel = 0.05 * rng.standard_normal((n, 3))
    cfg = _cfg(1.0 / n, (0, 0, 0), (1, 1, 1), 1)
    cfg.av_kind = 2
    sim = O.Sim(cfg, pos, vel, h, np.full(n, 1.0))
    sim.set_av(alpha=np.full(n, 0.2), soundspeed=np.full(n, 0.7))
    sim.evolve_once()
    before = sim.get_av()
    _, dt, _ = sim.get_time()
    sim.evolve_once()
    av = sim.get_av()
    hh = sim.get()["hpart"]
    fact = dt * before["soundspeed"] * 0.1 / hh
    new = (before["alpha_AV"] + np.maximum(-av["divv"], 0) * dt + fact * 0.0) / (1 + fact)
    assert dt > 0
    assert np.allclose(av["alpha_AV"], np.minimum(new, 1.0), rtol=1e-12, atol=1e-15)
