"""The step's recovery paths, forced from the host by inputs and configuration, FP64
against the oracle (Solver.cpp:1080-1276 for the h sub-cycles, 2506-2616 for the
corrector loop).  Nothing here can fault or hang a GPU: every path is a host-side
decision on values the step already reads back.

- h restart: smoothing lengths set to half their converged size.  The Newton step
  wants h to grow by more than the sub-cycle limit (htol 1.1), eps = -1, and the
  sub-cycle restarts with a rebuilt tree and cache; identical sub-cycle and iteration
  counts, fields bit for bit.
- clustered random points (uniform half, Gaussian clump half, both as independent
  random points): near-coincident pairs take the restart path at 8,192 particles, and
  at 16,384 the iteration does not converge at all; with the sub-cycle count capped at
  2 the step runs 3 sub-cycles, carries on with the last h and reports it (the
  reference logs an error and continues), bit for bit with the oracle.
- corrector rerun: a dt seven times the CFL step fails the eps_v > 1e-2 test; the
  corrector reruns with the CFL multiplier halved, as many times as the oracle.
- corrector give-up: with the evaluation cap below what that dt needs, the step
  returns GBSPH_ERR_NOT_CONVERGED (the reference throws after 50 loops)."""

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

KEYS = ("n_ghost", "leaf_count", "cache_size", "h_subcycles", "h_iterations", "corrector_iters",
        "next_dt", "cfl_mult")


def _pair(s, h_max_subcycles=100, corrector_max_iters=50):
    import shamrock_gb300 as sg

    ctx = sg.Context()
    m = sg.get_Model_SPH(context=ctx, vector_type="f64_3", sph_kernel="M4")
    cfg = m.gen_default_config()
    cfg.set_artif_viscosity_Constant(alpha_u=1.0, alpha_AV=1.0, beta_AV=2.0)
    cfg.set_boundary_periodic()
    cfg.set_eos_adiabatic(s["gamma"])
    cfg.set_particle_mass(s["pmass"])
    cfg.set_precision("fp64")
    cfg.h_max_subcycles_count = h_max_subcycles
    cfg.corrector_max_iters = corrector_max_iters
    m.set_solver_config(cfg)
    m.resize_simulation_box(s["box_min"], s["box_max"])
    m.set_particles(s["pos"], s["vel"], s["h"], s["u"])
    m.set_cfl_cour(0.3)
    m.set_cfl_force(0.3)
    oc = O.OrcConfig(gamma=s["gamma"], pmass=s["pmass"], alpha_u=1.0, alpha_AV=1.0, beta_AV=2.0,
                     cfl_cour=0.3, cfl_force=0.3, cfl_mult_stiffness=2.0, htol_up_coarse=1.1,
                     htol_up_fine=1.1, epsilon_h=1e-6, h_iter_per_subcycles=50,
                     h_max_subcycles=h_max_subcycles, tree_reduction_level=3, periodic=1)
    oc.bmin[:] = list(s["box_min"])
    oc.bmax[:] = list(s["box_max"])
    return m, O.Sim(oc, s["pos"], s["vel"], s["h"], s["u"])


def _same(m, sim, lg, lo, what):
    for k in KEYS:
        assert lg[k] == lo[k], (what, k, lg[k], lo[k])
    g, o = m.collect_data(), sim.get()
    for k in ("xyz", "vxyz", "axyz", "hpart", "uint", "duint", "omega"):
        assert np.array_equal(g[k], o[k]), (what, k)


def test_h_restart_from_small_h():
    from shamrock_gb300 import setups

    s = setups.sedov_taylor(8, jitter=0.05, seed=3)
    s["h"] = 0.5 * s["h"]
    m, sim = _pair(s)
    for step in range(2):
        lg, lo = m.evolve_once(), sim.evolve_once()
        _same(m, sim, lg, lo, step)
        if step == 0:
            assert lg["h_subcycles"] > 1, lg  # the restart path ran


def test_clustered_random_points_restart():
    from shamrock_gb300 import setups

    s = setups.clustered_box(8192, seed=12345, sigma=0.05, literal=True)
    m, sim = _pair(s)
    subcycles = []
    for step in range(3):
        lg, lo = m.evolve_once(), sim.evolve_once()
        _same(m, sim, lg, lo, step)
        subcycles.append(lg["h_subcycles"])
    assert max(subcycles) > 1, subcycles


def test_h_subcycles_exhausted_carries_on():
    from shamrock_gb300 import setups

    s = setups.clustered_box(16384, seed=12345, sigma=0.05, literal=True)
    m, sim = _pair(s, h_max_subcycles=2)
    with pytest.warns(RuntimeWarning, match="not converged"):
        lg = m.evolve_once()
    lo = sim.evolve_once()
    assert lg["h_subcycles"] == 3 and lo["h_subcycles"] == 3, (lg, lo)
    assert "not converged" in lg["note"]
    _same(m, sim, lg, lo, "exhausted")


def _rerun_setup():
    from shamrock_gb300 import setups

    s = setups.sedov_taylor(6, jitter=0.05, seed=1)
    return s


def test_corrector_rerun_halves_cfl():
    s = _rerun_setup()
    m, sim = _pair(s)
    lg, lo = m.evolve_once(), sim.evolve_once()
    _same(m, sim, lg, lo, "dt=0 step")
    dt = 7.0 * lg["next_dt"]
    m.dt = dt
    t, _, cm = sim.get_time()
    sim.set_time(t, dt, cm)
    lg, lo = m.evolve_once(), sim.evolve_once()
    assert lg["corrector_iters"] >= 2, lg
    _same(m, sim, lg, lo, "rerun")
    assert abs(lg["eps_v"] - lo["eps_v"]) <= 1e-12 * abs(lo["eps_v"])


def test_corrector_gives_up():
    import shamrock_gb300 as sg

    s = _rerun_setup()
    m, sim = _pair(s, corrector_max_iters=1)
    m.evolve_once()
    sim.evolve_once()
    dt = 7.0 * m.logs[-1]["next_dt"]
    m.dt = dt
    t, _, cm = sim.get_time()
    sim.set_time(t, dt, cm)
    lo = sim.evolve_once()
    assert lo["corrector_iters"] > 1  # the oracle needed more evaluations than the cap
    with pytest.raises(sg.GbsphError, match="corrector has made over 1 loops"):
        m.evolve_once()
