"""The oracle's varying viscosity (Cullen & Dehnen 2010) on the Sedov blast (16,384
particles, alpha_AV starting at 0, t = 0.05): the switch is on at the shock and has
decayed in the hot gas behind it.

Ahead of the shock the ambient gas is cold (u = 1e-5, c_s ~ 3e-3): there the limiter
10 h^2 A / c_s^2 saturates at alpha_max on the smallest d(div v)/dt, and the decay time
h / (sigma c_s) is long, so alpha stays high; that follows from the update formula
(UpdateViscosity.cpp) and is not checked against anything here.  Measured: mean alpha
0.945 within 0.03 of the shock radius 0.347, 0.029 between 0.23 R and 0.6 R."""

import numpy as np

from oracle import oracle as O


def test_cd10_switch_on_sedov_blast():
    from shamrock_gb300 import setups
    from shamrock_gb300.sedov import SedovTaylor

    s = setups.sedov_taylor(16, jitter=0.0)
    n = len(s["h"])
    oc = O.OrcConfig(gamma=s["gamma"], pmass=s["pmass"], alpha_u=1.0, alpha_AV=0.0, beta_AV=2.0,
                     cfl_cour=0.3, cfl_force=0.3, cfl_mult_stiffness=2.0, htol_up_coarse=1.1,
                     htol_up_fine=1.1, epsilon_h=1e-6, h_iter_per_subcycles=50,
                     h_max_subcycles=100, tree_reduction_level=3, periodic=1, av_kind=1,
                     alpha_min=0.0, alpha_max=1.0, sigma_decay=0.1)
    oc.bmin[:] = [0.0, 0.0, 0.0]
    oc.bmax[:] = [1.0, 1.0, 1.0]
    sim = O.Sim(oc, s["pos"], s["vel"], s["h"], s["u"])
    sim.set_av(alpha=np.zeros(n), soundspeed=np.zeros(n))
    sim.evolve_once()  # dt = 0
    t_end = 0.05
    for _ in range(2000):
        t, dt, mult = sim.get_time()
        if t >= t_end - 1e-12:
            break
        sim.set_time(t, min(dt, t_end - t), mult)
        sim.evolve_once()
    assert sim.get_time()[0] >= t_end - 1e-12
    d, av = sim.get(), sim.get_av()
    alpha = av["alpha_AV"]
    assert np.all((alpha >= 0.0) & (alpha <= 1.0))
    R = SedovTaylor(gamma=s["gamma"], t=t_end).shock_radius
    r = np.linalg.norm(d["xyz"] - 0.5, axis=1)
    at_shock = np.abs(r - R) < 0.03
    behind = (r > 0.23 * R) & (r < 0.6 * R)
    assert at_shock.sum() > 100 and behind.sum() > 100
    assert alpha[at_shock].mean() > 0.85, alpha[at_shock].mean()
    assert alpha[behind].mean() < 0.15, alpha[behind].mean()
