"""Physics check of the whole step on the GPU: the Sedov-Taylor blast against the
self-similar solution, and energy conservation through the FP64 conservation totals.

The strong-shock radius of a point explosion of energy E in a uniform medium of density
rho is R(t) = xi0 (E t^2 / rho)^(1/5), xi0 = 1.1517 for gamma = 5/3 (Sedov 1959; the
reference compares its runs with the same solution, shamphys/src/SedovTaylor.cpp).  SPH
spreads the shock over a couple of smoothing lengths, so the radius of the density peak is
checked to 10 %."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_sedov_blast_radius_and_energy(precision):
    import shamrock_gb300 as sg
    from shamrock_gb300 import setups

    s = setups.sedov_taylor(20, jitter=0.0)
    ctx = sg.Context()
    model = sg.get_Model_SPH(context=ctx, vector_type="f64_3", sph_kernel="M4")
    cfg = model.gen_default_config()
    cfg.set_artif_viscosity_Constant(alpha_u=1.0, alpha_AV=1.0, beta_AV=2.0)
    cfg.set_boundary_periodic()
    cfg.set_eos_adiabatic(s["gamma"])
    cfg.set_particle_mass(s["pmass"])
    cfg.set_precision(precision)
    model.set_solver_config(cfg)
    model.resize_simulation_box(s["box_min"], s["box_max"])
    model.set_particles(s["pos"], s["vel"], s["h"], s["u"])
    model.set_cfl_cour(0.3)
    model.set_cfl_force(0.3)
    model.evolve_once()  # dt = 0: h, Omega, a, du and the first CFL step
    e0 = model.conservation_totals()["energy"]
    t_end, steps = 0.05, 0
    while model.time < t_end and steps < 20000:
        model.dt = min(model.dt, t_end - model.time)
        model.evolve_once()
        steps += 1
    assert model.time >= t_end - 1e-12
    tot = model.conservation_totals()
    d = model.collect_data()
    rho = s["pmass"] * (1.2 / d["hpart"]) ** 3
    r = np.linalg.norm(d["xyz"] - 0.5, axis=1)
    edges = np.linspace(0.0, 0.48, 49)
    idx = np.digitize(r, edges) - 1
    ok = (idx >= 0) & (idx < len(edges) - 1)
    mean = np.bincount(idx[ok], weights=rho[ok], minlength=len(edges) - 1) / np.maximum(
        np.bincount(idx[ok], minlength=len(edges) - 1), 1)
    r_peak = 0.5 * (edges[np.argmax(mean)] + edges[np.argmax(mean) + 1])
    r_th = 1.1517 * (1.0 * t_end**2 / 1.0) ** 0.2
    assert abs(r_peak - r_th) / r_th < 0.1, (r_peak, r_th, steps)
    # a compressed shell: 4 rho0 behind an ideal strong shock, about 1.8 rho0 once SPH
    # smooths it over ~2 h at this resolution (32,000 particles)
    assert mean.max() > 1.5
    assert abs(tot["energy"] - e0) / e0 < 1e-2, (tot["energy"], e0)
