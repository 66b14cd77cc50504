"""The FP64 oracle's whole step against physics: the Sedov-Taylor blast (32,000
particles, t = 0.05) checked against the closed-form similarity solution
(shamrock_gb300.sedov, pinned to the reference's tabulated solution).

The reference's unit tests hold no vectors for the derivatives, the EOS, the CFL step
or the leapfrog; this check pins their composition physically.  The GPU FP64 path is
bit-identical to the oracle, so the same numbers hold for it (tests/test_gpu_sedov_physics.py
repeats the check on the GPU in both precisions)."""

import numpy as np
import pytest

from oracle import oracle as O


def test_oracle_sedov_blast():
    from shamrock_gb300 import setups
    from shamrock_gb300.sedov import SedovTaylor

    s = setups.sedov_taylor(20, jitter=0.0)
    oc = O.OrcConfig(gamma=s["gamma"], pmass=s["pmass"], alpha_u=1.0, alpha_AV=1.0, beta_AV=2.0,
                     cfl_cour=0.3, cfl_force=0.3, cfl_mult_stiffness=2.0, htol_up_coarse=1.1,
                     htol_up_fine=1.1, epsilon_h=1e-6, h_iter_per_subcycles=50,
                     h_max_subcycles=100, tree_reduction_level=3, periodic=1)
    oc.bmin[:] = [0.0, 0.0, 0.0]
    oc.bmax[:] = [1.0, 1.0, 1.0]
    sim = O.Sim(oc, s["pos"], s["vel"], s["h"], s["u"])
    pm = s["pmass"]

    def energy(d):
        return float(np.sum(pm * (0.5 * np.sum(d["vxyz"] ** 2, axis=1) + d["uint"])))

    sim.evolve_once()  # dt = 0
    e0 = energy(sim.get())
    t_end, steps = 0.05, 0
    while steps < 2000:
        t, dt, mult = sim.get_time()
        if t >= t_end - 1e-12:
            break
        sim.set_time(t, min(dt, t_end - t), mult)
        sim.evolve_once()
        steps += 1
    d = sim.get()
    assert sim.get_time()[0] >= t_end - 1e-12
    # total energy (leapfrog with the corrector): conserved to 2e-4 over the run
    assert abs(energy(d) - e0) / e0 < 2e-4, (energy(d), e0, steps)

    sol = SedovTaylor(gamma=s["gamma"], t=t_end, e_blast=1.0, rho0=1.0)
    r = np.linalg.norm(d["xyz"] - 0.5, axis=1)
    rhat = (d["xyz"] - 0.5) / np.maximum(r, 1e-300)[:, None]
    vr = np.sum(d["vxyz"] * rhat, axis=1)
    rho = pm * (1.2 / d["hpart"]) ** 3
    edges = np.linspace(0.0, 0.48, 49)
    idx = np.digitize(r, edges) - 1
    ok = (idx >= 0) & (idx < len(edges) - 1)
    cnt = np.maximum(np.bincount(idx[ok], minlength=len(edges) - 1), 1)

    def binned(x):
        return np.bincount(idx[ok], weights=x[ok], minlength=len(edges) - 1) / cnt

    mid = 0.5 * (edges[1:] + edges[:-1])
    rho_b, v_b, v_th = binned(rho), binned(vr), binned(sol.profile(r)[1])
    R = sol.shock_radius
    assert abs(mid[np.argmax(rho_b)] - R) / R < 0.1
    assert abs(mid[np.argmax(v_b)] - R) / R < 0.1
    assert v_b.max() == pytest.approx(v_th.max(), rel=0.1)
    # ahead of the shock the gas is still at rest and at the ambient density
    far = mid > 1.3 * R
    assert np.all(np.abs(v_b[far]) < 0.05 * sol.u_s)
    assert np.all(np.abs(rho_b[far] - 1.0) < 0.05)
    rg = np.linspace(0.0, R * (1 - 1e-12), 20001)
    rho_a, v_a, _ = sol.profile(rg)
    p_th = float(np.trapezoid(rho_a * v_a * 4 * np.pi * rg * rg, rg))
    assert float(np.sum(pm * vr)) == pytest.approx(p_th, rel=0.1)
