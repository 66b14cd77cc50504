"""The FP64 oracle's step on a travelling sound wave (the sound-wave configuration's
set-up, shamrock_gb300.setups.sound_wave, without noise): the wave moves in +x at about
the sound speed, and the error of the measured speed shrinks with resolution.

Measured phase speeds after a quarter period (cs = 1): 1.044 at 16 particles per
wavelength, 1.033 at 24, 1.029 at 32 (SPH with the M4 kernel, hfact 1.2, on a simple
cubic lattice).  The check guards the pressure force and the time integration against
gross errors (a wrong factor in the force changes the speed by tens of per cent) and
the set-up against a flipped direction."""

import numpy as np
import pytest

from oracle import oracle as O


def _phase_speed(n_side, t_end=0.25):
    from shamrock_gb300 import setups

    s = setups.sound_wave(n_side, amp=1e-4, noise=0.0)
    oc = O.OrcConfig(gamma=s["gamma"], pmass=s["pmass"], alpha_u=1.0, alpha_AV=0.1, beta_AV=2.0,
                     cfl_cour=0.3, cfl_force=0.3, cfl_mult_stiffness=2.0, htol_up_coarse=1.1,
                     htol_up_fine=1.1, epsilon_h=1e-6, h_iter_per_subcycles=50,
                     h_max_subcycles=100, tree_reduction_level=3, periodic=1)
    oc.bmin[:] = [0.0, 0.0, 0.0]
    oc.bmax[:] = [1.0, 1.0, 1.0]
    sim = O.Sim(oc, s["pos"], s["vel"], s["h"], s["u"])
    sim.evolve_once()  # dt = 0
    for _ in range(1000):
        t, dt, mult = sim.get_time()
        if t >= t_end - 1e-12:
            break
        sim.set_time(t, min(dt, t_end - t), mult)
        sim.evolve_once()
    d = sim.get()
    x, v = d["xyz"][:, 0], d["vxyz"][:, 0]
    # v = A sin(2 pi (x - c t)): projections on sin and cos give the phase 2 pi c t
    a_s = 2 * np.mean(v * np.sin(2 * np.pi * x))
    a_c = 2 * np.mean(v * np.cos(2 * np.pi * x))
    c = np.arctan2(-a_c, a_s) / (2 * np.pi * t_end)
    return c, np.hypot(a_s, a_c) / 1e-4, np.abs(d["vxyz"][:, 1:]).max() / 1e-4


def test_sound_wave_speed():
    c16, amp16, trans16 = _phase_speed(16)
    assert c16 == pytest.approx(1.0, rel=0.06), c16
    assert amp16 == pytest.approx(1.0, rel=0.1), amp16
    assert trans16 < 1e-4  # the plane wave stays plane
    c24, _, _ = _phase_speed(24)
    assert abs(c24 - 1.0) < abs(c16 - 1.0), (c16, c24)
