"""Adjoint of the step with a varying viscosity (the Cullen & Dehnen 2010 switch the
reference's own benchmark runs, UpdateViscosity.cpp:122-215, and the Morris & Monaghan
1997 one, :53-118): the reverse of the velocity gradients (div v, curl v and the
corrected d(div v)/dt, DiffOperator*.cpp), of the switch and of the per-particle alpha in
the derivatives, with alpha_AV and the stored sound speed carried as state.

A small periodic box (a jittered 4*6^3 lattice with random velocities, so that the gas
compresses and the switch fires, alpha_max low enough that some particles reach it),
4 steps with a checkpoint every 2, loss = |v_final - v_target|^2.  Gradients with
respect to initial velocities, energies and the switch's alpha_min / alpha_max: the
FP64 adjoint against FP64 central differences (Richardson-combined steps eps and 2 eps),
within 1e-4 of the largest checked gradient of each kind; the FP32-mixed adjoint against
the FP64 one."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _set_up():
    from shamrock_gb300 import setups

    s = setups.sedov_taylor(6, jitter=0.1, seed=5, E=0.1)
    rng = np.random.default_rng(5)
    n = len(s["h"])
    s["vel"] = rng.normal(0.0, 0.3, size=(n, 3))
    s["u"] = s["u"] + rng.uniform(0.5, 1.5, size=n)
    return s


def _model(s, kind, precision, amin, amax):
    import shamrock_gb300 as sg

    m = sg.get_Model_SPH(context=sg.Context(), vector_type="f64_3", sph_kernel="M4")
    cfg = m.gen_default_config()
    if kind == "cd10":
        cfg.set_artif_viscosity_VaryingCD10(alpha_min=amin, alpha_max=amax, sigma_decay=0.1,
                                            alpha_u=1.0, beta_AV=2.0)
    else:
        cfg.set_artif_viscosity_VaryingMM97(alpha_min=amin, alpha_max=amax, sigma_decay=0.1,
                                            alpha_u=1.0, beta_AV=2.0)
    cfg.set_boundary_periodic()
    cfg.set_eos_adiabatic(s["gamma"])
    cfg.set_particle_mass(s["pmass"])
    cfg.set_precision(precision)
    if precision == "fp64":
        cfg.set_epsilon_h(1e-13)
        cfg.set_epsilon_h_particle(1e-13)
    m.set_solver_config(cfg)
    m.resize_simulation_box(s["box_min"], s["box_max"])
    m.set_particles(s["pos"], s["vel"], s["h"], s["u"])
    m.set_cfl_cour(0.3)
    m.set_cfl_force(0.3)
    m.evolve_once()  # dt = 0: h, Omega, a, du, the first alpha and sound speed
    return m


@pytest.mark.parametrize("kind", ["cd10", "mm97"])
def test_varying_av_adjoint_fd(kind):
    import torch

    from shamrock_gb300 import adjoint
    from shamrock_gb300.adjoint import _restore, _snapshot

    s = _set_up()
    amin, amax = (0.05, 0.5)
    steps, ck = 4, 2
    n = len(s["h"])
    rng = np.random.default_rng(11)
    v_t_np = 0.3 * rng.standard_normal((3, n))
    out = {}
    for prec in ("fp64", "mixed"):
        m = _model(s, kind, prec, amin, amax)
        warm, ts = _snapshot(m), (m.time, m.dt, m.cfl_mult)
        v_t = torch.as_tensor(v_t_np, device=warm["vxyz"].device)
        v0 = warm["vxyz"].clone().requires_grad_(True)
        u0 = warm["uint"].clone().requires_grad_(True)
        al = torch.tensor([amin, amax], dtype=torch.float64, requires_grad=True)
        dts = out["dts"] if "dts" in out else None
        x, v, u = adjoint.rollout(m, v0, u0, al, steps, ck, dts=dts)
        ((v - v_t) ** 2).sum().backward()
        out[prec] = dict(v=v0.grad.cpu().numpy(), u=u0.grad.cpu().numpy(),
                         a=al.grad.cpu().numpy())
        if prec == "fp64":
            out["dts"] = list(adjoint.rollout.last_dts)
            m64, warm64, ts64 = m, warm, ts
            alpha_state = m._to_device()["alpha_AV"].cpu().numpy()
    assert alpha_state.max() > 0, "the switch never fired"

    def loss(kind_, idx, d):
        _restore(m64, warm64)
        m64.time, m64.dt, m64.cfl_mult = ts64
        vv, uu = warm64["vxyz"].clone(), warm64["uint"].clone()
        aa = [amin, amax]
        if kind_ == "v":
            vv[idx] += d
        elif kind_ == "u":
            uu[idx] += d
        else:
            aa[idx[0]] += d
        v_t = torch.as_tensor(v_t_np, device=vv.device)
        with torch.no_grad():
            x, v, u = adjoint.rollout(m64, vv, uu, torch.tensor(aa, dtype=torch.float64), steps,
                                      ck, dts=out["dts"])
            return float(((v - v_t) ** 2).sum())

    coords = [("v", (int(rng.integers(3)), int(rng.integers(n)))) for _ in range(6)]
    coords += [("u", (int(rng.integers(n)),)) for _ in range(4)]
    coords += [("a", (0,)), ("a", (1,))]
    res = []
    for kind_, idx in coords:
        eps = 1e-6 * float(warm64["uint"][idx[0]]) if kind_ == "u" else 1e-6
        d1 = (loss(kind_, idx, eps) - loss(kind_, idx, -eps)) / (2 * eps)
        d2 = (loss(kind_, idx, 2 * eps) - loss(kind_, idx, -2 * eps)) / (4 * eps)
        fd = (4 * d1 - d2) / 3
        g64 = float(out["fp64"][kind_][idx])
        g32 = float(out["mixed"][kind_][idx])
        res.append((kind_, idx, g64, g32, fd))
    big = {k: max(abs(r[4]) for r in res if r[0] == k) for k in ("v", "u", "a")}
    errs = []
    for kind_, idx, g64, g32, fd in res:
        e64, e32 = abs(g64 - fd) / big[kind_], abs(g32 - fd) / big[kind_]
        print(f"{kind} {kind_} {idx}: fd {fd:.9e} fp64 {g64:.9e} ({e64:.1e}) "
              f"mixed {g32:.9e} ({e32:.1e})")
        errs.append((e64, e32, kind_, idx))
    assert big["a"] > 0
    assert max(e[0] for e in errs) < 1e-4, errs
    assert max(e[1] for e in errs) < 1e-2, errs
