"""Adjoint of the SPH step (gbsph_adjoint_step, shamrock_gb300.adjoint.rollout) against
FP64 central finite differences of the same map.

The map: n steps from a warmed-up state with the dt sequence, the corrector counts and
the neighbour caches of the forward pass held fixed (the finite-difference runs replay
the recorded dt sequence).  Loss L = sum |v_final - v_target|^2 + sum (u_final - u_t)^2
with seeded targets.  Gradients with respect to initial velocities, internal energies,
positions and alpha_AV agree with central differences (eps = 1e-6 times the
coordinate's scale) to 1e-4, relative to the largest checked component."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def make_model(n_cells=6, jitter=0.05, vel_sigma=0.05, seed=3, precision="fp64"):
    import shamrock_gb300 as sg
    from shamrock_gb300 import setups

    rng = np.random.default_rng(seed)
    pos = setups.fcc_lattice(n_cells)
    N = pos.shape[0]
    spacing = 1.0 / n_cells
    pos = np.mod(pos + jitter * spacing * rng.standard_normal(pos.shape), 1.0)
    vel = vel_sigma * rng.standard_normal((N, 3))
    u = 1.0 + 0.2 * rng.random(N)
    pmass = 1.0 / N
    h = setups.HFACT_M4 * (pmass / 1.0) ** (1.0 / 3.0) * np.ones(N)
    ctx = sg.Context()
    m = sg.get_Model_SPH(context=ctx, vector_type="f64_3", sph_kernel="M4")
    cfg = m.gen_default_config()
    cfg.set_artif_viscosity_Constant(alpha_u=1.0, alpha_AV=1.0, beta_AV=2.0)
    cfg.set_boundary_periodic()
    cfg.set_eos_adiabatic(5.0 / 3.0)
    cfg.set_particle_mass(pmass)
    cfg.set_precision(precision)
    m.set_solver_config(cfg)
    m.resize_simulation_box((0, 0, 0), (1, 1, 1))
    m.set_particles(pos, vel, h, u)
    m.set_cfl_cour(0.3)
    m.set_cfl_force(0.3)
    m.evolve_once()  # dt = 0: initial h, Omega, a, du
    return m


def test_adjoint_matches_central_differences():
    import torch

    from shamrock_gb300 import adjoint

    m = make_model()
    from shamrock_gb300.adjoint import _restore, _snapshot

    warm = _snapshot(m)
    t0, dt0, cm0 = m.time, m.dt, m.cfl_mult
    N = m.get_total_part_count()
    rng = np.random.default_rng(7)
    dev = warm["vxyz"].device
    v_t = torch.as_tensor(0.05 * rng.standard_normal((3, N)), device=dev)
    u_t = torch.as_tensor(1.0 + 0.2 * rng.random(N), device=dev)
    n_steps, ck = 4, 2

    def loss_of(x, v, u):
        return ((v - v_t) ** 2).sum() + ((u - u_t) ** 2).sum()

    def run(v0, u0, alpha, x0, dts=None, grad=False):
        _restore(m, warm)
        m.time, m.dt, m.cfl_mult = t0, dt0, cm0
        x, v, u = adjoint.rollout(m, v0, u0, alpha, n_steps, ck, dts=dts, x0=x0)
        return loss_of(x, v, u)

    v0 = warm["vxyz"].clone().requires_grad_(True)
    u0 = warm["uint"].clone().requires_grad_(True)
    x0 = warm["xyz"].clone().requires_grad_(True)
    alpha = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
    L = run(v0, u0, alpha, x0)
    dts = list(adjoint.rollout.last_dts)
    assert all(d > 0 for d in dts)
    L.backward()
    g = dict(v=v0.grad.detach().cpu().numpy(), u=u0.grad.detach().cpu().numpy(),
             x=x0.grad.detach().cpu().numpy(), a=float(alpha.grad))

    # coordinates: 5 velocities, 4 energies, 3 positions, alpha
    coords = [("v", (int(rng.integers(3)), int(rng.integers(N)))) for _ in range(5)]
    coords += [("u", (int(rng.integers(N)),)) for _ in range(4)]
    coords += [("x", (int(rng.integers(3)), int(rng.integers(N)))) for _ in range(3)]
    coords += [("a", ())]
    base = dict(v=warm["vxyz"], u=warm["uint"], x=warm["xyz"])
    res = []
    for kind, idx in coords:
        scale = {"v": 0.05, "u": 1.0, "x": 1.0 / 6, "a": 1.0}[kind]
        eps = 1e-6 * scale
        Ls = []
        for sgn in (1, -1):
            vv, uu, xx = base["v"].clone(), base["u"].clone(), base["x"].clone()
            aa = 1.0
            if kind == "v":
                vv[idx] += sgn * eps
            elif kind == "u":
                uu[idx] += sgn * eps
            elif kind == "x":
                xx[idx] += sgn * eps
            else:
                aa += sgn * eps
            with torch.no_grad():
                Ls.append(float(run(vv, uu, torch.tensor(aa, dtype=torch.float64), xx, dts=dts)))
        fd = (Ls[0] - Ls[1]) / (2 * eps)
        ad = g[kind] if kind == "a" else float(g[kind][idx])
        res.append((kind, idx, ad, fd))
    big = max(abs(r[3]) for r in res)
    for kind, idx, ad, fd in res:
        err = abs(ad - fd) / max(abs(fd), 1e-3 * big)
        print(f"{kind} {idx}: adjoint {ad:.10e} fd {fd:.10e} rel err {err:.2e}")
        assert err < 1e-4, (kind, idx, ad, fd, err)


def _grads(precision, n_steps=4, ck=2, dts=None):
    import torch

    from shamrock_gb300 import adjoint
    from shamrock_gb300.adjoint import _snapshot

    m = make_model(precision=precision)
    warm = _snapshot(m)
    N = m.get_total_part_count()
    rng = np.random.default_rng(7)
    dev = warm["vxyz"].device
    v_t = torch.as_tensor(0.05 * rng.standard_normal((3, N)), device=dev)
    u_t = torch.as_tensor(1.0 + 0.2 * rng.random(N), device=dev)
    v0 = warm["vxyz"].clone().requires_grad_(True)
    u0 = warm["uint"].clone().requires_grad_(True)
    x0 = warm["xyz"].clone().requires_grad_(True)
    alpha = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
    x, v, u = adjoint.rollout(m, v0, u0, alpha, n_steps, ck, dts=dts, x0=x0)
    (((v - v_t) ** 2).sum() + ((u - u_t) ** 2).sum()).backward()
    return (dict(v=v0.grad.cpu().numpy(), u=u0.grad.cpu().numpy(), x=x0.grad.cpu().numpy(),
                 a=float(alpha.grad)), list(adjoint.rollout.last_dts))


def test_mixed_adjoint_matches_fp64_adjoint():
    """FP32-mixed forward + FP32 reverse pair arithmetic against the FP64 adjoint on the
    same dt sequence: each gradient field within 1e-3 in relative L2 norm."""
    g64, dts = _grads("fp64")
    g32, _ = _grads("mixed", dts=dts)
    for k in ("v", "u", "x"):
        rel = np.linalg.norm(g32[k] - g64[k]) / np.linalg.norm(g64[k])
        print(f"{k}: relative L2 difference {rel:.2e}")
        assert rel < 1e-3, (k, rel)
    rel_a = abs(g32["a"] - g64["a"]) / abs(g64["a"])
    print(f"alpha: {g32['a']:.10e} vs {g64['a']:.10e} rel {rel_a:.2e}")
    assert rel_a < 1e-3
