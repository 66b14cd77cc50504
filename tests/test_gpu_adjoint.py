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


def test_sound_wave_gradients_fd():
    """The differentiable sound wave: 64^3 = 2^18 particles, rho = 1 + 1e-4 sin(2 pi x),
    gamma 1.0001, alpha_AV 0.1, 40 steps with a checkpoint every 5, loss = |v_final -
    v_target|^2 (seeded target).  Gradients with respect to initial v, u and alpha_AV on
    16 seeded coordinates against FP64 central differences taken at two steps, eps and
    2 eps (v: 1e-7, alpha 1e-6 relative, u 1e-7 relative; the initial velocities are
    ~1e-4, and a step of 1e-6 on them leaves a truncation error of ~1e-4 in the
    differences), combined by Richardson extrapolation (4 D(eps) - D(2 eps)) / 3.
    The difference of the two steps is the differences' own error: a coordinate whose
    differences agree to 1e-5 resolves its gradient, and there the FP64 adjoint must
    agree to 1e-4.  Every v and alpha coordinate must also agree to 1e-4 of the largest
    checked gradient of its kind.  The u gradients (~1e-9 with gamma - 1 = 1e-4) pass
    through the conductivity speed |P_a - P_b|^(1/2), whose derivative grows as
    |dP|^(-1/2) for pairs of nearly equal pressure: no u coordinate's differences resolve
    to 1e-5, and they are held to 1e-3 of the largest.  The set-up carries seeded 1e-4
    velocity / energy noise so that no pair sits exactly on a kink of the step.  The FP64
    runs converge h to round-off (epsilon_h = epsilon_h_particle = 1e-13).
    The error-controlled mixed rollout runs its steps in the compensated tier (the FP32
    tier's estimate exceeds 1e-5 here) with the FP32 reverse pass; over the whole field
    its gradients agree with the FP64 adjoint to 1e-4 (v, relative L2), 1e-5 (alpha) and
    3e-3 (u, relative L2)."""
    import torch

    import bench
    from shamrock_gb300 import adjoint, setups
    from shamrock_gb300.adjoint import _restore, _snapshot

    s = setups.sound_wave(n_side=64, amp=1e-4, gamma=1.0001)
    steps, ck = 40, 5
    rng = np.random.default_rng(12345)
    N = len(s["h"])
    coords = [("v", (int(rng.integers(3)), int(rng.integers(N)))) for _ in range(8)]
    coords += [("u", (int(rng.integers(N)),)) for _ in range(7)]
    coords += [("a", ())]
    v_t_np = 1e-4 * rng.standard_normal((3, N))

    def setup(precision):
        m = bench.make_model(s, precision, 0, alpha_AV=0.1)
        if precision == "fp64":
            # h converged to round-off in every run, so that the differences resolve the
            # map the adjoint differentiates (h as the exact root of the density
            # constraint) rather than the 1e-6 Newton stopping noise
            m.cfg.set_epsilon_h(1e-13)
            m.cfg.set_epsilon_h_particle(1e-13)
        m.evolve_once()  # dt = 0
        return m, _snapshot(m), (m.time, m.dt, m.cfl_mult)

    def grads(m, warm, tstate, dts):
        _restore(m, warm)
        m.time, m.dt, m.cfl_mult = tstate
        v_t = torch.as_tensor(v_t_np, device=warm["vxyz"].device)
        v0 = warm["vxyz"].clone().requires_grad_(True)
        u0 = warm["uint"].clone().requires_grad_(True)
        al = torch.tensor(0.1, dtype=torch.float64, requires_grad=True)
        x, v, u = adjoint.rollout(m, v0, u0, al, steps, ck, dts=dts)
        ((v - v_t) ** 2).sum().backward()
        return (dict(v=v0.grad.cpu().numpy(), u=u0.grad.cpu().numpy(), a=float(al.grad)),
                list(adjoint.rollout.last_dts), list(adjoint.rollout.last_records))

    m64, warm64, ts64 = setup("fp64")
    g64, dts, _ = grads(m64, warm64, ts64, None)
    m32, warm32, ts32 = setup("mixed")
    g32, _, rec32 = grads(m32, warm32, ts32, dts)
    assert all(r[3] == 2 for r in rec32), [r[3] for r in rec32]  # compensated tier

    v_t = torch.as_tensor(v_t_np, device=warm64["vxyz"].device)

    def central(kind, idx, eps):
        Ls = []
        for sgn in (1, -1):
            _restore(m64, warm64)
            m64.time, m64.dt, m64.cfl_mult = ts64
            vv, uu, aa = warm64["vxyz"].clone(), warm64["uint"].clone(), 0.1
            if kind == "v":
                vv[idx] += sgn * eps
            elif kind == "u":
                uu[idx] += sgn * eps
            else:
                aa += sgn * eps
            with torch.no_grad():
                x, v, u = adjoint.rollout(m64, vv, uu, torch.tensor(aa, dtype=torch.float64),
                                          steps, ck, dts=dts)
                Ls.append(float(((v - v_t) ** 2).sum()))
        return (Ls[0] - Ls[1]) / (2 * eps)

    res = []
    for kind, idx in coords:
        eps = {"v": 1e-7, "u": 1e-7 * float(warm64["uint"][0]), "a": 1e-6 * 0.1}[kind]
        d1, d2 = central(kind, idx, eps), central(kind, idx, 2 * eps)
        fd = (4 * d1 - d2) / 3
        a64 = g64[kind] if kind == "a" else float(g64[kind][idx])
        res.append((kind, idx, a64, fd, abs(d1 - d2) / abs(d1)))
    big = {k: max(abs(r[3]) for r in res if r[0] == k) for k in ("v", "u", "a")}
    resolved = 0
    for kind, idx, a64, fd, self_err in res:
        e_own, e_big = abs(a64 - fd) / abs(fd), abs(a64 - fd) / big[kind]
        print(f"{kind} {idx}: fd {fd:.9e} (self {self_err:.1e}) fp64 {a64:.9e} "
              f"({e_own:.1e} own, {e_big:.1e} of largest)")
        if self_err < 1e-5:
            resolved += 1
            assert e_own <= 1e-4, (kind, idx, e_own)
        assert e_big <= (1e-3 if kind == "u" else 1e-4), (kind, idx, e_big)
    print(f"{resolved} of {len(res)} coordinates resolved by their differences")
    assert resolved >= 6
    # the mixed (compensated forward, FP32 reverse) gradients against the FP64 adjoint
    rel = {k: float(np.linalg.norm(g32[k] - g64[k]) / np.linalg.norm(g64[k])) for k in ("v", "u")}
    rel["a"] = abs(g32["a"] - g64["a"]) / abs(g64["a"])
    print("mixed vs fp64 adjoint:", rel)
    assert rel["v"] <= 1e-4 and rel["a"] <= 1e-5 and rel["u"] <= 3e-3, rel


def _disc_model(s, precision):
    import shamrock_gb300 as sg

    m = sg.get_Model_SPH(context=sg.Context(), vector_type="f64_3", sph_kernel="M4")
    cfg = m.gen_default_config()
    cfg.set_artif_viscosity_Constant(alpha_u=1.0, alpha_AV=0.5, beta_AV=2.0)
    cfg.set_boundary_free()
    cfg.set_eos_locally_isothermalLP07(cs0=s["cs0"], q=s["q"], r0=s["r0"])
    cfg.add_ext_force_point_mass(s["M"], 0.0)
    cfg.set_constant_G(s["G"])
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
    m.evolve_once()  # dt = 0
    return m


def test_disc_adjoint_kinetic_energy_fd():
    """Keplerian disc (locally isothermal LP07 EOS, central point mass, free boundary):
    loss = total kinetic energy after 6 steps (checkpoint every 3); gradients with
    respect to the initial velocities and alpha_AV against FP64 central differences
    (relative steps 1e-6), within 1e-4 of the largest checked component of each kind;
    the FP32-mixed gradients within 1e-2."""
    import torch

    from shamrock_gb300 import adjoint, setups
    from shamrock_gb300.adjoint import _restore, _snapshot

    s = setups.keplerian_disc(4000, seed=7)
    steps, ck = 6, 3
    out = {}
    for prec in ("fp64", "mixed"):
        m = _disc_model(s, prec)
        warm, ts = _snapshot(m), (m.time, m.dt, m.cfl_mult)
        v0 = warm["vxyz"].clone().requires_grad_(True)
        u0 = warm["uint"].clone().requires_grad_(True)
        al = torch.tensor(0.5, dtype=torch.float64, requires_grad=True)
        dts = out["dts"] if "dts" in out else None
        x, v, u = adjoint.rollout(m, v0, u0, al, steps, ck, dts=dts)
        (0.5 * s["pmass"] * (v * v).sum()).backward()
        out[prec] = (v0.grad.cpu().numpy(), float(al.grad))
        if prec == "fp64":
            out["dts"] = list(adjoint.rollout.last_dts)
            m64, warm64, ts64 = m, warm, ts
    rng = np.random.default_rng(3)
    N = len(s["h"])
    coords = [("v", (int(rng.integers(3)), int(rng.integers(N)))) for _ in range(8)] + [("a", ())]
    res = []
    for kind, idx in coords:
        eps = 1e-6 if kind == "v" else 0.5e-6
        Ls = []
        for sgn in (1, -1):
            _restore(m64, warm64)
            m64.time, m64.dt, m64.cfl_mult = ts64
            vv, aa = warm64["vxyz"].clone(), 0.5
            if kind == "v":
                vv[idx] += sgn * eps
            else:
                aa += sgn * eps
            with torch.no_grad():
                x, v, u = adjoint.rollout(m64, vv, warm64["uint"].clone(),
                                          torch.tensor(aa, dtype=torch.float64), steps, ck,
                                          dts=out["dts"])
                Ls.append(float(0.5 * s["pmass"] * (v * v).sum()))
        fd = (Ls[0] - Ls[1]) / (2 * eps)
        g64 = out["fp64"][1] if kind == "a" else float(out["fp64"][0][idx])
        g32 = out["mixed"][1] if kind == "a" else float(out["mixed"][0][idx])
        res.append((kind, idx, g64, g32, fd))
    # normalised by the largest checked component of the kind: the v_z gradients of this
    # thin disc are ~1e-3 of the in-plane ones and their differences sit at round-off
    big = {k: max(abs(r[4]) for r in res if r[0] == k) for k in ("v", "a")}
    errs = []
    for kind, idx, g64, g32, fd in res:
        e64, e32 = abs(g64 - fd) / big[kind], abs(g32 - fd) / big[kind]
        print(f"{kind} {idx}: fd {fd:.9e} fp64 {g64:.9e} ({e64:.1e}) mixed {g32:.9e} ({e32:.1e})")
        errs.append((e64, e32, kind, idx))
    assert max(e[0] for e in errs) < 1e-4, errs
    assert max(e[1] for e in errs) < 1e-2, errs


@pytest.mark.parametrize("precision", ["fp64", "mixed_fp32"])
def test_record_reverse_equals_adjoint_step(precision):
    """gbsph_adjoint_record + gbsph_adjoint_reverse on a context of their own give the
    cotangents of gbsph_adjoint_step bit for bit (and dL/d alpha_AV, a sum the blocks add
    in arrival order, to round-off); a reverse without a recording is refused
    (GBSPH_ERR_STATE); the state after a recorded step equals the forward step's."""
    import ctypes as C

    import torch

    from shamrock_gb300 import _lib as L
    from shamrock_gb300 import adjoint
    from shamrock_gb300.adjoint import _cot_struct, _particles_of, _snapshot

    m = make_model(precision=precision)
    start = _snapshot(m)
    t, dt = m.time, m.dt
    log = m.evolve_once()
    after_fwd = _snapshot(m)
    N = m.get_total_part_count()
    dev = start["vxyz"].device
    rng = np.random.default_rng(11)

    def cot0():
        c = adjoint._zero_cot(N, dev)
        c["gv"].copy_(torch.as_tensor(rng.standard_normal((3, N)), device=dev))
        c["gu"].copy_(torch.as_tensor(rng.standard_normal(N), device=dev))
        return c

    ref = cot0()
    cot = {k: v.clone() for k, v in ref.items()}
    g_ref = adjoint.adjoint_step(m, start, t, dt, log["corrector_iters"], ref, log["tier"])

    ctx = L.Context(0)
    p = _particles_of(start)
    cfg = m._config_struct(log["tier"])
    cs = _cot_struct(cot)
    g = C.c_double(0.0)
    rc = ctx.lib.gbsph_adjoint_reverse(ctx.handle, C.byref(p), C.byref(cfg), float(dt),
                                       C.byref(cs), C.byref(g), None)
    assert rc == L.GBSPH_ERR_STATE
    after = L.Particles()
    ctx.check(ctx.lib.gbsph_adjoint_record(ctx.handle, C.byref(p), C.byref(cfg), float(t),
                                           float(dt), int(log["corrector_iters"]), C.byref(after),
                                           None))
    torch.cuda.synchronize()
    # the recomputed state after the step is the forward step's, bit for bit
    class _View:  # a device array the library owns, seen through the CUDA array interface
        def __init__(self, ptr):
            self.__cuda_array_interface__ = {"shape": (N,), "typestr": "<f8", "data": (ptr, False),
                                             "version": 2}

    for k, ptr in (("hpart", after.hpart), ("uint", after.uint), ("duint", after.duint)):
        got = torch.as_tensor(_View(ptr), device=dev).clone()
        assert torch.equal(got, after_fwd[k]), k
    ctx.check(ctx.lib.gbsph_adjoint_reverse(ctx.handle, C.byref(p), C.byref(cfg), float(dt),
                                            C.byref(cs), C.byref(g), None))
    torch.cuda.synchronize()
    for k in ref:
        assert torch.equal(cot[k], ref[k]), k
    assert abs(g.value - g_ref) <= 1e-12 * abs(g_ref)
    ctx.close()
