"""Full Solver::evolve_once on the GPU through the reference-shaped model API, against
the oracle's FP64 evolve_once.

FP64: particle fields after every step are bit-identical to the oracle; the step
bookkeeping (ghost count, leaves, cache size, sub-cycles, Newton iterations, corrector
iterations, next dt, CFL multiplier) matches exactly, eps_v to 1e-12 (its global sum
is reduced in a different order).
FP32-mixed: one step from the same state; density (through h) and |a|, du/dt within
1e-5 of FP64, normalised by the field's largest magnitude."""

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def make_pair(setup, precision="fp64", cfl=0.3, periodic=True, stride4=False):
    import shamrock_gb300 as sg

    s = setup
    ctx = sg.Context()
    model = sg.get_Model_SPH(context=ctx, vector_type="f64_3", sph_kernel="M4")
    cfg = model.gen_default_config()
    cfg.set_artif_viscosity_Constant(alpha_u=1.0, alpha_AV=1.0, beta_AV=2.0)
    if periodic:
        cfg.set_boundary_periodic()
    else:
        cfg.set_boundary_free()
    cfg.set_eos_adiabatic(s["gamma"])
    cfg.set_particle_mass(s["pmass"])
    cfg.set_precision(precision)
    model.set_solver_config(cfg)
    model.resize_simulation_box(s["box_min"], s["box_max"])
    model.set_particles(s["pos"], s["vel"], s["h"], s["u"])
    model.set_cfl_cour(cfl)
    model.set_cfl_force(cfl)
    oc = O.OrcConfig(gamma=s["gamma"], pmass=s["pmass"], alpha_u=1.0, alpha_AV=1.0, beta_AV=2.0,
                     cfl_cour=cfl, cfl_force=cfl, cfl_mult_stiffness=2.0, htol_up_coarse=1.1,
                     htol_up_fine=1.1, epsilon_h=1e-6, h_iter_per_subcycles=50,
                     h_max_subcycles=100, tree_reduction_level=3, periodic=1 if periodic else 0)
    oc.bmin[:] = list(s["box_min"])
    oc.bmax[:] = list(s["box_max"])
    sim = O.Sim(oc, s["pos"], s["vel"], s["h"], s["u"])
    return model, sim


KEYS_EXACT = ("n_ghost", "leaf_count", "cache_size", "h_subcycles", "h_iterations",
              "corrector_iters", "next_dt", "cfl_mult")


def compare_fields(model, sim):
    g = model.collect_data()
    o = sim.get()
    for k in ("xyz", "vxyz", "axyz", "hpart", "uint", "duint", "omega"):
        assert np.array_equal(g[k], o[k]), k


@pytest.mark.parametrize("n_cells,jitter,steps", [(8, 0.0, 6), (10, 0.05, 4)])
def test_sedov_fp64_bitexact(n_cells, jitter, steps):
    from shamrock_gb300 import setups

    s = setups.sedov_taylor(n_cells, jitter=jitter, seed=1)
    model, sim = make_pair(s)
    for k in range(steps):
        lg = model.evolve_once()
        lo = sim.evolve_once()
        for key in KEYS_EXACT:
            assert lg[key] == lo[key], (k, key, lg[key], lo[key])
        assert abs(lg["eps_v"] - lo["eps_v"]) <= 1e-12 * max(abs(lo["eps_v"]), 1e-300) + 1e-300
        compare_fields(model, sim)


def test_duplicate_morton_keys_fp64_bitexact():
    """Pairs of particles 1e-6 apart share their Morton cell: equal keys, whose order is
    fixed by the bitonic network.  The step sorts with the radix sort first and must
    notice the ties and fall back to the network (fifty tied pairs in the stable order
    of the radix sort would not match the oracle's permutation by chance)."""
    from shamrock_gb300 import setups

    s = setups.sedov_taylor(8, jitter=0.05, seed=6)
    rng = np.random.default_rng(6)
    pick = rng.choice(len(s["h"]), 50, replace=False)
    extra = s["pos"][pick] + 1e-6 * rng.standard_normal((50, 3))
    s = dict(s)
    s["pos"] = np.concatenate([s["pos"], extra])
    s["vel"] = np.concatenate([s["vel"], s["vel"][pick]])
    s["h"] = np.concatenate([s["h"], s["h"][pick]])
    s["u"] = np.concatenate([s["u"], s["u"][pick]])
    model, sim = make_pair(s)
    for k in range(2):
        lg = model.evolve_once()
        lo = sim.evolve_once()
        for key in KEYS_EXACT:
            assert lg[key] == lo[key], (k, key)
        compare_fields(model, sim)


def test_conservation_totals():
    """gbsph_conservation (the reference's ConservativeCheck sums) against numpy sums of
    the same fields: FP64, agreement to summation-order round-off."""
    from shamrock_gb300 import setups

    s = setups.sedov_taylor(8, jitter=0.05, seed=2)
    model, _ = make_pair(s)
    for _ in range(2):
        model.evolve_once()
    tot = model.conservation_totals()
    d = model.collect_data()
    m = s["pmass"]
    v, a = d["vxyz"], d["axyz"]
    scale_v = m * np.abs(v).sum()
    scale_a = m * np.abs(a).sum()
    assert np.allclose(tot["momentum"], m * v.sum(0), rtol=0, atol=1e-12 * scale_v)
    assert np.allclose(tot["force"], m * a.sum(0), rtol=0, atol=1e-12 * scale_a)
    e = m * np.sum(d["uint"] + 0.5 * np.sum(v * v, 1))
    de = m * np.sum(np.sum(v * a, 1) + d["duint"])
    assert abs(tot["energy"] - e) <= 1e-12 * abs(e)
    assert abs(tot["energy_rate"] - de) <= 1e-10 * (m * np.sum(np.abs(np.sum(v * a, 1)) + np.abs(d["duint"])))


def test_clustered_free_boundary_fp64_bitexact():
    from shamrock_gb300 import setups

    s = setups.clustered_box(8000, seed=4, sigma=0.2)
    s["vel"] = s["vel"] * 0.1
    model, sim = make_pair(s, periodic=False)
    for k in range(3):
        lg = model.evolve_once()
        lo = sim.evolve_once()
        for key in KEYS_EXACT:
            assert lg[key] == lo[key], (k, key)
        compare_fields(model, sim)


def test_aos_stride4_layout_matches_soa():
    """The reference's padded f64_3 layout (stride 4) through the C ABI gives the same
    step as structure-of-arrays."""
    import ctypes as C

    import torch

    import shamrock_gb300 as sg
    from shamrock_gb300 import _lib as L
    from shamrock_gb300 import setups

    s = setups.sedov_taylor(6, jitter=0.05, seed=2)
    model, _ = make_pair(s)
    model.evolve_once()
    ref = model.collect_data()
    # same first step through a stride-4 AoS particle struct
    m2, _ = make_pair(s)
    cfg = m2._config_struct()
    n = len(s["h"])
    dev = "cuda"
    aos = {k: torch.zeros((n, 4), dtype=torch.float64, device=dev) for k in ("xyz", "vxyz", "axyz")}
    aos["xyz"][:, :3] = torch.as_tensor(s["pos"], device=dev)
    aos["vxyz"][:, :3] = torch.as_tensor(s["vel"], device=dev)
    h = torch.as_tensor(s["h"].copy(), device=dev)
    u = torch.as_tensor(s["u"].copy(), device=dev)
    du = torch.zeros(n, dtype=torch.float64, device=dev)
    p = L.Particles()
    p.n = n
    for k in ("xyz", "vxyz", "axyz"):
        b = aos[k].data_ptr()
        setattr(p, k, L.Vec3(b, b + 8, b + 16, 4, 0))
    p.hpart, p.uint, p.duint, p.omega = h.data_ptr(), u.data_ptr(), du.data_ptr(), None
    ts = L.TimeState(0.0, 0.0, 1e-2)
    log = L.StepLog()
    lib = m2._lib()
    lib.check(lib.lib.gbsph_evolve_once(lib.handle, C.byref(p), C.byref(cfg), C.byref(ts),
                                        C.byref(log), None))
    assert np.array_equal(aos["xyz"][:, :3].cpu().numpy(), ref["xyz"])
    assert np.array_equal(aos["axyz"][:, :3].cpu().numpy(), ref["axyz"])
    assert np.array_equal(h.cpu().numpy(), ref["hpart"])
    assert np.array_equal(du.cpu().numpy(), ref["duint"])


def _norm_err(x, ref):
    x, ref = np.asarray(x), np.asarray(ref)
    if ref.ndim > 1:
        return np.linalg.norm(x - ref, axis=1).max() / np.linalg.norm(ref, axis=1).max()
    return np.abs(x - ref).max() / np.abs(ref).max()


@pytest.mark.parametrize("n_cells,jitter", [(10, 0.05), (12, 0.05)])
def test_mixed_step_error(n_cells, jitter):
    from shamrock_gb300 import setups

    s = setups.sedov_taylor(n_cells, jitter=jitter, seed=1)
    m64, _ = make_pair(s, "fp64")
    m32, _ = make_pair(s, "mixed")
    # first step (dt = 0) from the same state, then a second from each one's own state
    m64.evolve_once()
    m32.evolve_once()
    g64, g32 = m64.collect_data(), m32.collect_data()
    rho64 = s["pmass"] * (1.2 / g64["hpart"]) ** 3
    rho32 = s["pmass"] * (1.2 / g32["hpart"]) ** 3
    tol = 1e-5
    assert np.abs(rho32 - rho64).max() / rho64.max() <= tol
    assert np.max(np.abs(rho32 - rho64) / rho64) <= tol
    assert _norm_err(g32["axyz"], g64["axyz"]) <= tol
    assert _norm_err(g32["duint"], g64["duint"]) <= tol
    assert _norm_err(g32["omega"], g64["omega"]) <= tol


def _disc_pair(s, precision="fp64", alpha_AV=0.5):
    import shamrock_gb300 as sg

    ctx = sg.Context()
    m = sg.get_Model_SPH(context=ctx, vector_type="f64_3", sph_kernel="M4")
    cfg = m.gen_default_config()
    cfg.set_artif_viscosity_Constant(alpha_u=1.0, alpha_AV=alpha_AV, beta_AV=2.0)
    cfg.set_boundary_free()
    cfg.set_eos_locally_isothermalLP07(cs0=s["cs0"], q=s["q"], r0=s["r0"])
    cfg.add_ext_force_point_mass(s["M"], 0.0)
    cfg.set_constant_G(s["G"])
    cfg.set_particle_mass(s["pmass"])
    cfg.set_precision(precision)
    m.set_solver_config(cfg)
    m.resize_simulation_box(s["box_min"], s["box_max"])
    m.set_particles(s["pos"], s["vel"], s["h"], s["u"])
    m.set_cfl_cour(0.3)
    m.set_cfl_force(0.3)
    oc = O.OrcConfig(gamma=s["gamma"], pmass=s["pmass"], alpha_u=1.0, alpha_AV=alpha_AV,
                     beta_AV=2.0, cfl_cour=0.3, cfl_force=0.3, cfl_mult_stiffness=2.0,
                     htol_up_coarse=1.1, htol_up_fine=1.1, epsilon_h=1e-6,
                     h_iter_per_subcycles=50, h_max_subcycles=100, tree_reduction_level=3,
                     periodic=0, eos_kind=1, ext_kind=1, cs0=s["cs0"], eos_r0=s["r0"],
                     eos_q=s["q"], central_mass=s["M"], constant_G=s["G"])
    oc.bmin[:] = list(s["box_min"])
    oc.bmax[:] = list(s["box_max"])
    return m, O.Sim(oc, s["pos"], s["vel"], s["h"], s["u"])


def test_disc_locally_isothermal_point_mass_fp64_vs_oracle():
    """Keplerian disc with the locally isothermal (LP07) EOS and the central point mass:
    the FP64 step against the oracle.  c_s^2 goes through pow, whose last bit differs
    between CUDA and the C library, so fields agree to round-off (1e-12) rather than bit
    for bit; the step bookkeeping (leaves, cache, sub-cycles, iterations) is identical."""
    from shamrock_gb300 import setups

    s = setups.keplerian_disc(6000, seed=5)
    model, sim = _disc_pair(s)
    for k in range(3):
        lg = model.evolve_once()
        lo = sim.evolve_once()
        for key in ("n_ghost", "leaf_count", "cache_size", "h_subcycles", "h_iterations",
                    "corrector_iters"):
            assert lg[key] == lo[key], (k, key, lg[key], lo[key])
        assert lg["next_dt"] == pytest.approx(lo["next_dt"], rel=1e-12)
        g, o = model.collect_data(), sim.get()
        for f in ("xyz", "vxyz", "axyz", "hpart", "uint", "duint", "omega"):
            scale = np.abs(o[f]).max()
            assert np.abs(g[f] - o[f]).max() <= 1e-12 * scale, (k, f)


def test_disc_mixed_vs_fp64_one_step():
    """The same disc, one FP32-mixed step against one FP64 step from the same state:
    h (density) per particle and |a|, du/dt normalised by their largest magnitude
    within 1e-5."""
    from shamrock_gb300 import setups

    s = setups.keplerian_disc(20000, seed=6)
    m64, _ = _disc_pair(s, "fp64")
    m32, _ = _disc_pair(s, "mixed")
    m64.evolve_once()
    m32.evolve_once()
    a, b = m32.collect_data(), m64.collect_data()
    assert np.abs(a["hpart"] / b["hpart"] - 1).max() < 1e-5
    for f in ("axyz", "duint"):
        d = np.abs(a[f] - b[f]).max()
        assert d <= 1e-5 * np.abs(b[f]).max(), (f, d / np.abs(b[f]).max())
