"""Restart from a Phantom dump on the GPU: a run is dumped, the dump is read back into a
new model with the configuration it implies (gen_config_from_phantom_dump: varying CD10
viscosity, the dump's CFL and particle mass, periodic box), and the restarted FP64 run
is bit-identical to the oracle started from the same loaded state."""

import warnings

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

KEYS_EXACT = ("n_ghost", "leaf_count", "cache_size", "h_subcycles", "h_iterations",
              "corrector_iters", "next_dt", "cfl_mult")


def test_restart_from_dump_bitexact(tmp_path):
    import shamrock_gb300 as sg
    from test_gpu_cd10 import _setup, make_pair

    s = _setup()
    model, _ = make_pair(s, cs0=0.2)
    for _ in range(2):
        model.evolve_once()
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")  # no unit system: SI defaults
        dump = model.make_phantom_dump()
    f = tmp_path / "restart_00002"
    dump.save_dump(str(f))

    back = sg.load_phantom_dump(str(f))
    m2 = sg.get_Model_SPH(context=sg.Context(), vector_type="f64_3", sph_kernel="M4")
    cfg = m2.gen_config_from_phantom_dump(back)
    cfg.set_precision("fp64")
    m2.set_solver_config(cfg)
    m2.init_from_phantom_dump(back)
    assert m2.get_time() == model.get_time()
    start = m2.collect_data()
    a = model.collect_data()
    assert np.array_equal(start["xyz"], a["xyz"]) and np.array_equal(start["uint"], a["uint"])
    assert np.array_equal(start["hpart"], a["hpart"].astype(np.float32).astype(np.float64))

    oc = O.OrcConfig(gamma=s["gamma"], pmass=s["pmass"], alpha_u=1.0, alpha_AV=0.0, beta_AV=2.0,
                     cfl_cour=0.3, cfl_force=0.3, cfl_mult_stiffness=2.0, htol_up_coarse=1.1,
                     htol_up_fine=1.1, epsilon_h=1e-6, h_iter_per_subcycles=50,
                     h_max_subcycles=100, tree_reduction_level=3, periodic=1, av_kind=1,
                     alpha_min=0.0, alpha_max=1.0, sigma_decay=0.1)
    oc.bmin[:] = list(m2.box_min)
    oc.bmax[:] = list(m2.box_max)
    sim = O.Sim(oc, start["xyz"], start["vxyz"], start["hpart"], start["uint"])
    sim.set_av(alpha=start["alpha_AV"], soundspeed=start["soundspeed"])
    sim.set_time(m2.get_time(), m2.get_dt(), m2.get_cfl_multipler())
    for k in range(3):
        lg = m2.evolve_once()
        lo = sim.evolve_once()
        for key in KEYS_EXACT:
            assert lg[key] == lo[key], (k, key, lg[key], lo[key])
        g, o = m2.collect_data(), sim.get()
        for key in ("xyz", "vxyz", "axyz", "hpart", "uint", "duint"):
            assert np.array_equal(g[key], o[key]), (k, key)
        assert np.array_equal(g["alpha_AV"], sim.get_av()["alpha_AV"]), k
