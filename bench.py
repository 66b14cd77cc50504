"""Benchmark of the GB300 SPH timestep hot path (one JSON line on stdout, rank 0).

Workload (SPH particle-steps/s): Sedov-Taylor blast, FCC lattice 4*64^3 = 1,048,576
equal-mass particles in the periodic unit cube, Gaussian position jitter 0.05 of the
lattice spacing (seed 1), rho = 1, u = 1e-5, E = 1 injected within r < 2 spacings,
gamma = 5/3, M4, hfact 1.2, constant AV alpha = 1 beta = 2, CFL 0.3, tree and
neighbour cache rebuilt every step; FP32-mixed pair arithmetic (--precision fp64
for the FP64 path).  One step = one full Solver::evolve_once.

Arms
  default          the GB300 path: `value` is device-timed (CUDA events, inputs resident
                   in HBM); `e2e` is the same metric through the public model API with the
                   particle state copied from pinned host memory before and back after
                   every step; `cpu_baseline` times the FP64 oracle on the host cores on
                   a bounded sample; `roofline` reports the dominant stage.
  --impl reference the reference's CPU implementation of the path: the reference cannot
                   be built here (SYCL), so this is the FP64 oracle restatement, OpenMP on
                   every host core, on the same workload.
Under torchrun each rank runs an independent replica (the path does not shard across
GPUs in this build); value = all ranks' particle-steps / max rank time.
"""

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "SPH particle-steps/s (FP32-mixed vs FP64 at <=1e-5 rel err)"
UNIT = "particle-steps/s"
L2_BYTES = 126 * 2**20


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--precision", default="mixed",
                   choices=["mixed", "mixed_fp32", "mixed_compensated", "fp64"],
                   help="mixed: error-controlled (FP32 pair arithmetic, compensated where the "
                        "step's error estimate exceeds 1e-5); mixed_fp32: FP32 without the "
                        "control; mixed_compensated: the compensated tier on every step")
    p.add_argument("--workload", default="sedov",
                   choices=["sedov", "sedov_plain", "clustered", "soundwave", "disc", "homogeneous"],
                   help="sedov: jittered Sedov-Taylor (default, 4*cells^3); sedov_plain: the "
                        "same without jitter; clustered: 8,388,608 particles, half uniform, "
                        "half in a Gaussian clump; soundwave: 64^3 travelling sound wave; "
                        "disc: 4,194,304-particle Keplerian disc (locally isothermal EOS, "
                        "central point mass, free boundary); homogeneous: the reference's own "
                        "SPH benchmark, 33,848,064-particle HCP box, varying CD10 viscosity, "
                        "dt = 0 steps")
    p.add_argument("--cells", type=int, default=64, help="FCC cells per axis (4*cells^3 particles)")
    p.add_argument("--n-target", type=int, default=1 << 25,
                   help="homogeneous: particle count the HCP box is sized for (the reference's "
                        "benchmark uses 2^25)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-accuracy", action="store_true")
    p.add_argument("--no-adjoint", action="store_true")
    p.add_argument("--cpu-seconds", type=float, default=20.0,
                   help="bounded CPU-baseline sample, seconds of host work")
    return p.parse_args()


def workload(cells, kind="sedov", n_target=1 << 25):
    """Seeded synthetic inputs with the shapes of the benchmark configurations (no
    dataset is involved).  Returns (set-up dict, name, alpha_AV)."""
    from shamrock_gb300 import setups

    if kind == "homogeneous":
        s = homogeneous_setup(n_target)
        name = ("homogeneous_hcp_box_%d (the reference's examples/benchmarks/"
                "sph_homogeneous_benchmark.py: HCP lattice in the periodic box it closes, rho 1, "
                "u = 0 but a central injection u_inj W(r, 16 dr), gamma 5/3, M4, varying CD10 "
                "viscosity alpha in [0, 1] sigma 0.1 alpha_u 1 beta 2, CFL 0.1, every step "
                "with dt = 0 as its set_next_dt(0.0), tree rebuilt every step)" % len(s["h"]))
        return s, name, 0.0
    if kind == "clustered":
        s = setups.clustered_box(8388608, seed=12345, sigma=0.05)
        name = ("clustered_box_8388608 (half uniform, half Gaussian clump sigma 0.05, "
                "v ~ N(0, 0.1^2), u ~ U[0.5, 1.5], gamma 5/3, M4, constant AV a=1 b=2, "
                "CFL 0.3, periodic, tree rebuilt every step)")
        return s, name, 1.0
    if kind == "disc":
        s = setups.keplerian_disc(4194304, seed=12345)
        name = ("keplerian_disc_4194304 (point mass M=1 G=1, r in [0.1, 1], Sigma ~ 1/r, H/R 0.05 "
                "at r=1, locally isothermal LP07 c_s ~ r^-0.25, constant AV a=0.5 b=2, CFL 0.3, "
                "free boundary, tree rebuilt every step)")
        return s, name, 0.5
    if kind == "soundwave":
        s = setups.sound_wave(n_side=64, amp=1e-4, gamma=1.0001)
        name = ("sound_wave_cubic_64^3 (N=262144, amp 1e-4, gamma 1.0001, constant AV "
                "a=0.1 b=2, CFL 0.3, periodic)")
        return s, name, 0.1
    jitter = 0.05 if kind == "sedov" else 0.0
    s = setups.sedov_taylor(cells, jitter=jitter, seed=1)
    name = (f"sedov_taylor_fcc_4x{cells}^3_jitter{jitter:g}_periodic (N={len(s['h'])}, M4, "
            "constant AV a=1 b=2, gamma=5/3, CFL 0.3, tree rebuilt every step)")
    return s, name, 1.0


def homogeneous_setup(n_target):
    from shamrock_gb300 import setups

    s = setups.homogeneous_box(n_target)
    s.update(av="cd10", cfl=0.1, dt_zero=True)
    return s


def step(m, s, **kw):
    """One evolve_once; the homogeneous benchmark sets the next dt to 0 before each."""
    if s.get("dt_zero"):
        m.dt = 0.0
    return m.evolve_once(**kw)


def ostep(sim, s):
    if s.get("dt_zero"):
        t, _, cm = sim.get_time()
        sim.set_time(t, 0.0, cm)
    return sim.evolve_once()


def make_model(s, precision, device=0, alpha_AV=1.0):
    import shamrock_gb300 as sg

    ctx = sg.Context(device)
    m = sg.get_Model_SPH(context=ctx, vector_type="f64_3", sph_kernel="M4")
    cfg = m.gen_default_config()
    if s.get("av") == "cd10":
        cfg.set_artif_viscosity_VaryingCD10(alpha_min=0.0, alpha_max=1.0, sigma_decay=0.1,
                                            alpha_u=1.0, beta_AV=2.0)
    else:
        cfg.set_artif_viscosity_Constant(alpha_u=1.0, alpha_AV=alpha_AV, beta_AV=2.0)
    if s.get("periodic", True):
        cfg.set_boundary_periodic()
    else:
        cfg.set_boundary_free()
    if "cs0" in s:
        cfg.set_eos_locally_isothermalLP07(cs0=s["cs0"], q=s["q"], r0=s["r0"])
        cfg.add_ext_force_point_mass(s["M"], 0.0)
        cfg.set_constant_G(s["G"])
    else:
        cfg.set_eos_adiabatic(s["gamma"])
    cfg.set_particle_mass(s["pmass"])
    cfg.set_precision(precision)
    m.set_solver_config(cfg)
    m.resize_simulation_box(s["box_min"], s["box_max"])
    m.set_particles(s["pos"], s["vel"], s["h"], s["u"])
    m.set_cfl_cour(s.get("cfl", 0.3))
    m.set_cfl_force(s.get("cfl", 0.3))
    return m


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        # a private temporary file (BENCH_CLOCKS_CSV keeps the samples somewhere chosen)
        self.path = os.environ.get("BENCH_CLOCKS_CSV") or os.path.join(
            tempfile.gettempdir(), f"gbsph_bench_clocks_{os.getpid()}_rank{device}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return None
        sm, smax, reasons = [], 0.0, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = max(smax, float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


# ----------------------------------------------------------------------------- roofline
# Compulsory DRAM bytes per unit of each stage (neighbour-field gathers are counted as
# L1/L2 hits; index streams and per-particle fields are counted).  units: rows (local
# particles), entries (CSR entries), keys (sorted slots).
def stage_bytes(stage, n, N, entries, P, precision, h_iters, kept=None):
    mixed = precision.startswith("mixed")
    vec = 64 if mixed else 88
    table = {
        # row_rank, row_local, cnt, off, own fields, CSR entries, caller a/du/v/u in+out,
        # h; every particle's record read once from DRAM (further gathers: L1/L2 hits)
        # (entries: the rows as the derivatives read them, compacted in the FP32 tier)
        "derivs": n * (16 + vec + 128 + 8) + 4 * (kept or entries) + N * vec,
        # per Newton iteration: CSR entries + own position + per-row h/eps state
        "h_iterate": (n * (16 + (32 if mixed else 24) + 40) + 4 * entries) * h_iters,
        "cache_fill": n * (4 + 4 + 4 + 32) + 4 * entries,
        "cache_count": n * (4 + 4 + 4 + 32),
        "omega": n * (16 + 32 + 8 + 8) + 4 * entries,
        "morton_sort": 16 * P,
        "gather_eos": N * (4 + 4 + 8 * 8) + N * (80 if mixed else 64),
    }
    return table.get(stage)


def roofline(prof, log, n, precision, peaks_path):
    ms = {k: v[0] for k, v in prof.items()}
    dom = max(ms, key=ms.get)
    launches = prof[dom][1]
    entries = int(log["cache_size"])
    # the entries the derivatives visit (the FP32 tier's compacted rows)
    kept = int(log.get("cache_kept") or entries)
    N = n + int(log["n_ghost"])
    P = 1 << (N - 1).bit_length()
    h_iters = max(1, int(log["h_iterations"]))
    nbytes = stage_bytes(dom, n, N, entries, P, precision, h_iters, kept)
    peak, peak_src = 6800.0, "fallback"
    try:
        with open(peaks_path) as f:
            peak = float(json.load(f)["hbm_gbs"])
            peak_src = "measured"
    except (OSError, KeyError, ValueError):
        pass
    out = {"bound": "hbm", "kernel": dom, "unit": "GB/s", "peak": peak, "peak_source": peak_src,
           "launches": launches, "ms_per_launch": ms[dom] / max(launches, 1),
           "share_of_step": ms[dom] / max(sum(ms.values()), 1e-12)}
    if nbytes is not None and launches:
        achieved = nbytes / (ms[dom] / launches * 1e-3) / 1e9
        out.update(achieved=achieved, frac=achieved / peak, algorithmic_bytes=nbytes)
    else:
        out.update(achieved=None, frac=None, algorithmic_bytes=None)
    out["traffic"] = traffic_from_profiles(dom, n)
    out["stages_ms"] = {k: round(v, 4) for k, v in ms.items()}
    return out


def traffic_from_profiles(stage, n):
    """DRAM bytes per launch of `stage` from the committed ncu summary (bytes per local
    particle of one launch), scaled to n local particles."""
    path = os.path.join(ROOT, "profiles", "dram_traffic.txt")
    try:
        for line in open(path):
            parts = line.split()
            if len(parts) >= 2 and parts[0] == stage and not line.startswith("#"):
                return float(parts[1]) * n
    except (OSError, ValueError):
        pass
    return None


# ----------------------------------------------------------------------------- arms
def dist_setup(backend=None):
    """Rank / world from the torchrun environment; a process group when world > 1
    (NCCL on GPUs, gloo otherwise).  Ranks are independent replicas: the group only
    carries the barrier and the max-over-ranks time."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch
        import torch.distributed as dist

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        if backend is None:
            backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend)
        pg = dist
    return world, rank, local, pg


def max_over_ranks(t_ms, dist, device="cpu"):
    """The slowest rank's time (the whole job ends when it does)."""
    if dist is None:
        return float(t_ms)
    import torch

    t = torch.tensor([float(t_ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(n_per_rank, world, steps, t_max_ms):
    """Particle-steps per second of all replicas together."""
    return n_per_rank * world * steps / (t_max_ms * 1e-3)


def reference_rank_runs(world, rank):
    """Under torchrun the reference arm runs on rank 0 alone; other ranks exit 0."""
    return world <= 1 or rank == 0


def oracle_config(O, s, alpha_AV):
    """The oracle's configuration of workload `s` (same solver settings as make_model)."""
    disc = "cs0" in s
    cfl = s.get("cfl", 0.3)
    oc = O.OrcConfig(gamma=s["gamma"], pmass=s["pmass"], alpha_u=1.0, alpha_AV=alpha_AV, beta_AV=2.0,
                     cfl_cour=cfl, cfl_force=cfl, cfl_mult_stiffness=2.0, htol_up_coarse=1.1,
                     htol_up_fine=1.1, epsilon_h=1e-6, h_iter_per_subcycles=50,
                     h_max_subcycles=100, tree_reduction_level=3,
                     periodic=1 if s.get("periodic", True) else 0)
    if disc:
        oc.eos_kind, oc.ext_kind = 1, 1
        oc.cs0, oc.eos_r0, oc.eos_q = s["cs0"], s["r0"], s["q"]
        oc.central_mass, oc.constant_G = s["M"], s["G"]
    if s.get("av") == "cd10":
        oc.av_kind, oc.alpha_min, oc.alpha_max, oc.sigma_decay = 1, 0.0, 1.0, 0.1
    oc.bmin[:] = list(s["box_min"])
    oc.bmax[:] = list(s["box_max"])
    return oc


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else the machine type)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform

    return platform.machine()


def cpu_baseline(s, seconds, threads=None, alpha_AV=1.0, first_step=None):
    """FP64 oracle (OpenMP) on the same workload, bounded to about `seconds`.  first_step:
    a dict that receives the set-up and the oracle's state after its first (untimed,
    dt = 0) step, for the parity check against the GPU."""
    from oracle import oracle as O

    if threads:
        O.set_threads(threads)
    cores = O.get_threads()
    s, what = cpu_sample(s)
    oc = oracle_config(O, s, alpha_AV)
    sim = O.Sim(oc, s["pos"], s["vel"], s["h"], s["u"])
    log0 = sim.evolve_once()  # dt = 0 step (h convergence, first CFL), untimed
    if first_step is not None:
        first_step.update(setup=s, what=what, log=log0, state=sim.get(),
                          av=sim.get_av() if s.get("av") == "cd10" else None)
    n = len(s["h"])
    t0 = time.time()
    steps = 0
    while True:
        ostep(sim, s)
        steps += 1
        if time.time() - t0 >= seconds:
            break
    el = time.time() - t0
    return {"value": n * steps / el, "unit": UNIT, "cores": cores, "kind": "port",
            "cpu_model": cpu_model(),
            "sample": f"{steps} FP64 oracle steps of {what} ({n} particles) after one "
                      f"untimed dt=0 step, {el:.1f} s, OpenMP {cores} threads"}


def cpu_sample(s):
    """The CPU arms time the full workload, except the 33.8M-particle homogeneous box (one
    oracle step of it takes minutes): there the same set-up at 2^20 target particles."""
    if s.get("dt_zero"):
        return homogeneous_setup(1 << 20), "the same homogeneous set-up at 2^20 target particles"
    return s, "the full workload"


def run_reference(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if not reference_rank_runs(world, rank):
        return 0
    s, name, alpha_av = workload(args.cells, args.workload, args.n_target)
    from oracle import oracle as O

    O.set_threads(os.cpu_count())
    cores = O.get_threads()
    s, what = cpu_sample(s)
    oc = oracle_config(O, s, alpha_av)
    sim = O.Sim(oc, s["pos"], s["vel"], s["h"], s["u"])
    n = len(s["h"])
    # the requested untimed warm-up steps (at least one: the first step converges h)
    warm = max(1, args.warmup)
    for _ in range(warm):
        ostep(sim, s)
    budget = 150.0
    t0 = time.time()
    steps = 0
    while steps < args.steps:
        ostep(sim, s)
        steps += 1
        if time.time() - t0 > budget:
            break
    el = time.time() - t0
    value = n * steps / el
    sample = (f"{steps} of {args.steps} requested FP64 steps of {what} ({n} particles; "
              f"stopped at a {budget:.0f} s budget if reached), after "
              f"{warm} untimed warm-up steps")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": steps, "warmup": warm, "ms_per_step": el / steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": name, "precision": "fp64", "particles": n,
                       "implementation": "FP64 CPU restatement of the reference path (oracle/, "
                                         "OpenMP); the reference itself needs a SYCL compiler"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "cpu_model": cpu_model(), "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def precision_control(logs):
    """Which tier the timed steps ran in and the FP32 tier's estimated errors."""
    n = max(len(logs), 1)
    return {"steps_fp32": sum(1 for g in logs if g["tier"] == 1),
            "steps_compensated": sum(1 for g in logs if g["tier"] == 2),
            "steps_fp64": sum(1 for g in logs if g["tier"] == 0),
            "reruns": sum(int(g["tier_reruns"]) for g in logs),
            "estimate_refreshes": sum(int(g.get("est_refreshed", 1)) for g in logs),
            "compensated_fraction": sum(1 for g in logs if g["tier"] == 2) / n,
            "fp32_err_est_max": {"a": max(g["err_est_a"] for g in logs) if logs else None,
                                 "du_dt": max(g["err_est_du"] for g in logs) if logs else None},
            "definition": "tier per timed step (error-controlled mixed precision: FP32 pair "
                          "arithmetic while the estimated error of the FP32 tier stays within "
                          "1e-5, else the compensated tier; a rerun recomputes a step that "
                          "started in FP32 compensated); estimates relative to each field's "
                          "largest magnitude, refreshed on every fourth step where they cannot "
                          "reach the tolerance in the steps between"}


def accuracy(s, alpha_AV=1.0, precision="mixed"):
    """Max / RMS relative error of rho, |a|, du/dt and v_sig-driven dt of one mixed step
    against one FP64 step from the same initial state (the first, dt = 0, step)."""
    import numpy as np

    res = {}
    d = {}
    for prec in ("fp64", precision):
        m = make_model(s, prec, alpha_AV=alpha_AV)
        m.evolve_once()
        d[prec] = m.collect_data()
    a, b = d[precision], d["fp64"]
    rho_a = s["pmass"] * (1.2 / a["hpart"]) ** 3
    rho_b = s["pmass"] * (1.2 / b["hpart"]) ** 3
    rel = np.abs(rho_a - rho_b) / rho_b
    res["rho"] = {"max": float(rel.max()), "rms": float(np.sqrt(np.mean(rel**2)))}
    for k, key in (("axyz", "a"), ("duint", "du_dt"), ("omega", "omega")):
        x, y = a[k], b[k]
        if x.ndim > 1:
            dx, ny = np.linalg.norm(x - y, axis=1), np.linalg.norm(y, axis=1)
        else:
            dx, ny = np.abs(x - y), np.abs(y)
        res[key] = {"max": float(dx.max() / ny.max()),
                    "rms": float(np.sqrt(np.mean(dx**2)) / np.sqrt(np.mean(ny**2)))}
    res["definition"] = ("one step from the same state, mixed vs FP64 GPU path (the FP64 path is "
                         "bit-identical to the FP64 oracle); rho per particle relative; a, du/dt, "
                         "omega normalised by the field's max magnitude (max) or rms (rms)")
    return res


PARITY_FIELDS = ("xyz", "vxyz", "axyz", "hpart", "uint", "duint", "omega")
PARITY_KEYS = ("n_ghost", "leaf_count", "cache_size", "h_subcycles", "h_iterations",
               "corrector_iters", "next_dt", "cfl_mult")


def oracle_parity(first, alpha_AV, precision):
    """The GPU's first step against the oracle's from the same initial state (the set-up
    the CPU leg timed: the full workload, or its 2^20-particle sample for the 33.8M
    homogeneous box).  FP64: every field and the step's bookkeeping bit for bit.  Mixed:
    max / RMS errors against the oracle (rho per particle, a, du/dt and Omega normalised
    by the field's largest magnitude) and the precision tier the step ran in."""
    import numpy as np

    s, o = first["setup"], first["state"]
    out = {"particles": int(len(s["h"])), "set_up": first["what"]}
    m64 = make_model(s, "fp64", alpha_AV=alpha_AV)
    l64 = m64.evolve_once()
    g = m64.collect_data()
    diff = [k for k in PARITY_FIELDS if not np.array_equal(g[k], o[k])]
    if first.get("av") is not None:
        diff += [k for k in ("alpha_AV", "soundspeed") if not np.array_equal(g[k], first["av"][k])]
    diff += ["log." + k for k in PARITY_KEYS if l64[k] != first["log"][k]]
    out["fp64_bitexact"] = not diff
    out["fp64_mismatches"] = diff
    # the largest difference of each mismatched field, relative to the field's largest
    # magnitude (e.g. the LP07 sound speed, whose power function the GPU and the host C
    # library each round in their own way)
    maxrel = {}
    for k in diff:
        if k.startswith("log."):
            continue
        x = np.asarray(g[k])
        y = np.asarray(o[k] if k in PARITY_FIELDS else first["av"][k])
        maxrel[k] = float(np.abs(x - y).max() / max(np.abs(y).max(), 1e-300))
    if maxrel:
        out["fp64_max_rel_diff"] = maxrel
    del m64
    mm = make_model(s, precision, alpha_AV=alpha_AV)
    lm = mm.evolve_once()
    d = mm.collect_data()
    err = {}
    rho_d, rho_o = s["pmass"] * (1.2 / d["hpart"]) ** 3, s["pmass"] * (1.2 / o["hpart"]) ** 3
    rel = np.abs(rho_d - rho_o) / rho_o
    err["rho"] = {"max": float(rel.max()), "rms": float(np.sqrt(np.mean(rel**2)))}
    for k, key in (("axyz", "a"), ("duint", "du_dt"), ("omega", "omega")):
        x, y = d[k], o[k]
        if x.ndim > 1:
            dx, ny = np.linalg.norm(x - y, axis=1), np.linalg.norm(y, axis=1)
        else:
            dx, ny = np.abs(x - y), np.abs(y)
        err[key] = {"max": float(dx.max() / ny.max()),
                    "rms": float(np.sqrt(np.mean(dx**2)) / np.sqrt(np.mean(ny**2)))}
    err["tier"] = int(lm["tier"])
    out["mixed_vs_oracle"] = err
    return out


def run_gb300(args):
    import numpy as np
    import torch

    world, rank, local, dist = dist_setup()
    torch.cuda.set_device(local)
    s, name, alpha_av = workload(args.cells, args.workload, args.n_target)
    n = len(s["h"])
    m = make_model(s, args.precision, device=local, alpha_AV=alpha_av)
    lib = m._lib()
    for _ in range(max(args.warmup, 3)):
        step(m, s)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    lib.profile(True)
    l0 = lib.lib.gbsph_kernel_launches()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    logs = []
    with ClockSampler(local) as clocks:
        e0.record(stream)
        for _ in range(args.steps):
            logs.append(step(m, s, stream=None))
        e1.record(stream)
        torch.cuda.synchronize()
    if dist:
        dist.barrier()
    launches = lib.lib.gbsph_kernel_launches() - l0
    prof = lib.profile_read()
    lib.profile(False)
    t_ms = e0.elapsed_time(e1)
    t_max = max_over_ranks(t_ms, dist, device="cuda")
    value = whole_job_rate(n, world, args.steps, t_max)
    clk = clocks.summary()

    # end-to-end through the public API with host buffers, every step:
    # pinned host -> device state copy, evolve_once, device -> pinned host state copy
    e2e = None
    if not args.no_e2e:
        d = m._to_device()
        names = ("xyz", "vxyz", "axyz", "hpart", "uint", "duint")
        if s.get("av") == "cd10":
            names = names + ("alpha_AV", "soundspeed")
        host = {k: torch.empty(d[k].shape, dtype=torch.float64, pin_memory=True) for k in names}
        for k in names:
            host[k].copy_(d[k])
        h2d = sum(host[k].numel() * 8 for k in names)
        steps_e2e = max(3, args.steps // 2)
        torch.cuda.synchronize()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        for _ in range(steps_e2e):
            for k in names:
                d[k].copy_(host[k], non_blocking=True)
            step(m, s)
            for k in names:
                host[k].copy_(d[k], non_blocking=True)
        f1.record(stream)
        torch.cuda.synchronize()
        te = max_over_ranks(f0.elapsed_time(f1), dist, device="cuda")
        e2e = {"value": whole_job_rate(n, world, steps_e2e, te), "unit": UNIT,
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": h2d, "steps": steps_e2e}

    if rank != 0:
        return 0
    log = logs[-1]
    rl = roofline(prof, log, n, args.precision, os.path.join(ROOT, "MEASURED_PEAKS.json"))
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": t_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "fp32-mixed" if args.precision.startswith("mixed") else "f64", "data": "synthetic",
        "config": {"workload": name, "precision": args.precision, "particles": n,
                   "ghosts": int(log["n_ghost"]), "leaves": int(log["leaf_count"]),
                   "cache_entries": int(log["cache_size"]),
                   "cache_entries_in_support": int(log.get("cache_kept") or log["cache_size"]),
                   "l2": "inputs larger than L2 (fields + neighbour cache ~%d MB per step)"
                         % ((int(log["cache_size"]) * 4 + n * 200) // 2**20),
                   "parallelism": f"replicas x{world}"},
        "gpu_launches": int(launches),
        "clocks": clk,
        "e2e": e2e,
        "roofline": rl,
        "step_log": {k: log[k] for k in ("h_subcycles", "h_iterations", "corrector_iters",
                                          "next_dt", "cfl_mult")},
        "precision_control": precision_control(logs),
    }
    if args.workload == "homogeneous" and args.n_target == 1 << 25:
        # the reference's own published figure for this set-up (FP64, varying CD10 AV,
        # 33,848,064 particles, one H100): examples/benchmarks/sph_homogeneous_bench_result.json
        line["published_reference"] = {
            "value": 25502056.0, "unit": UNIT, "hardware": "NVIDIA H100, DPC++, 1 rank",
            "precision": "fp64", "this_over_published": value / 25502056.0}
    if world == 1 and not args.no_accuracy:
        line["accuracy_mixed_vs_fp64"] = accuracy(s, alpha_AV=alpha_av, precision=args.precision)
        # FP64 GPU rate on the same workload (the x3 denominator), a few steps
        m64 = make_model(s, "fp64", alpha_AV=alpha_av)
        for _ in range(2):
            step(m64, s)
        torch.cuda.synchronize()
        g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        k64 = 3
        g0.record(stream)
        for _ in range(k64):
            step(m64, s)
        g1.record(stream)
        torch.cuda.synchronize()
        v64 = n * k64 / (g0.elapsed_time(g1) * 1e-3)
        line["fp64_gpu"] = {"value": v64, "unit": UNIT, "steps": k64}
        if args.precision.startswith("mixed"):
            line["mixed_over_fp64"] = value / v64
    if world == 1 and not args.no_adjoint:
        if args.workload == "disc":
            line["adjoint"] = adjoint_bench(steps=50, ck=5, precision=args.precision, device=local,
                                            workload="disc")
        elif args.workload == "homogeneous":
            line["adjoint"] = adjoint_bench(steps=20, ck=5, precision=args.precision, device=local,
                                            workload="homogeneous", n_target=args.n_target)
        else:
            line["adjoint"] = adjoint_bench(precision=args.precision, device=local)
    if world == 1 and not args.no_cpu_baseline:
        first = {}
        line["cpu_baseline"] = cpu_baseline(s, args.cpu_seconds, threads=os.cpu_count(),
                                            alpha_AV=alpha_av, first_step=first)
        if not args.no_accuracy:
            prec = args.precision if args.precision.startswith("mixed") else "mixed"
            line["parity_vs_oracle"] = oracle_parity(first, alpha_av, prec)
    print(json.dumps(line), flush=True)
    return 0


def adjoint_bench(steps=40, ck=5, precision="mixed", device=0, workload="soundwave",
                  n_target=1 << 22):
    """Adjoint / forward time of a differentiable rollout of `steps` steps with a
    checkpoint every `ck` steps; gradients with respect to initial v, u and alpha_AV.
    soundwave: 2^18 particles (simple cubic 64^3), density perturbation 1e-4 sin(2 pi x),
    gamma 1.0001, alpha_AV 0.1, loss = |v_final - v_target|^2 (seeded target).
    disc: the 4,194,304-particle Keplerian disc (locally isothermal EOS, central point
    mass, free boundary), alpha_AV 0.5, loss = total kinetic energy.  The backward time
    includes the recomputation between checkpoints."""
    import numpy as np
    import torch

    from shamrock_gb300 import adjoint, setups

    if workload == "disc":
        s = setups.keplerian_disc(4194304, seed=12345)
        alpha0 = 0.5
    elif workload == "homogeneous":
        # the reference's benchmark set-up with its varying (CD10) viscosity, advanced with
        # the CFL step; differentiated parameters: the switch's alpha_min and alpha_max
        s = dict(homogeneous_setup(n_target), dt_zero=False)
        alpha0 = [0.0, 1.0]
    else:
        s = setups.sound_wave(n_side=64, amp=1e-4, gamma=1.0001)
        alpha0 = 0.1
    m = make_model(s, precision, device, alpha_AV=0.0 if workload == "homogeneous" else alpha0)
    m.evolve_once()  # dt = 0: initial h, Omega, a, du
    d = m._to_device()
    n = d["hpart"].shape[0]
    rng = np.random.default_rng(12345)
    v_t = torch.as_tensor(1e-4 * rng.standard_normal((3, n)), device=d["vxyz"].device)
    v0 = d["vxyz"].clone().requires_grad_(True)
    u0 = d["uint"].clone().requires_grad_(True)
    alpha = torch.tensor(alpha0, dtype=torch.float64, requires_grad=True)

    def loss_of(v):
        # disc, homogeneous box: total kinetic energy; sound wave: distance to a seeded
        # target field
        if workload in ("disc", "homogeneous"):
            return 0.5 * s["pmass"] * (v * v).sum()
        return ((v - v_t) ** 2).sum()

    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    lib = m._lib()
    # untimed warm-up rollout + backward (lazy kernel loading, autograd worker thread)
    warm = adjoint._snapshot(m)
    t_w, dt_w, cm_w = m.time, m.dt, m.cfl_mult
    xw, vw, uw = adjoint.rollout(m, v0, u0, alpha, ck, ck)
    loss_of(vw).backward()
    v0.grad = u0.grad = alpha.grad = None
    adjoint._restore(m, warm)
    m.time, m.dt, m.cfl_mult = t_w, dt_w, cm_w
    torch.cuda.synchronize()
    ev[0].record()
    x, v, u = adjoint.rollout(m, v0, u0, alpha, steps, ck)
    ev[1].record()
    loss = loss_of(v)
    torch.cuda.synchronize()
    lib.profile(True)
    ev[2].record()
    loss.backward()
    ev[3].record()
    torch.cuda.synchronize()
    prof = lib.profile_read()
    lib.profile(False)
    f_ms, b_ms = ev[0].elapsed_time(ev[1]), ev[2].elapsed_time(ev[3])
    iters = [r[2] for r in adjoint.rollout.last_records]
    if workload == "disc":
        wname = ("keplerian_disc_4194304 (LP07, point mass, alpha_AV 0.5, free boundary); loss = "
                 "total kinetic energy")
    elif workload == "homogeneous":
        wname = ("homogeneous_hcp_box_%d (the reference's benchmark set-up, varying CD10 viscosity "
                 "alpha in [0, 1], CFL steps); loss = total kinetic energy; gradients with respect "
                 "to v0, u0, alpha_min, alpha_max" % n)
    else:
        wname = ("sound_wave_cubic_64^3 (N=%d, amp 1e-4, gamma 1.0001, alpha_AV 0.1, periodic); "
                 "loss = |v - v_target|^2" % n)
    return {"workload": wname,
            "precision": precision, "steps": steps, "checkpoint_every": ck,
            "forward_ms": f_ms, "backward_ms": b_ms, "adjoint_over_forward": b_ms / f_ms,
            "loss": float(loss.detach()),
            "grad_norm": {"v": float(v0.grad.norm()), "u": float(u0.grad.norm()),
                          "alpha": alpha.grad.tolist()},
            "corrector_iters": iters,
            "backward_stages_ms": {k: round(v[0], 3) for k, v in prof.items() if v[1]},
            "definition": "backward (recompute between checkpoints + reverse steps) / forward "
                          "(steps + checkpoint copies), CUDA events, same process, after one "
                          "untimed warm-up rollout + backward of checkpoint_every steps"}


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
