"""Python mirror of the reference's SPH model interface for the hot path.

Names, argument meaning and error behaviour follow the pybind11 module of the
reference (shammodels/sph/src/pySPHModel.cpp: get_Model_SPH :1725-1754, the
SolverConfig setters :107-262, model methods :773-1433), so that scripts written
for ``shamrock.get_Model_SPH(context=ctx, vector_type="f64_3", sph_kernel="M4")``
run unchanged on the subset the GB300 path covers: one patch, periodic or free
box, M4 kernel, constant or varying (CD10, MM97) artificial viscosity, adiabatic or
locally isothermal EOS, a central point mass, Phantom dump I/O.

Particle fields live on the GPU as float64 torch tensors in structure-of-arrays
layout; every step runs through the C ABI (``libgbsph.so``).  Setup helpers work
on host numpy arrays until the first step uploads them.
"""

import json
import math

import numpy as np

from . import _lib as L

# SolverConfig.precision -> gbsph_config.precision
PRECISION_CODES = {"fp64": L.GBSPH_FP64, "mixed": L.GBSPH_MIXED_GUARDED,
                   "mixed_fp32": L.GBSPH_MIXED, "mixed_compensated": L.GBSPH_MIXED_COMPENSATED}

FIELDS_VEC = ("xyz", "vxyz", "axyz")
FIELDS_SCAL = ("hpart", "uint", "duint")
# fields of the varying (CD10) viscosity: state alpha_AV and soundspeed, diagnostics
# divv, curlv, dtdivv (the reference adds them to the layout for that AV only)
FIELDS_AV_SCAL = ("alpha_AV", "soundspeed", "divv", "dtdivv")
FIELDS_AV_VEC = ("curlv",)
# the gravitational constant in SI (shamunits/Constants.hpp:130)
G_SI = 6.6743015e-11


class UnitSystem:
    """shamrock.UnitSystem (shamunits/UnitSystem.hpp:148-160, pyUnits.cpp:30-55): the SI
    value of one code unit of time, length and mass."""

    def __init__(self, unit_time=1.0, unit_length=1.0, unit_mass=1.0):
        self.unit_time = float(unit_time)
        self.unit_length = float(unit_length)
        self.unit_mass = float(unit_mass)

    def constant_G(self):
        """G in code units: G_SI M T^2 / L^3."""
        return G_SI * self.unit_mass * self.unit_time**2 / self.unit_length**3


class SolverConfig:
    """Hot-path subset of shammodels::sph::SolverConfig (SolverConfig.hpp)."""

    def __init__(self):
        self.gpart_mass = 0.0
        self.av = dict(type="constant", alpha_u=1.0, alpha_AV=1.0, beta_AV=2.0)
        self.boundary = "free"
        self.eos = None
        self.cfl_cour = 0.0
        self.cfl_force = 0.0
        self.cfl_multiplier_stiffness = 2.0
        self.tree_reduction_level = 3
        self.use_two_stage_search = True
        self.htol_up_coarse_cycle = 1.1
        self.htol_up_fine_cycle = 1.1
        self.epsilon_h = 1e-6
        self.epsilon_h_particle = 1e-6
        self.h_iter_per_subcycles = 50
        self.h_max_subcycles_count = 100
        self.precision = "fp64"
        self.mixed_tol = 0.0  # 0: the library's 1e-5
        # corrector evaluations before a step gives up (the reference's fixed 50; GB300
        # extension so that the give-up path can be exercised)
        self.corrector_max_iters = 50
        self.ext_forces = []
        # G without a unit system is the SI value, as the reference's get_constant_G
        self.constant_G = G_SI
        self.units = None

    # -- setters named as the reference's python bindings
    def set_artif_viscosity_Constant(self, alpha_u, alpha_AV, beta_AV):
        self.av = dict(type="constant", alpha_u=float(alpha_u), alpha_AV=float(alpha_AV),
                       beta_AV=float(beta_AV))

    def set_artif_viscosity_VaryingMM97(self, *, alpha_min, alpha_max, sigma_decay, alpha_u,
                                        beta_AV):
        """Morris & Monaghan (1997) switch (pySPHModel.cpp, UpdateViscosity.cpp:53-118)."""
        self.av = dict(type="mm97", alpha_min=float(alpha_min), alpha_max=float(alpha_max),
                       sigma_decay=float(sigma_decay), alpha_u=float(alpha_u),
                       beta_AV=float(beta_AV), alpha_AV=0.0)

    def set_artif_viscosity_VaryingCD10(self, *, alpha_min, alpha_max, sigma_decay, alpha_u,
                                        beta_AV):
        """Cullen & Dehnen (2010) switch (pySPHModel.cpp:171-186, UpdateViscosity.cpp)."""
        self.av = dict(type="cd10", alpha_min=float(alpha_min), alpha_max=float(alpha_max),
                       sigma_decay=float(sigma_decay), alpha_u=float(alpha_u),
                       beta_AV=float(beta_AV), alpha_AV=0.0)

    def set_boundary_periodic(self):
        self.boundary = "periodic"

    def set_boundary_free(self):
        self.boundary = "free"

    def set_eos_adiabatic(self, gamma):
        self.eos = dict(type="adiabatic", gamma=float(gamma))

    def set_eos_locally_isothermalLP07(self, cs0, q, r0):
        """c_s^2 = cs0^2 (R^2 / r0^2)^(-q), P = c_s^2 rho (pySPHModel.cpp:111-113)."""
        self.eos = dict(type="locally_isothermal_lp07", cs0=float(cs0), q=float(q), r0=float(r0))

    def add_ext_force_point_mass(self, central_mass, Racc):
        """Central point mass at the origin (SolverConfig::add_ext_force_point_mass).
        Accretion of particles inside Racc is not on the GB300 path: Racc must be 0."""
        if Racc != 0:
            raise ValueError("point-mass accretion is not on the GB300 path: use Racc=0")
        self.ext_forces.append(dict(type="point_mass", central_mass=float(central_mass)))

    def set_constant_G(self, G):
        """Gravitational constant in code units (GB300 extension; the reference derives it
        from the unit system, SI without one)."""
        self.constant_G = float(G)

    def set_units(self, units):
        """SolverConfig::set_units: the code's unit system; G follows it."""
        self.units = units
        self.constant_G = units.constant_G()

    def set_particle_mass(self, pmass):
        self.gpart_mass = float(pmass)

    def set_tree_reduction_level(self, level):
        self.tree_reduction_level = int(level)

    def set_two_stage_search(self, enable):
        # the one- and two-stage searches produce the same pair set in the same order
        self.use_two_stage_search = bool(enable)

    def set_cfl_cour(self, v):
        self.cfl_cour = float(v)

    def set_cfl_force(self, v):
        self.cfl_force = float(v)

    def set_cfl_mult_stiffness(self, v):
        self.cfl_multiplier_stiffness = float(v)

    def set_smoothing_length_density_based(self):
        pass

    def set_epsilon_h(self, eps):
        """Global h-iteration convergence threshold (SolverConfig::epsilon_h)."""
        self.epsilon_h = float(eps)

    def set_epsilon_h_particle(self, eps):
        """Per-particle Newton threshold (1e-6 in the reference's kernel).  Lowering it
        together with epsilon_h converges h further (GB300 extension)."""
        self.epsilon_h_particle = float(eps)

    PRECISIONS = ("fp64", "mixed", "mixed_fp32", "mixed_compensated")

    def set_precision(self, precision, tol=None):
        """"fp64": bit-identical to the FP64 oracle.  "mixed": error-controlled mixed
        precision, FP32 pair arithmetic where the step's error estimate stays within
        ``tol`` (default 1e-5 of the largest acceleration and du/dt), the compensated
        tier where it does not.  "mixed_fp32": FP32 pair arithmetic without the control.
        "mixed_compensated": the compensated tier on every step (GB300 extensions)."""
        if precision not in self.PRECISIONS:
            raise ValueError("precision must be one of " + ", ".join(self.PRECISIONS))
        self.precision = precision
        if tol is not None:
            self.mixed_tol = float(tol)

    def has_field_alphaAV(self):
        return self.av["type"] in ("cd10", "mm97")

    def to_dict(self):
        d = dict(self.__dict__)
        if self.units is not None:
            d["units"] = dict(self.units.__dict__)
        return d

    def print_status(self):
        print(json.dumps(self.to_dict(), indent=1))


class Context:
    """Stand-in for shamrock.Context: holds the model attached to it."""

    def __init__(self, device=0):
        self.device = device
        self.model = None

    def pdata_layout_new(self):
        pass

    def collect_data(self):
        if self.model is None:
            raise RuntimeError("no model attached to this context")
        return self.model.collect_data()


def get_Model_SPH(context, vector_type="f64_3", sph_kernel="M4"):
    """shamrock.get_Model_SPH (pySPHModel.cpp:1725-1754)."""
    if vector_type != "f64_3":
        raise ValueError(f"unknown vector type {vector_type}: the SPH solver is instantiated "
                         "for f64_3 only (Solver.cpp:3276-3282)")
    if sph_kernel != "M4":
        raise ValueError(f"kernel {sph_kernel} is not on the GB300 path (M4 only)")
    m = Model(context)
    context.model = m
    return m


class Model:
    """shammodels::sph::Model<f64_3, M4> for one patch on one GB300."""

    def __init__(self, context):
        self.ctx_py = context
        self.cfg = SolverConfig()
        self.box_min = np.zeros(3)
        self.box_max = np.ones(3)
        self._host = {k: np.zeros((0, 3)) for k in FIELDS_VEC + FIELDS_AV_VEC}
        self._host.update({k: np.zeros(0) for k in FIELDS_SCAL + FIELDS_AV_SCAL})
        self._dev = None  # dict of torch tensors once uploaded
        self._omega = None
        self.time = 0.0
        self.dt = 0.0
        self.cfl_mult = 1e-2
        self.logs = []
        self._lib_ctx = None
        self.scheduler = (None, None)

    # ------------------------------------------------------------------ config
    def gen_default_config(self):
        return SolverConfig()

    def set_solver_config(self, cfg):
        self.cfg = cfg

    def get_solver_config(self):
        return self.cfg

    def init_scheduler(self, crit_split, crit_merge):
        self.scheduler = (crit_split, crit_merge)

    def resize_simulation_box(self, box_min, box_max):
        self.box_min = np.asarray(box_min, float)
        self.box_max = np.asarray(box_max, float)

    def set_particle_mass(self, pmass):
        self.cfg.set_particle_mass(pmass)

    def get_particle_mass(self):
        return self.cfg.gpart_mass

    def set_cfl_cour(self, v):
        self.cfg.set_cfl_cour(v)

    def set_cfl_force(self, v):
        self.cfg.set_cfl_force(v)

    def set_cfl_mult_stiffness(self, v):
        self.cfg.set_cfl_mult_stiffness(v)

    def get_hfact(self):
        return 1.2

    def rho_h(self, h):
        return self.cfg.gpart_mass * (self.get_hfact() / np.asarray(h)) ** 3

    def total_mass_to_part_mass(self, totmass):
        n = self.get_total_part_count()
        if n == 0:
            raise RuntimeError("no particles")
        return totmass / n

    # ------------------------------------------------------------------ particles (setup)
    def get_total_part_count(self):
        if self._dev is not None:
            return int(self._dev["hpart"].shape[0])
        return int(self._host["hpart"].shape[0])

    def push_particle(self, pos, hpart, upart):
        self._to_host()
        pos = np.asarray(pos, float).reshape(-1, 3)
        n = pos.shape[0]
        self._host["xyz"] = np.concatenate([self._host["xyz"], pos])
        self._host["vxyz"] = np.concatenate([self._host["vxyz"], np.zeros((n, 3))])
        self._host["axyz"] = np.concatenate([self._host["axyz"], np.zeros((n, 3))])
        self._host["hpart"] = np.concatenate([self._host["hpart"], np.asarray(hpart, float)])
        self._host["uint"] = np.concatenate([self._host["uint"], np.asarray(upart, float)])
        self._host["duint"] = np.concatenate([self._host["duint"], np.zeros(n)])
        for k in FIELDS_AV_SCAL:
            self._host[k] = np.concatenate([self._host[k], np.zeros(n)])
        self._host["curlv"] = np.concatenate([self._host["curlv"], np.zeros((n, 3))])

    def add_cube_fcc_3d(self, dr, box_min, box_max):
        """Close-packed lattice of the reference's add_particles_fcc
        (shammodels/common/include/shammodels/common/setup/generators.hpp:82-127), keeping
        the sites inside the half-open box; h = 2 dr (the reference pushes r_particle and the
        model later rescales by hfact)."""
        bmin = np.asarray(box_min, float)
        bmax = np.asarray(box_max, float)
        dim = (bmax - bmin) / np.array([2.0, math.sqrt(3.0), 2.0 * math.sqrt(6.0) / 3.0]) / dr
        ix, iy, iz = (int(math.ceil(v)) for v in dim)
        i, j, k = np.meshgrid(np.arange(ix), np.arange(iy), np.arange(iz), indexing="ij")
        i, j, k = i.ravel(), j.ravel(), k.ravel()
        pos = np.stack([2 * i + ((j + k) % 2),
                        math.sqrt(3.0) * (j + (1.0 / 3.0) * (k % 2)),
                        2 * math.sqrt(6.0) * k / 3.0], 1) * dr + bmin
        keep = np.all((pos >= bmin) & (pos < bmax), axis=1)
        pos = pos[keep]
        self.push_particle(pos, np.full(len(pos), 2 * dr), np.zeros(len(pos)))

    def set_particles(self, pos, vel=None, h=None, u=None, alpha=None):
        """Replace all particles (host arrays); h defaults to hfact*(m/rho=1)^(1/3); the
        varying-viscosity fields start at zero (alpha_AV = alpha if given), as the
        reference's zero-initialised fields."""
        pos = np.asarray(pos, float).reshape(-1, 3)
        n = pos.shape[0]
        self._dev = None
        self._host = dict(
            xyz=pos.copy(), vxyz=np.zeros((n, 3)) if vel is None else np.asarray(vel, float).copy(),
            axyz=np.zeros((n, 3)),
            hpart=np.full(n, 1.2 * (1.0 / n) ** (1 / 3)) if h is None else np.asarray(h, float).copy(),
            uint=np.zeros(n) if u is None else np.asarray(u, float).copy(), duint=np.zeros(n))
        for k in FIELDS_AV_SCAL:
            self._host[k] = np.zeros(n)
        self._host["curlv"] = np.zeros((n, 3))
        if alpha is not None:
            self._host["alpha_AV"] = np.broadcast_to(np.asarray(alpha, float), (n,)).copy()

    def _field_host(self, name):
        self._to_host()
        return self._host[name]

    def set_value_in_a_box(self, field_name, field_type, value, box_min, box_max, ivar=0):
        self._to_host()
        pos = self._host["xyz"]
        sel = np.all((pos >= np.asarray(box_min)) & (pos < np.asarray(box_max)), axis=1)
        self._host[field_name][sel] = value

    def add_kernel_value(self, field_name, field_type, value, center, h_ker):
        """Adds value * W_M4(|r - center|, h_ker) / W_M4(0, h_ker) ... as the reference's
        add_kernel_value: value times the normalised M4 kernel at each particle."""
        self._to_host()
        r = np.linalg.norm(self._host["xyz"] - np.asarray(center, float), axis=1)
        q = r / h_ker
        f = np.where(q < 1, 0.25 * (2 - q) ** 3 - (1 - q) ** 3, np.where(q < 2, 0.25 * (2 - q) ** 3, 0))
        self._host[field_name] += value * f / (math.pi * h_ker**3)

    def get_sum(self, field_name, field_type):
        self._to_host()
        return float(np.sum(self._host[field_name]))

    # ------------------------------------------------------------------ device data
    def _lib(self):
        if self._lib_ctx is None:
            self._lib_ctx = L.Context(self.ctx_py.device if self.ctx_py else 0)
        return self._lib_ctx

    def _to_device(self):
        import torch

        if self._dev is not None:
            return self._dev
        dev = torch.device("cuda", self.ctx_py.device if self.ctx_py else 0)
        d = {}
        for k in FIELDS_VEC + FIELDS_AV_VEC:
            d[k] = torch.as_tensor(np.ascontiguousarray(self._host[k].T), device=dev).contiguous()
        for k in FIELDS_SCAL + FIELDS_AV_SCAL:
            d[k] = torch.as_tensor(self._host[k], device=dev).contiguous()
        d["omega"] = torch.ones_like(d["hpart"])
        self._dev = d
        return d

    def _to_host(self):
        if self._dev is None:
            return
        for k in FIELDS_VEC + FIELDS_AV_VEC:
            self._host[k] = self._dev[k].T.cpu().numpy().copy()
        for k in FIELDS_SCAL + FIELDS_AV_SCAL:
            self._host[k] = self._dev[k].cpu().numpy().copy()
        self._omega = self._dev["omega"].cpu().numpy().copy()
        self._dev = None

    def get_field_tensor(self, name):
        """Device tensor of a field: (3, N) for vectors, (N,) for scalars (torch binding)."""
        return self._to_device()[name]

    def collect_data(self):
        """Host copy of the particle fields, keyed as the reference's ctx.collect_data()."""
        if self._dev is not None:
            out = {k: self._dev[k].T.cpu().numpy().copy() for k in FIELDS_VEC + FIELDS_AV_VEC}
            out.update({k: self._dev[k].cpu().numpy().copy() for k in FIELDS_SCAL + FIELDS_AV_SCAL})
            out["omega"] = self._dev["omega"].cpu().numpy().copy()
            return out
        out = {k: v.copy() for k, v in self._host.items()}
        if self._omega is not None:
            out["omega"] = self._omega.copy()
        return out

    def _particles_struct(self):
        d = self._to_device()
        n = d["hpart"].shape[0]
        p = L.Particles()
        p.n = n
        for k in FIELDS_VEC:
            t = d[k]
            v = L.Vec3(t[0].data_ptr(), t[1].data_ptr(), t[2].data_ptr(), 1, 0)
            setattr(p, k, v)
        p.hpart = d["hpart"].data_ptr()
        p.uint = d["uint"].data_ptr()
        p.duint = d["duint"].data_ptr()
        p.omega = d["omega"].data_ptr()
        if self.cfg.av["type"] in ("cd10", "mm97"):
            p.alpha_AV = d["alpha_AV"].data_ptr()
            p.soundspeed = d["soundspeed"].data_ptr()
            p.divv = d["divv"].data_ptr()
            p.dtdivv = d["dtdivv"].data_ptr()
            t = d["curlv"]
            p.curlv = L.Vec3(t[0].data_ptr(), t[1].data_ptr(), t[2].data_ptr(), 1, 0)
        return p

    def _config_struct(self, tier=None):
        """The C configuration; tier: a concrete precision tier (GBSPH_FP64, GBSPH_MIXED or
        GBSPH_MIXED_COMPENSATED) in place of the configured precision."""
        c = self.cfg
        if c.eos is None:
            raise RuntimeError("an equation of state must be set (set_eos_adiabatic or "
                               "set_eos_locally_isothermalLP07)")
        if len(c.ext_forces) > 1:
            raise RuntimeError("one external force (a point mass) at most on the GB300 path")
        if c.gpart_mass == 0:
            raise RuntimeError(f"invalid gpart_mass {c.gpart_mass}, this configuration can not "
                               "converge.\nPlease set it using either model.set_particle_mass(pmass)"
                               " or cfg.set_particle_mass(pmass)")
        s = L.Config()
        if c.eos["type"] == "adiabatic":
            s.gamma = c.eos["gamma"]
            s.eos_kind = 0
        else:
            s.gamma = 1.0
            s.eos_kind = 1
            s.cs0, s.eos_q, s.eos_r0 = c.eos["cs0"], c.eos["q"], c.eos["r0"]
        if c.ext_forces:
            s.ext_kind = 1
            s.central_mass = c.ext_forces[0]["central_mass"]
            s.constant_G = c.constant_G
        s.pmass = c.gpart_mass
        s.alpha_u, s.alpha_AV, s.beta_AV = c.av["alpha_u"], c.av["alpha_AV"], c.av["beta_AV"]
        if c.av["type"] in ("cd10", "mm97"):
            s.av_kind = L.GBSPH_AV_VARYING_CD10 if c.av["type"] == "cd10" else L.GBSPH_AV_VARYING_MM97
            s.alpha_min, s.alpha_max = c.av["alpha_min"], c.av["alpha_max"]
            s.sigma_decay = c.av["sigma_decay"]
        s.cfl_cour, s.cfl_force = c.cfl_cour, c.cfl_force
        s.cfl_mult_stiffness = c.cfl_multiplier_stiffness
        s.htol_up_coarse, s.htol_up_fine = c.htol_up_coarse_cycle, c.htol_up_fine_cycle
        s.epsilon_h = c.epsilon_h
        s.epsilon_h_particle = c.epsilon_h_particle
        s.h_iter_per_subcycles = c.h_iter_per_subcycles
        s.h_max_subcycles = c.h_max_subcycles_count
        s.tree_reduction_level = c.tree_reduction_level
        s.periodic = 1 if c.boundary == "periodic" else 0
        s.box_min = L.d3(self.box_min)
        s.box_max = L.d3(self.box_max)
        s.precision = PRECISION_CODES[c.precision] if tier is None else int(tier)
        s.mixed_tol = getattr(c, "mixed_tol", 0.0)
        s.corrector_max_iters = int(getattr(c, "corrector_max_iters", 50))
        return s

    # ------------------------------------------------------------------ time stepping
    def evolve_once(self, stream=None, tier=None):
        """Solver::evolve_once (Solver.cpp:1942-3272) on the GPU; returns the step log.
        tier: run this precision tier instead of the configured precision (a recompute of
        an error-controlled step, given its log's "tier")."""
        lib = self._lib()
        p = self._particles_struct()
        cfg = self._config_struct(tier)
        ts = L.TimeState(self.time, self.dt, self.cfl_mult)
        log = L.StepLog()
        import ctypes as C

        rc = lib.lib.gbsph_evolve_once(lib.handle, C.byref(p), C.byref(cfg), C.byref(ts),
                                       C.byref(log), stream)
        lib.check(rc)
        self.time, self.dt, self.cfl_mult = ts.t, ts.dt, ts.cfl_mult
        d = log.as_dict()
        # a step that completed with a warning (the h iteration not converged after the
        # last sub-cycle: the reference logs an error and carries on, Solver.cpp:1271-1273)
        note = lib.lib.gbsph_last_error(lib.handle)
        d["note"] = note.decode() if note else ""
        if d["note"]:
            import warnings

            warnings.warn("evolve_once: " + d["note"], RuntimeWarning)
        self.logs.append(d)
        return d

    def timestep(self):
        return self.evolve_once()

    def conservation_totals(self):
        """FP64 totals of the reference's ConservativeCheck: momentum sum m v, force sum
        m a, energy sum m (u + v^2/2) and its rate sum m (v.a + du/dt)."""
        import ctypes as C

        lib = self._lib()
        p = self._particles_struct()
        out = (C.c_double * 8)()
        lib.check(lib.lib.gbsph_conservation(lib.handle, C.byref(p), self.cfg.gpart_mass, out, None))
        return dict(momentum=np.array(out[0:3]), force=np.array(out[3:6]), energy=out[6],
                    energy_rate=out[7])

    def evolve_once_override_time(self, t_current, dt_input):
        self.time = float(t_current)
        self.dt = float(dt_input)
        self.evolve_once()
        return self.dt

    def evolve_until(self, target_time, niter_max=-1):
        it = 0
        while self.time < target_time:
            if niter_max >= 0 and it >= niter_max:
                return False
            if self.time + self.dt > target_time:
                self.dt = target_time - self.time
            self.evolve_once()
            it += 1
        return True

    def get_time(self):
        return self.time

    def get_dt(self):
        return self.dt

    def set_next_dt(self, dt):
        self.dt = float(dt)

    def set_time(self, t):
        self.time = float(t)

    def set_cfl_multipler(self, m):
        self.cfl_mult = float(m)

    def get_cfl_multipler(self):
        return self.cfl_mult

    def solver_logs_last_rate(self):
        return self.logs[-1]["rate"] if self.logs else 0.0

    def solver_logs_last_obj_count(self):
        return self.logs[-1]["n_local"] if self.logs else 0

    def solver_logs_step_count(self):
        return len(self.logs)

    # ------------------------------------------------------------------ analysis (FP64 totals)
    def get_kinetic_energy(self):
        d = self._to_device()
        v = d["vxyz"]
        return float(0.5 * self.cfg.gpart_mass * (v * v).sum().item())

    def get_total_momentum(self):
        d = self._to_device()
        return tuple((self.cfg.gpart_mass * d["vxyz"].sum(dim=1)).cpu().numpy().tolist())

    def get_thermal_energy(self):
        d = self._to_device()
        return float(self.cfg.gpart_mass * d["uint"].sum().item())

    # ------------------------------------------------------------------ Phantom dumps
    def gen_config_from_phantom_dump(self, dump, bypass_error=False):
        """Model::gen_config_from_phantom_dump (Model.cpp:1203-1222): particle mass from
        massoftype[0], C_cour and C_force, the EOS of the dump's ieos, the varying CD10
        viscosity (alpha in [0, 1], sigma 0.1, the dump's alphau, beta 2), the dump's
        units, periodic boundaries when the header holds a box (xmin) and free ones
        otherwise."""
        from . import phantom as P

        cfg = SolverConfig()
        cfg.gpart_mass = dump.read_header_floats("massoftype")[0]
        cfg.cfl_cour = dump.read_header_float("C_cour")
        cfg.cfl_force = dump.read_header_float("C_force")
        cfg.eos = P.eos_config_from_dump(dump, bypass_error)
        cfg.set_artif_viscosity_VaryingCD10(alpha_min=0.0, alpha_max=1.0, sigma_decay=0.1,
                                            alpha_u=dump.read_header_float("alphau"), beta_AV=2.0)
        cfg.set_units(UnitSystem(unit_time=dump.read_header_float("utime"),
                                 unit_length=dump.read_header_float("udist"),
                                 unit_mass=dump.read_header_float("umass")))
        cfg.boundary = "periodic" if dump.has_header_entry("xmin") else "free"
        return cfg

    def init_from_phantom_dump(self, dump, hpart_fact_load=1.0):
        """Model::init_from_phantom_dump (Model.cpp:1225-1429) for one patch: the box from
        the header's xmin..zmax, else the particles' bounding box grown 1.2 times about its
        centre; the gas particles of block 0 inside the box with h >= 0 (Phantom marks
        accreted or dead particles with h < 0), in file order, h scaled by
        hpart_fact_load; u and alpha_AV when the dump holds them; the dump's time.  Sink
        particles (block 1) are not on the GB300 path: a dump holding any raises."""
        b0 = dump.blocks[0]
        x, y, z = (b0.fill_vec(k) for k in ("x", "y", "z"))
        if dump.has_header_entry("xmin"):
            bmin = np.array([dump.read_header_float(k) for k in ("xmin", "ymin", "zmin")])
            bmax = np.array([dump.read_header_float(k) for k in ("xmax", "ymax", "zmax")])
        else:
            lo = np.array([x.min(), y.min(), z.min()])
            hi = np.array([x.max(), y.max(), z.max()])
            center = (lo + hi) * 0.5
            d = (hi - lo) * 0.5 * 1.2
            bmin, bmax = center - d, center + d
        self.resize_simulation_box(bmin, bmax)
        if len(dump.blocks) > 1 and dump.blocks[1].tot_count > 0:
            raise NotImplementedError("sink particles are not on the GB300 path")
        h = b0.fill_vec("h")
        v = np.stack([b0.fill_vec(k) for k in ("vx", "vy", "vz")], 1)
        u = b0.fill_vec("u")
        alpha = b0.fill_vec("alpha")
        self.set_time(dump.read_header_float("time"))
        pos = np.stack([x, y, z], 1)
        keep = np.all((pos >= self.box_min) & (pos < self.box_max), axis=1) & (h >= 0)
        if keep.all():
            keep = slice(None)  # views: set_particles makes the one copy
        if v.size == 0:
            v = np.zeros((x.size, 3))
        self.set_particles(pos[keep], v[keep], h[keep] * hpart_fact_load,
                           u[keep] if u.size else None,
                           alpha=alpha[keep] if alpha.size else None)

    def make_phantom_dump(self):
        """Model::make_phantom_dump (Model.cpp:1491-1621): the header Phantom needs to
        restart (counts, EOS, time, dt, CFL, massoftype, the box when periodic, units)
        and block 0 with x, y, z, vx, vy, vz, u (real*8) and h, plus alpha and divv with a
        varying viscosity (real*4).

        Written as the reference writes them except ymax and zmax, which hold the box's
        upper y and z bounds (the reference stores its upper x bound in both, correct for
        cubic boxes only)."""
        from . import phantom as P

        c = self.cfg
        d = self.collect_data()
        n = int(d["hpart"].shape[0])
        dump = P.PhantomDump()
        dump.override_magic_number()
        dump.iversion = 1
        dump.fileid = f"{'FT:Phantom Shamrock writer':100s}"
        fi, i64, i32, fr, f64 = (dump.table_header_fort_int, dump.table_header_i64,
                                 dump.table_header_i32, dump.table_header_fort_real,
                                 dump.table_header_f64)
        for t in (fi, i64):
            t.add("nparttot", n)
            t.add("ntypes", 8)
            t.add("npartoftype", n)
            for _ in range(7):
                t.add("npartoftype", 0)
        for k, v in (("nblocks", 1), ("nptmass", 0), ("ndustlarge", 0), ("ndustsmall", 0),
                     ("idust", 7), ("idtmax_n", 1), ("idtmax_frac", 0), ("idumpfile", 0),
                     ("majorv", 2023), ("minorv", 0), ("microv", 0), ("isink", 0)):
            fi.add(k, v)
        i32.add("iexternalforce", 0)
        P.write_eos_in_dump(c.eos, dump)
        for k, v in (("time", self.time), ("dtmax", self.dt), ("rhozero", 0.0),
                     ("hfact", self.get_hfact()), ("tolh", 0.0001), ("C_cour", c.cfl_cour),
                     ("C_force", c.cfl_force), ("alpha", 0.0), ("alphau", 1.0), ("alphaB", 1.0)):
            fr.add(k, v)
        fr.add("massoftype", c.gpart_mass)
        for _ in range(7):
            fr.add("massoftype", 0.0)
        for k in ("Bextx", "Bexty", "Bextz", "dum"):
            fr.add(k, 0.0)
        if c.boundary == "periodic":
            for ax, k in enumerate("xyz"):
                fr.add(k + "min", float(self.box_min[ax]))
                fr.add(k + "max", float(self.box_max[ax]))
        for k, v in (("get_conserv", -1.0), ("etot_in", 0.59762), ("angtot_in", 0.0189694),
                     ("totmom_in", 0.0306284)):
            fr.add(k, v)
        P.write_units_in_dump(c.units, dump)
        blk = P.PhantomDumpBlock(n)
        for ax, k in enumerate("xyz"):
            blk.set_array("fort_real", k, d["xyz"][:, ax])
        blk.set_array("f32", "h", d["hpart"])
        if c.has_field_alphaAV():
            blk.set_array("f32", "alpha", d["alpha_AV"])
            blk.set_array("f32", "divv", d["divv"])
        for ax, k in enumerate(("vx", "vy", "vz")):
            blk.set_array("fort_real", k, d["vxyz"][:, ax])
        blk.set_array("fort_real", "u", d["uint"])
        dump.blocks.append(blk)
        return dump
