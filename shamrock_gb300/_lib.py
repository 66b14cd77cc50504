"""ctypes binding of libgbsph.so (include/gbsph.h).

There is no CPU fallback: if the CUDA library cannot be loaded (or built with nvcc
for sm_103a) every entry point raises.
"""

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgbsph.so")

GBSPH_OK = 0
GBSPH_ERR_ARG = 1
GBSPH_ERR_CUDA = 2
GBSPH_ERR_CAPACITY = 3
GBSPH_ERR_NOT_CONVERGED = 4
GBSPH_ERR_STATE = 5
GBSPH_FP64 = 0
GBSPH_MIXED = 1
GBSPH_MIXED_COMPENSATED = 2
GBSPH_MIXED_GUARDED = 3
GBSPH_AV_CONSTANT = 0
GBSPH_AV_VARYING_CD10 = 1
GBSPH_AV_VARYING_MM97 = 2

_vp = C.c_void_p
_u32 = C.c_uint32
_u64 = C.c_uint64
_f64 = C.c_double
_d3 = C.c_double * 3


class Vec3(C.Structure):
    _fields_ = [("x", _vp), ("y", _vp), ("z", _vp), ("stride", _u32), ("pad", _u32)]


class Particles(C.Structure):
    _fields_ = [("n", _u32), ("pad", _u32), ("xyz", Vec3), ("vxyz", Vec3), ("axyz", Vec3),
                ("hpart", _vp), ("uint", _vp), ("duint", _vp), ("omega", _vp),
                ("alpha_AV", _vp), ("soundspeed", _vp), ("divv", _vp), ("curlv", Vec3),
                ("dtdivv", _vp)]


class Config(C.Structure):
    _fields_ = [("gamma", _f64), ("pmass", _f64), ("alpha_u", _f64), ("alpha_AV", _f64),
                ("beta_AV", _f64), ("cfl_cour", _f64), ("cfl_force", _f64),
                ("cfl_mult_stiffness", _f64), ("htol_up_coarse", _f64), ("htol_up_fine", _f64),
                ("epsilon_h", _f64), ("h_iter_per_subcycles", _u32), ("h_max_subcycles", _u32),
                ("tree_reduction_level", _u32), ("periodic", _u32), ("box_min", _d3),
                ("box_max", _d3), ("precision", _u32), ("pad", _u32),
                ("epsilon_h_particle", _f64), ("eos_kind", _u32), ("ext_kind", _u32),
                ("cs0", _f64), ("eos_r0", _f64), ("eos_q", _f64), ("central_mass", _f64),
                ("constant_G", _f64), ("av_kind", _u32), ("pad2", _u32), ("alpha_min", _f64),
                ("alpha_max", _f64), ("sigma_decay", _f64), ("mixed_tol", _f64),
                ("corrector_max_iters", _u32), ("pad3", _u32)]


class TimeState(C.Structure):
    _fields_ = [("t", _f64), ("dt", _f64), ("cfl_mult", _f64)]


class StepLog(C.Structure):
    _fields_ = [("t", _f64), ("dt", _f64), ("next_dt", _f64), ("cfl_mult", _f64),
                ("n_local", _u32), ("n_ghost", _u32), ("leaf_count", _u32), ("h_subcycles", _u32),
                ("h_iterations", _u32), ("corrector_iters", _u32), ("cache_size", _u64),
                ("eps_v", _f64), ("max_eps_h", _f64), ("elapsed_s", _f64), ("rate", _f64),
                ("tier", _u32), ("tier_reruns", _u32), ("err_est_a", _f64), ("err_est_du", _f64),
                ("cache_kept", _u64), ("est_refreshed", _u32), ("pad4", _u32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Cotangents(C.Structure):
    _fields_ = [("n", _u32), ("pad", _u32), ("gx", Vec3), ("gv", Vec3), ("ga", Vec3),
                ("gu", _vp), ("gdu", _vp), ("galpha", _vp), ("gsoundspeed", _vp),
                ("g_alpha_min", _f64), ("g_alpha_max", _f64), ("g_sigma_decay", _f64)]


_P = C.POINTER
SIGNATURES = {
    "gbsph_create": (C.c_int, [_P(_vp), C.c_int]),
    "gbsph_destroy": (None, [_vp]),
    "gbsph_last_error": (C.c_char_p, [_vp]),
    "gbsph_version": (C.c_char_p, []),
    "gbsph_morton_codes": (C.c_int, [_vp, _vp, _vp, _vp, _u32, _u32, _P(_f64), _P(_f64), C.c_int,
                                     _vp, _vp]),
    "gbsph_sort_by_key": (C.c_int, [_vp, _vp, _vp, _u32, C.c_int, _vp]),
    "gbsph_build_tree": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _u32, _P(_f64), _P(_f64), _u32, _f64,
                                   C.c_int, _u32, _vp]),
    "gbsph_tree_counts": (C.c_int, [_vp, _P(_u32), _P(_u32)]),
    "gbsph_tree_export": (C.c_int, [_vp] * 13 + [_vp]),
    "gbsph_tree_query": (C.c_int, [_vp, _vp, _vp, _vp, _u32, C.c_int, _f64, _vp, _vp, _u64,
                                   _P(_u64), _vp]),
    "gbsph_neighbour_cache": (C.c_int, [_vp, _u32, _f64, _u32, _vp]),
    "gbsph_cache_size": (C.c_int, [_vp, _P(_u64), _P(_u64)]),
    "gbsph_cache_export": (C.c_int, [_vp, _vp, _vp, _vp, _vp]),
    "gbsph_h_iterate": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _u32, _f64,
                                  _f64, _f64, _u32, _P(_f64), _P(_f64), _P(_u32), _vp]),
    "gbsph_omega": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _u32, _f64, _vp, _vp]),
    "gbsph_eos_adiabatic": (C.c_int, [_vp, _vp, _vp, _u32, _f64, _f64, _vp, _vp, _vp]),
    "gbsph_eos_locally_isothermal": (C.c_int, [_vp, Vec3, _vp, _u32, _f64, _f64, _f64, _f64, _vp,
                                               _vp, _vp]),
    "gbsph_derivs_constAV": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                       _vp, _vp, _vp, _vp, _u32, _u32, _f64, _f64, _f64, _f64,
                                       _u32, _vp, _vp, _vp, _vp, _vp, _vp]),
    "gbsph_derivs_constAV_mixed_noalloc": (C.c_int, [_vp] * 14 + [_u32, _u32, _f64, _f64, _f64,
                                                                   _f64] + [_vp] * 6),
    "gbsph_periodic_ghosts": (C.c_int, [_vp, Vec3, _vp, _u32, _P(_f64), _P(_f64), _f64, _P(_u32),
                                        _vp]),
    "gbsph_ghost_export": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "gbsph_evolve_once": (C.c_int, [_vp, _P(Particles), _P(Config), _P(TimeState), _P(StepLog),
                                    _vp]),
    "gbsph_kdk_predict": (C.c_int, [_vp, _P(Particles), _f64, _u32, _P(_f64), _P(_f64), _vp]),
    "gbsph_kdk_correct": (C.c_int, [_vp, _P(Particles), Vec3, _vp, _f64, _P(_f64), _vp]),
    "gbsph_cfl": (C.c_int, [_vp, _vp, _vp, Vec3, _u32, _f64, _f64, _vp, _P(_f64), _vp]),
    "gbsph_adjoint_step": (C.c_int, [_vp, _P(Particles), _P(Config), _f64, _f64, _u32,
                                     _P(Cotangents), _P(_f64), _vp]),
    "gbsph_adjoint_record": (C.c_int, [_vp, _P(Particles), _P(Config), _f64, _f64, _u32,
                                       _P(Particles), _vp]),
    "gbsph_adjoint_reverse": (C.c_int, [_vp, _P(Particles), _P(Config), _f64, _P(Cotangents),
                                        _P(_f64), _vp]),
    "gbsph_profile_kinds": (_u32, []),
    "gbsph_kernel_launches": (_u64, []),
    "gbsph_set_cache_budget": (C.c_int, [_vp, _u64]),
    "gbsph_profile_name": (C.c_char_p, [_u32]),
    "gbsph_profile_enable": (C.c_int, [_vp, C.c_int]),
    "gbsph_profile_read": (C.c_int, [_vp, _vp, _vp, _vp, _u32]),
    "gbsph_conservation": (C.c_int, [_vp, _P(Particles), _f64, _P(_f64), _vp]),
}

_lib = None


class GbsphError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"gbsph error {code}: {msg}")
        self.code = code


def load(build_if_missing=True):
    """Load libgbsph.so, compiling it with nvcc first when it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise ImportError(f"{LIB_PATH} is missing: run `python -m shamrock_gb300.build`")
        from . import build as _build
        _build.build()
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def exported_symbols():
    return list(SIGNATURES)


def d3(v):
    return (_f64 * 3)(*[float(x) for x in v])


class Context:
    """Owns one gbsph_ctx (the library's scratch arena) on one device."""

    def __init__(self, device=0):
        self.lib = load()
        h = _vp()
        rc = self.lib.gbsph_create(C.byref(h), int(device))
        if rc != GBSPH_OK:
            raise GbsphError(rc, "gbsph_create failed (no CUDA device?)")
        self.handle = h
        self.device = device

    def check(self, rc):
        if rc != GBSPH_OK:
            raise GbsphError(rc, self.lib.gbsph_last_error(self.handle).decode())
        return rc

    def call(self, name, *args):
        return self.check(getattr(self.lib, name)(self.handle, *args))

    def profile(self, on=True):
        self.check(self.lib.gbsph_profile_enable(self.handle, 1 if on else 0))

    def profile_read(self):
        """{stage: (ms, launches, units)} accumulated since profile(True)."""
        k = self.lib.gbsph_profile_kinds()
        ms = (C.c_double * k)()
        la = (C.c_uint64 * k)()
        un = (C.c_uint64 * k)()
        self.check(self.lib.gbsph_profile_read(self.handle, ms, la, un, k))
        return {self.lib.gbsph_profile_name(i).decode(): (ms[i], la[i], un[i]) for i in range(k)}

    def close(self):
        if getattr(self, "handle", None):
            self.lib.gbsph_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
