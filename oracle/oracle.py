"""ORACLE — TEST INFRASTRUCTURE ONLY.

ctypes/numpy wrapper around ``libgbsph_oracle.so`` (the FP64 CPU restatement of
the Shamrock SPH hot path in ``gbsph_oracle.cpp``).  Imported only by the test
suite, by ``__graft_entry__.smoke()`` and by the CPU-baseline leg of
``bench.py`` — as the checker, never as the measured or shipped path.
"""

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgbsph_oracle.so")

_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C")
_u64p = np.ctypeslib.ndpointer(np.uint64, flags="C")
_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C")
_vp = C.c_void_p


class OrcConfig(C.Structure):
    """Mirror of orc::Config (gbsph_oracle.cpp)."""
    _fields_ = [
        ("gamma", C.c_double), ("pmass", C.c_double),
        ("alpha_u", C.c_double), ("alpha_AV", C.c_double), ("beta_AV", C.c_double),
        ("cfl_cour", C.c_double), ("cfl_force", C.c_double), ("cfl_mult_stiffness", C.c_double),
        ("htol_up_coarse", C.c_double), ("htol_up_fine", C.c_double),
        ("epsilon_h", C.c_double),
        ("h_iter_per_subcycles", C.c_uint32), ("h_max_subcycles", C.c_uint32),
        ("tree_reduction_level", C.c_uint32), ("periodic", C.c_uint32),
        ("bmin", C.c_double * 3), ("bmax", C.c_double * 3),
        ("eos_kind", C.c_uint32), ("ext_kind", C.c_uint32),
        ("cs0", C.c_double), ("eos_r0", C.c_double), ("eos_q", C.c_double),
        ("central_mass", C.c_double), ("constant_G", C.c_double),
        ("av_kind", C.c_uint32), ("pad", C.c_uint32),
        ("alpha_min", C.c_double), ("alpha_max", C.c_double), ("sigma_decay", C.c_double),
    ]


class OrcStepLog(C.Structure):
    """Mirror of orc::StepLog."""
    _fields_ = [
        ("t", C.c_double), ("dt", C.c_double), ("next_dt", C.c_double), ("cfl_mult", C.c_double),
        ("n_local", C.c_uint32), ("n_ghost", C.c_uint32), ("leaf_count", C.c_uint32),
        ("h_subcycles", C.c_uint32), ("h_iterations", C.c_uint32), ("corrector_iters", C.c_uint32),
        ("cache_size", C.c_uint64), ("eps_v", C.c_double), ("max_eps_h", C.c_double),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def build(force=False):
    """Compile the oracle with its Makefile (seconds)."""
    srcs = [os.path.join(HERE, f) for f in ("gbsph_oracle.cpp", "Makefile")]
    if force or not os.path.exists(LIB_PATH) or (
            os.path.getmtime(LIB_PATH) < max(os.path.getmtime(f) for f in srcs)):
        subprocess.check_call(["make", "-s", "-C", HERE])


_lib = None


def lib():
    global _lib
    if _lib is not None:
        return _lib
    build()
    L = C.CDLL(LIB_PATH)
    sig = {
        "orc_set_threads": (None, [C.c_int]),
        "orc_get_threads": (C.c_int, []),
        "orc_morton32": (None, [_f64p, C.c_uint32, C.c_uint32, _f64p, _f64p, _u32p]),
        "orc_morton64": (None, [_f64p, C.c_uint32, C.c_uint32, _f64p, _f64p, _u64p]),
        "orc_bitonic32": (None, [_u32p, _u32p, C.c_uint32]),
        "orc_bitonic64": (None, [_u64p, _u32p, C.c_uint32]),
        "orc_bitonic32_stencil16": (None, [_u32p, _u32p, C.c_uint32]),
        "orc_bitonic64_stencil16": (None, [_u64p, _u32p, C.c_uint32]),
        "orc_reduce32": (C.c_uint32, [_u32p, C.c_uint32, C.c_uint32, _u32p]),
        "orc_reduce64": (C.c_uint32, [_u64p, C.c_uint32, C.c_uint32, _u32p]),
        "orc_karras32": (None, [_u32p, C.c_uint32, _u32p, _u32p, _u8p, _u8p, _u32p]),
        "orc_karras64": (None, [_u64p, C.c_uint32, _u32p, _u32p, _u8p, _u8p, _u32p]),
        "orc_tree_build": (_vp, [_f64p, _vp, C.c_uint32, _f64p, _f64p, C.c_uint32, C.c_int,
                                 C.c_double, C.c_uint32]),
        "orc_tree_free": (None, [_vp]),
        "orc_tree_leaf_count": (C.c_uint32, [_vp]),
        "orc_tree_morton_count": (C.c_uint32, [_vp]),
        "orc_tree_export": (None, [_vp] + [_vp] * 12),
        "orc_tree_query": (C.c_uint64, [_vp, _f64p, C.c_uint32, C.c_int, C.c_double, _vp, _vp]),
        "orc_cache_build": (_vp, [_vp, _f64p, _f64p, C.c_uint32, C.c_double]),
        "orc_cache_free": (None, [_vp]),
        "orc_cache_total": (C.c_uint64, [_vp]),
        "orc_cache_leaf_total": (C.c_uint64, [_vp]),
        "orc_cache_export": (None, [_vp] * 8),
        "orc_h_iterate_once": (None, [C.c_uint32, _u32p, _u32p, _u32p, _f64p, _f64p, _f64p, _f64p,
                                      C.c_double, C.c_double, C.c_double]),
        "orc_omega": (None, [C.c_uint32, _u32p, _u32p, _u32p, _f64p, _f64p, C.c_double, _f64p]),
        "orc_eos_adiabatic": (None, [C.c_uint32, _f64p, _f64p, C.c_double, C.c_double, _f64p,
                                     _f64p]),
        "orc_derivs_constAV": (None, [C.c_uint32, _u32p, _u32p, _u32p, _f64p, _f64p, _f64p, _f64p,
                                      _f64p, _f64p, _f64p, C.c_double, C.c_double, C.c_double,
                                      C.c_double, _f64p, _f64p]),
        "orc_vsig": (None, [C.c_uint32, _u32p, _u32p, _u32p, _f64p, _f64p, _f64p, _f64p, _f64p]),
        "orc_cfl": (C.c_double, [C.c_uint32, _f64p, _f64p, _f64p, C.c_double, C.c_double, _vp]),
        "orc_eos_locally_isothermal": (None, [C.c_uint32, _f64p, _f64p, C.c_double, C.c_double,
                                              C.c_double, C.c_double, _f64p, _f64p]),
        "orc_predict": (None, [C.c_uint32, _f64p, _f64p, _f64p, _f64p, _f64p, C.c_double,
                               C.c_uint32, _f64p, _f64p]),
        "orc_correct": (C.c_double, [C.c_uint32, _f64p, _f64p, _f64p, _f64p, _f64p, _f64p,
                                     C.c_double]),
        "orc_periodic_ghosts": (C.c_uint32, [C.c_uint32, _f64p, _f64p, _f64p, _f64p, C.c_double,
                                             _vp, _vp, C.c_uint32]),
        "orc_sim_create": (_vp, [C.POINTER(OrcConfig), C.c_uint32, _f64p, _f64p, _f64p, _f64p]),
        "orc_sim_free": (None, [_vp]),
        "orc_sim_set_time": (None, [_vp, C.c_double, C.c_double, C.c_double]),
        "orc_sim_get_time": (None, [_vp, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                    C.POINTER(C.c_double)]),
        "orc_sim_set_derivs": (None, [_vp, _f64p, _f64p]),
        "orc_sim_evolve_once": (None, [_vp, C.POINTER(OrcStepLog)]),
        "orc_sim_get": (None, [_vp] + [_vp] * 7),
        "orc_sim_set_av": (None, [_vp, _vp, _vp]),
        "orc_sim_get_av": (None, [_vp] + [_vp] * 5),
        "orc_sim_ghost_count": (C.c_uint32, [_vp]),
        "orc_sim_ghosts": (None, [_vp, _u32p, _f64p]),
        "orc_sim_cache": (_vp, [_vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a if shape is None else a.reshape(shape)


def set_threads(n):
    lib().orc_set_threads(int(n))


def get_threads():
    return lib().orc_get_threads()


# --------------------------------------------------------------------------- modules
def morton_codes(pos, bmin, bmax, morton_count=None, key_bits=32):
    pos = _f64(pos, (-1, 3))
    n = pos.shape[0]
    mc = n if morton_count is None else morton_count
    if key_bits == 64:
        out = np.zeros(mc, np.uint64)
        lib().orc_morton64(pos, n, mc, _f64(bmin), _f64(bmax), out)
    else:
        out = np.zeros(mc, np.uint32)
        lib().orc_morton32(pos, n, mc, _f64(bmin), _f64(bmax), out)
    return out


def bitonic_sort(keys, vals=None, stencil16=False):
    keys = np.array(keys, copy=True)
    vals = np.arange(len(keys), dtype=np.uint32) if vals is None else np.array(vals, np.uint32)
    if keys.dtype == np.uint64:
        (lib().orc_bitonic64_stencil16 if stencil16 else lib().orc_bitonic64)(keys, vals, len(keys))
    else:
        keys = keys.astype(np.uint32)
        (lib().orc_bitonic32_stencil16 if stencil16 else lib().orc_bitonic32)(keys, vals, len(keys))
    return keys, vals


def reduce_morton(sorted_keys, cnt, level):
    out = np.zeros(cnt + 2, np.uint32)
    if sorted_keys.dtype == np.uint64:
        L = lib().orc_reduce64(np.ascontiguousarray(sorted_keys), cnt, level, out)
    else:
        L = lib().orc_reduce32(np.ascontiguousarray(sorted_keys, np.uint32), cnt, level, out)
    return out[:L + 2].copy(), L


def karras(keys):
    L = len(keys)
    I = max(L - 1, 0)
    lc, rc, er = (np.zeros(I, np.uint32) for _ in range(3))
    lf, rf = np.zeros(I, np.uint8), np.zeros(I, np.uint8)
    if keys.dtype == np.uint64:
        lib().orc_karras64(np.ascontiguousarray(keys), L, lc, rc, lf, rf, er)
    else:
        lib().orc_karras32(np.ascontiguousarray(keys, np.uint32), L, lc, rc, lf, rf, er)
    return dict(lchild_id=lc, rchild_id=rc, lchild_flag=lf, rchild_flag=rf, endrange=er)


class Tree:
    """CompressedLeafBVH built by the oracle (positions AoS (n,3))."""

    def __init__(self, pos, bmin, bmax, level, key_bits=32, h=None, htol=1.1, morton_count=0):
        self.pos = _f64(pos, (-1, 3))
        self.n = self.pos.shape[0]
        hh = None if h is None else _f64(h)
        self._h = hh
        self.handle = lib().orc_tree_build(self.pos, _ptr(hh), self.n, _f64(bmin), _f64(bmax),
                                           level, key_bits, htol, morton_count)
        L = lib().orc_tree_leaf_count(self.handle)
        P = lib().orc_tree_morton_count(self.handle)
        I, T = L - 1, 2 * L - 1
        self.leaf_count, self.morton_count = L, P
        self.sorted_keys = np.zeros(P, np.uint64)
        self.sort_index = np.zeros(P, np.uint32)
        self.reduc = np.zeros(L + 2, np.uint32)
        self.reduced = np.zeros(L, np.uint64)
        self.lchild_id, self.rchild_id, self.endrange = (np.zeros(I, np.uint32) for _ in range(3))
        self.lchild_flag, self.rchild_flag = np.zeros(I, np.uint8), np.zeros(I, np.uint8)
        self.aabb_min, self.aabb_max = np.zeros((T, 3)), np.zeros((T, 3))
        self.rint = np.zeros(T)
        lib().orc_tree_export(self.handle, *[_ptr(a) for a in (
            self.sorted_keys, self.sort_index, self.reduc, self.reduced, self.lchild_id,
            self.rchild_id, self.lchild_flag, self.rchild_flag, self.endrange, self.aabb_min,
            self.aabb_max, self.rint)])

    def query(self, mode, s=0.0, points=None):
        pts = self.pos if points is None else _f64(points, (-1, 3))
        counts = np.zeros(len(pts), np.uint32)
        tot = lib().orc_tree_query(self.handle, pts, len(pts), mode, s, _ptr(counts), None)
        out = np.zeros(tot, np.uint32)
        lib().orc_tree_query(self.handle, pts, len(pts), mode, s, _ptr(counts), _ptr(out))
        return counts, out

    def neigh_cache(self, pos_merged, h_merged, n_local, htol):
        c = lib().orc_cache_build(self.handle, _f64(pos_merged, (-1, 3)), _f64(h_merged),
                                  n_local, htol)
        try:
            tot = lib().orc_cache_total(c)
            ltot = lib().orc_cache_leaf_total(c)
            cnt, sc, own = (np.zeros(n_local, np.uint32) for _ in range(3))
            ent = np.zeros(tot, np.uint32)
            lc, ls = np.zeros(self.leaf_count, np.uint32), np.zeros(self.leaf_count, np.uint32)
            le = np.zeros(ltot, np.uint32)
            lib().orc_cache_export(c, *[_ptr(a) for a in (cnt, sc, ent, own, lc, ls, le)])
        finally:
            lib().orc_cache_free(c)
        return dict(cnt=cnt, scanned=sc, entries=ent, owner=own, leaf_cnt=lc, leaf_scanned=ls,
                    leaf_entries=le)

    def __del__(self):
        if getattr(self, "handle", None):
            lib().orc_tree_free(self.handle)
            self.handle = None


def csr_arrays(csr):
    return (np.ascontiguousarray(csr["cnt"], np.uint32),
            np.ascontiguousarray(csr["scanned"], np.uint32),
            np.ascontiguousarray(csr["entries"], np.uint32))


def h_iterate_once(csr, pos, h_old, h_new, eps, pmass, h_evol_max, h_evol_iter_max):
    """In place on h_new/eps (float64 arrays)."""
    cnt, sc, ent = csr_arrays(csr)
    lib().orc_h_iterate_once(len(cnt), cnt, sc, ent, _f64(pos, (-1, 3)), _f64(h_old), h_new, eps,
                             pmass, h_evol_max, h_evol_iter_max)


def omega(csr, pos, h, pmass):
    cnt, sc, ent = csr_arrays(csr)
    out = np.zeros(len(cnt))
    lib().orc_omega(len(cnt), cnt, sc, ent, _f64(pos, (-1, 3)), _f64(h), pmass, out)
    return out


def eos_adiabatic(h, u, pmass, gamma):
    h, u = _f64(h), _f64(u)
    P, cs = np.zeros(len(h)), np.zeros(len(h))
    lib().orc_eos_adiabatic(len(h), h, u, pmass, gamma, P, cs)
    return P, cs


def derivs_constAV(csr, pos, v, h, om, u, P, cs, pmass, alpha_u, alpha_AV, beta_AV):
    cnt, sc, ent = csr_arrays(csr)
    n = len(cnt)
    a, du = np.zeros((n, 3)), np.zeros(n)
    lib().orc_derivs_constAV(n, cnt, sc, ent, _f64(pos, (-1, 3)), _f64(v, (-1, 3)), _f64(h),
                             _f64(om), _f64(u), _f64(P), _f64(cs), pmass, alpha_u, alpha_AV,
                             beta_AV, a, du)
    return a, du


def vsig(csr, pos, v, h, cs):
    cnt, sc, ent = csr_arrays(csr)
    out = np.zeros(len(cnt))
    lib().orc_vsig(len(cnt), cnt, sc, ent, _f64(pos, (-1, 3)), _f64(v, (-1, 3)), _f64(h), _f64(cs),
                   out)
    return out


def cfl(h, vsig_, a, C_cour, C_force):
    h = _f64(h)
    dtp = np.zeros(len(h))
    m = lib().orc_cfl(len(h), h, _f64(vsig_), _f64(a, (-1, 3)), C_cour, C_force, _ptr(dtp))
    return m, dtp


def eos_locally_isothermal(pos, h, pmass, cs0, r0, q):
    h = _f64(h)
    P, cs = np.zeros(len(h)), np.zeros(len(h))
    lib().orc_eos_locally_isothermal(len(h), _f64(pos, (-1, 3)), h, pmass, cs0, r0, q, P, cs)
    return P, cs


def predict(pos, v, u, a, du, dt, periodic, bmin, bmax):
    """Leapfrog predictor + periodic wrap; returns new (pos, v, u)."""
    pos, v, u = _f64(pos, (-1, 3)).copy(), _f64(v, (-1, 3)).copy(), _f64(u).copy()
    lib().orc_predict(len(u), pos, v, u, _f64(a, (-1, 3)), _f64(du), dt, int(periodic),
                      _f64(bmin), _f64(bmax))
    return pos, v, u


def correct(v, u, a_new, a_old, du_new, du_old, dt):
    """Leapfrog corrector; returns new (v, u) and eps_v."""
    v, u = _f64(v, (-1, 3)).copy(), _f64(u).copy()
    e = lib().orc_correct(len(u), v, u, _f64(a_new, (-1, 3)), _f64(a_old, (-1, 3)), _f64(du_new),
                          _f64(du_old), dt)
    return v, u, e


def periodic_ghosts(pos, h, bmin, bmax, htol):
    pos, h = _f64(pos, (-1, 3)), _f64(h)
    g = lib().orc_periodic_ghosts(len(h), pos, h, _f64(bmin), _f64(bmax), htol, None, None, 0)
    src, off = np.zeros(g, np.uint32), np.zeros((g, 3))
    lib().orc_periodic_ghosts(len(h), pos, h, _f64(bmin), _f64(bmax), htol, _ptr(src), _ptr(off), g)
    return src, off


# --------------------------------------------------------------------------- full step
class Sim:
    """FP64 oracle simulation: one patch, the reference's evolve_once sequence."""

    def __init__(self, cfg, pos, vel, h, u):
        self.cfg = cfg
        pos, vel = _f64(pos, (-1, 3)), _f64(vel, (-1, 3))
        self.n = pos.shape[0]
        self.handle = lib().orc_sim_create(C.byref(cfg), self.n, pos, vel, _f64(h), _f64(u))

    def set_time(self, t, dt, cfl_mult):
        lib().orc_sim_set_time(self.handle, t, dt, cfl_mult)

    def get_time(self):
        t, dt, m = C.c_double(), C.c_double(), C.c_double()
        lib().orc_sim_get_time(self.handle, C.byref(t), C.byref(dt), C.byref(m))
        return t.value, dt.value, m.value

    def set_derivs(self, a, du):
        lib().orc_sim_set_derivs(self.handle, _f64(a, (-1, 3)), _f64(du))

    def evolve_once(self):
        log = OrcStepLog()
        lib().orc_sim_evolve_once(self.handle, C.byref(log))
        return log.as_dict()

    def get(self):
        n = self.n
        d = dict(xyz=np.zeros((n, 3)), vxyz=np.zeros((n, 3)), hpart=np.zeros(n), uint=np.zeros(n),
                 axyz=np.zeros((n, 3)), duint=np.zeros(n), omega=np.zeros(n))
        lib().orc_sim_get(self.handle, *[_ptr(d[k]) for k in (
            "xyz", "vxyz", "hpart", "uint", "axyz", "duint", "omega")])
        return d

    def set_av(self, alpha=None, soundspeed=None):
        """Varying-AV state: per-particle alpha_AV and the stored sound speed."""
        a = None if alpha is None else _f64(alpha)
        c = None if soundspeed is None else _f64(soundspeed)
        lib().orc_sim_set_av(self.handle, None if a is None else _ptr(a),
                             None if c is None else _ptr(c))

    def get_av(self):
        """alpha_AV, soundspeed, and the last step's divv, curlv (n, 3), dtdivv."""
        n = self.n
        d = dict(alpha_AV=np.zeros(n), soundspeed=np.zeros(n), divv=np.zeros(n),
                 curlv=np.zeros((n, 3)), dtdivv=np.zeros(n))
        lib().orc_sim_get_av(self.handle, *[_ptr(d[k]) for k in (
            "alpha_AV", "soundspeed", "divv", "curlv", "dtdivv")])
        return d

    def ghosts(self):
        g = lib().orc_sim_ghost_count(self.handle)
        src, off = np.zeros(g, np.uint32), np.zeros((g, 3))
        lib().orc_sim_ghosts(self.handle, src, off)
        return src, off

    def __del__(self):
        if getattr(self, "handle", None):
            lib().orc_sim_free(self.handle)
            self.handle = None
