"""Module-level access to the GB300 kernels through the C ABI, on torch CUDA tensors.

Each function mirrors one reference module (see include/gbsph.h for the exact
reference interfaces replaced).  Positions are (3, N) float64 tensors
(structure of arrays); CSR caches use the reference ObjectCache layout.
"""

import ctypes as C

import numpy as np
import torch

from . import _lib as L


def _p(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _cuda(a, dtype):
    if isinstance(a, torch.Tensor):
        return a.to(device="cuda", dtype=dtype).contiguous()
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device="cuda")


def soa(pos):
    """Positions as a (3, N) float64 CUDA tensor.  Host arrays and lists are read as
    (N, 3) rows; torch tensors are taken to be (3, N) already."""
    if isinstance(pos, torch.Tensor):
        return pos.to(device="cuda", dtype=torch.float64).contiguous()
    a = np.asarray(pos, dtype=np.float64).reshape(-1, 3)
    return torch.as_tensor(np.ascontiguousarray(a.T), device="cuda")


_KEY = {32: torch.int32, 64: torch.int64}


def morton_codes(ctx, pos, bmin, bmax, morton_count=None, key_bits=32):
    x = soa(pos)
    n = x.shape[1]
    mc = n if morton_count is None else morton_count
    out = torch.empty(mc, dtype=_KEY[key_bits], device="cuda")
    ctx.call("gbsph_morton_codes", _p(x[0]), _p(x[1]), _p(x[2]), n, mc, L.d3(bmin), L.d3(bmax),
             key_bits, _p(out), None)
    torch.cuda.synchronize()
    return out


def unsigned(t, key_bits):
    """Reinterpret a signed key tensor as numpy unsigned."""
    a = t.cpu().numpy()
    return a.view(np.uint32 if key_bits == 32 else np.uint64)


def sort_by_key(ctx, keys, vals=None, key_bits=32):
    keys = keys.clone()
    vals = torch.arange(keys.shape[0], dtype=torch.int32, device="cuda") if vals is None \
        else vals.clone()
    ctx.call("gbsph_sort_by_key", _p(keys), _p(vals), keys.shape[0], key_bits, None)
    torch.cuda.synchronize()
    return keys, vals


class Tree:
    """CompressedLeafBVH built on the GPU; export() returns host numpy arrays."""

    def __init__(self, ctx, pos, bmin, bmax, level, h=None, htol=1.1, key_bits=32, morton_count=0):
        self.ctx = ctx
        self.key_bits = key_bits
        self.pos = soa(pos)
        self.h = None if h is None else _cuda(h, torch.float64)
        n = self.pos.shape[1]
        ctx.call("gbsph_build_tree", _p(self.pos[0]), _p(self.pos[1]), _p(self.pos[2]), _p(self.h),
                 n, L.d3(bmin), L.d3(bmax), level, htol, key_bits, morton_count, None)
        P, Lc = C.c_uint32(), C.c_uint32()
        ctx.call("gbsph_tree_counts", C.byref(P), C.byref(Lc))
        self.morton_count, self.leaf_count = P.value, Lc.value

    def export(self):
        P, Lc = self.morton_count, self.leaf_count
        I, T = Lc - 1, 2 * Lc - 1
        dev = dict(
            sorted_keys=torch.empty(P, dtype=_KEY[self.key_bits], device="cuda"),
            sort_index=torch.empty(P, dtype=torch.int32, device="cuda"),
            reduc=torch.empty(Lc + 2, dtype=torch.int32, device="cuda"),
            reduced=torch.empty(Lc, dtype=_KEY[self.key_bits], device="cuda"),
            lchild_id=torch.empty(max(I, 1), dtype=torch.int32, device="cuda"),
            rchild_id=torch.empty(max(I, 1), dtype=torch.int32, device="cuda"),
            lchild_flag=torch.empty(max(I, 1), dtype=torch.uint8, device="cuda"),
            rchild_flag=torch.empty(max(I, 1), dtype=torch.uint8, device="cuda"),
            endrange=torch.empty(max(I, 1), dtype=torch.int32, device="cuda"),
            aabb_min=torch.empty((T, 3), dtype=torch.float64, device="cuda"),
            aabb_max=torch.empty((T, 3), dtype=torch.float64, device="cuda"),
            rint=torch.empty(T, dtype=torch.float64, device="cuda"))
        self.ctx.call("gbsph_tree_export", *[_p(dev[k]) for k in (
            "sorted_keys", "sort_index", "reduc", "reduced", "lchild_id", "rchild_id",
            "lchild_flag", "rchild_flag", "endrange", "aabb_min", "aabb_max", "rint")], None)
        out = {}
        for k, v in dev.items():
            a = v.cpu().numpy()
            if k in ("sorted_keys", "reduced"):
                a = a.view(np.uint32 if self.key_bits == 32 else np.uint64)
            elif a.dtype == np.int32:
                a = a.view(np.uint32)
            if k in ("lchild_id", "rchild_id", "lchild_flag", "rchild_flag", "endrange"):
                a = a[:I]
            out[k] = a
        return out

    def query(self, mode, s=0.0, points=None):
        q = self.pos if points is None else soa(points)
        nq = q.shape[1]
        counts = torch.zeros(nq, dtype=torch.int32, device="cuda")
        tot = C.c_uint64()
        self.ctx.call("gbsph_tree_query", _p(q[0]), _p(q[1]), _p(q[2]), nq, mode, s, _p(counts),
                      None, 0, C.byref(tot), None)
        out = torch.zeros(max(tot.value, 1), dtype=torch.int32, device="cuda")
        self.ctx.call("gbsph_tree_query", _p(q[0]), _p(q[1]), _p(q[2]), nq, mode, s, _p(counts),
                      _p(out), tot.value, C.byref(tot), None)
        return counts.cpu().numpy().view(np.uint32), out[:tot.value].cpu().numpy().view(np.uint32)


def neighbour_cache(ctx, n_local, htol, precision="fp64"):
    """Two-stage cache over the last tree; returns the reference-layout CSR on the GPU.
    precision "mixed" pre-tests pairs in FP32 (the resulting cache is the same)."""
    ctx.call("gbsph_neighbour_cache", n_local, htol,
             L.GBSPH_MIXED if precision == "mixed" else L.GBSPH_FP64, None)
    tot, ltot = C.c_uint64(), C.c_uint64()
    ctx.call("gbsph_cache_size", C.byref(tot), C.byref(ltot))
    cnt = torch.empty(n_local, dtype=torch.int32, device="cuda")
    sc = torch.empty(n_local, dtype=torch.int32, device="cuda")
    ent = torch.empty(max(tot.value, 1), dtype=torch.int32, device="cuda")
    ctx.call("gbsph_cache_export", _p(cnt), _p(sc), _p(ent), None)
    return dict(cnt=cnt, scanned=sc, entries=ent[:tot.value])


def csr_to_cuda(csr):
    return {k: _cuda(np.asarray(v).astype(np.int64).astype(np.int32) if not isinstance(v, torch.Tensor)
                     else v, torch.int32) for k, v in csr.items()}


def h_iterate(ctx, csr, pos, h_old, h_new, eps, pmass, h_evol_max, h_evol_iter_max, iters=1):
    """In place on the CUDA tensors h_new / eps; returns (max_eps, min_eps, iters_used)."""
    x = soa(pos)
    mx, mn, used = C.c_double(), C.c_double(), C.c_uint32()
    ctx.call("gbsph_h_iterate", _p(csr["cnt"]), _p(csr["scanned"]), _p(csr["entries"]), _p(x[0]),
             _p(x[1]), _p(x[2]), _p(h_old), _p(h_new), _p(eps), csr["cnt"].shape[0], pmass,
             h_evol_max, h_evol_iter_max, iters, C.byref(mx), C.byref(mn), C.byref(used), None)
    return mx.value, mn.value, used.value


def omega(ctx, csr, pos, h, pmass):
    x = soa(pos)
    h = _cuda(h, torch.float64)
    n = csr["cnt"].shape[0]
    out = torch.empty(n, dtype=torch.float64, device="cuda")
    ctx.call("gbsph_omega", _p(csr["cnt"]), _p(csr["scanned"]), _p(csr["entries"]), _p(x[0]),
             _p(x[1]), _p(x[2]), _p(h), n, pmass, _p(out), None)
    return out


def eos_adiabatic(ctx, h, u, pmass, gamma):
    h, u = _cuda(h, torch.float64), _cuda(u, torch.float64)
    P, cs = torch.empty_like(h), torch.empty_like(h)
    ctx.call("gbsph_eos_adiabatic", _p(h), _p(u), h.shape[0], pmass, gamma, _p(P), _p(cs), None)
    return P, cs


def derivs_constAV(ctx, csr, pos, v, h, om, u, P, cs, pmass, alpha_u, alpha_AV, beta_AV,
                   precision="fp64", want_vsig=True):
    x, vv = soa(pos), soa(v)
    h, om, u, P, cs = (_cuda(a, torch.float64) for a in (h, om, u, P, cs))
    n = csr["cnt"].shape[0]
    N = x.shape[1]
    a = torch.empty((3, n), dtype=torch.float64, device="cuda")
    du = torch.empty(n, dtype=torch.float64, device="cuda")
    vs = torch.empty(n, dtype=torch.float64, device="cuda") if want_vsig else None
    ctx.call("gbsph_derivs_constAV", _p(csr["cnt"]), _p(csr["scanned"]), _p(csr["entries"]),
             _p(x[0]), _p(x[1]), _p(x[2]), _p(vv[0]), _p(vv[1]), _p(vv[2]), _p(h), _p(om), _p(u),
             _p(P), _p(cs), n, N, pmass, alpha_u, alpha_AV, beta_AV,
             L.GBSPH_MIXED if precision == "mixed" else L.GBSPH_FP64, _p(a[0]), _p(a[1]), _p(a[2]),
             _p(du), _p(vs), None)
    return a, du, vs


def periodic_ghosts(ctx, pos, h, bmin, bmax, htol):
    x = soa(pos)
    h = _cuda(h, torch.float64)
    n = x.shape[1]
    g = C.c_uint32()
    ctx.call("gbsph_periodic_ghosts", L.Vec3(x[0].data_ptr(), x[1].data_ptr(), x[2].data_ptr(), 1, 0),
             _p(h), n, L.d3(bmin), L.d3(bmax), htol, C.byref(g), None)
    G = g.value
    src = torch.zeros(max(G, 1), dtype=torch.int32, device="cuda")
    oid = torch.zeros(max(G, 1), dtype=torch.uint8, device="cuda")
    m = torch.empty((4, n + G), dtype=torch.float64, device="cuda")
    ctx.call("gbsph_ghost_export", _p(src), _p(oid), _p(m[0]), _p(m[1]), _p(m[2]), _p(m[3]), None)
    return dict(src=src[:G].cpu().numpy().view(np.uint32), offset_id=oid[:G].cpu().numpy(),
                merged_pos=m[:3].T.cpu().numpy(), merged_h=m[3].cpu().numpy())


def _vec3(t):
    return L.Vec3(t[0].data_ptr(), t[1].data_ptr(), t[2].data_ptr(), 1, 0)


def _particles(x, v, a, h, u, du):
    p = L.Particles()
    p.n = h.shape[0]
    p.xyz, p.vxyz, p.axyz = _vec3(x), _vec3(v), _vec3(a)
    p.hpart, p.uint, p.duint = h.data_ptr(), u.data_ptr(), du.data_ptr()
    p.omega = None
    return p


def kdk_predict(ctx, pos, v, u, a, du, dt, periodic=False, bmin=(0, 0, 0), bmax=(1, 1, 1)):
    """Leapfrog predictor + periodic wrap; returns new (pos (3, N), v (3, N), u)."""
    x, vv, aa = soa(pos).clone(), soa(v).clone(), soa(a)
    uu, dd = _cuda(u, torch.float64).clone(), _cuda(du, torch.float64)
    h = torch.zeros_like(uu)
    p = _particles(x, vv, aa, h, uu, dd)
    ctx.call("gbsph_kdk_predict", C.byref(p), dt, 1 if periodic else 0, L.d3(bmin), L.d3(bmax), None)
    return x, vv, uu


def kdk_correct(ctx, v, u, a_new, a_old, du_new, du_old, dt):
    """Leapfrog corrector; returns new (v (3, N), u) and eps_v."""
    vv, aa, ao = soa(v).clone(), soa(a_new), soa(a_old)
    uu, dd, do = (_cuda(t, torch.float64) for t in (u, du_new, du_old))
    uu = uu.clone()
    x = torch.zeros_like(vv)
    h = torch.zeros_like(uu)
    p = _particles(x, vv, aa, h, uu, dd)
    e = C.c_double()
    ctx.call("gbsph_kdk_correct", C.byref(p), _vec3(ao), _p(do), dt, C.byref(e), None)
    return vv, uu, e.value


def cfl(ctx, h, vsig, a, C_cour, C_force):
    """Per-particle CFL dt and its minimum."""
    h, vs, aa = _cuda(h, torch.float64), _cuda(vsig, torch.float64), soa(a)
    dtp = torch.empty_like(h)
    m = C.c_double()
    ctx.call("gbsph_cfl", _p(h), _p(vs), _vec3(aa), h.shape[0], C_cour, C_force, _p(dtp),
             C.byref(m), None)
    return m.value, dtp
