"""The allocation-free derivatives entry point, called through the C ABI.

Some callers may not allocate device memory at all (their own memory pool owns every
device byte, or the call sits in a loop that must not allocate), so they cannot hold
a library context.  gbsph_derivs_constAV_mixed_noalloc serves them from a fixed
device array compiled into the library.  Both entry points launch the same staging and
pair kernels on the same inputs, so its results must equal the context entry point
gbsph_derivs_constAV in mixed precision bit for bit, on two calls in a row, also with the
merged count at the array's limit; and, as every mixed-precision result, agree with the
oracle's FP64 derivatives within 1e-5 of the field's largest magnitude.
This file is collected last and needs nothing from the other test files.
"""

import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

MAX_MERGED = 1 << 16


def _scene():
    from oracle import oracle as O
    from shamrock_gb300 import setups

    s = setups.sedov_taylor(8, jitter=0.05, seed=11)
    rng = np.random.default_rng(2)
    n = len(s["h"])
    vel = rng.normal(0, 0.1, size=(n, 3))
    src, off = O.periodic_ghosts(s["pos"], s["h"], [0, 0, 0], [1, 1, 1], 1.1)
    mpos = np.concatenate([s["pos"], s["pos"][src] + off])
    mh = np.concatenate([s["h"], s["h"][src]])
    lo, hi = np.nextafter(mpos.min(0), -np.inf), np.nextafter(mpos.max(0), np.inf)
    csr = O.Tree(mpos, lo, hi, 3, h=mh, htol=1.1).neigh_cache(mpos, mh, n, 1.1)
    om = O.omega(csr, mpos, mh[:n], s["pmass"])
    m = lambda f: np.concatenate([f, f[src]])
    P, cs = O.eos_adiabatic(mh, m(s["u"]), s["pmass"], s["gamma"])
    return dict(n=n, N=len(mh), pmass=s["pmass"], csr=csr, pos=mpos, v=m(vel), h=mh, om=m(om),
                u=m(s["u"]), P=P, cs=cs)


def _dev(a, dtype=torch.float64):
    return torch.as_tensor(np.ascontiguousarray(a), device="cuda").to(dtype)


def _noalloc(lib, sc, csr_t, f, n=None, N=None):
    n = sc["n"] if n is None else n
    N = sc["N"] if N is None else N
    a = torch.full((3, max(n, 1)), -7.0, dtype=torch.float64, device="cuda")
    du = torch.full((max(n, 1),), -7.0, dtype=torch.float64, device="cuda")
    vs = torch.full((max(n, 1),), -7.0, dtype=torch.float64, device="cuda")
    p = lambda t: C.c_void_p(t.data_ptr())
    rc = lib.gbsph_derivs_constAV_mixed_noalloc(
        p(csr_t["cnt"]), p(csr_t["scanned"]), p(csr_t["entries"]), p(f["x"][0]), p(f["x"][1]),
        p(f["x"][2]), p(f["v"][0]), p(f["v"][1]), p(f["v"][2]), p(f["h"]), p(f["om"]), p(f["u"]),
        p(f["P"]), p(f["cs"]), n, N, sc["pmass"], 1.0, 1.0, 2.0, p(a[0]), p(a[1]), p(a[2]), p(du),
        p(vs), None)
    torch.cuda.synchronize()
    return rc, a, du, vs


def _norm_err(x, ref):
    x, ref = np.asarray(x), np.asarray(ref)
    return np.abs(x - ref).max() / np.abs(ref).max()


def _fields(sc, pad_to=None):
    """Merged fields on the device; pad_to appends particles that no cache entry names
    (far outside the box), so that only the staged count changes."""
    k = 0 if pad_to is None else pad_to - sc["N"]
    ext = lambda a, v: np.concatenate([a, np.full((k,) + a.shape[1:], v)]) if k else a
    return dict(x=_dev(ext(sc["pos"], 5.0).T), v=_dev(ext(sc["v"], 0.0).T), h=_dev(ext(sc["h"], 0.01)),
                om=_dev(ext(sc["om"], 1.0)), u=_dev(ext(sc["u"], 1.0)), P=_dev(ext(sc["P"], 1.0)),
                cs=_dev(ext(sc["cs"], 1.0)))


def test_noalloc_matches_context_entry_point():
    from oracle import oracle as O
    from shamrock_gb300 import _lib, modules

    assert torch.cuda.is_available(), "GPU test run without a CUDA device"
    lib = _lib.load()
    ctx = _lib.Context(0)
    sc = _scene()
    assert sc["N"] < MAX_MERGED
    csr_t = {k: _dev(sc["csr"][k].astype(np.int64), torch.int32) for k in ("cnt", "scanned", "entries")}
    f = _fields(sc)
    a_ref, du_ref, vs_ref = modules.derivs_constAV(
        ctx, csr_t, sc["pos"], sc["v"], sc["h"], sc["om"], sc["u"], sc["P"], sc["cs"], sc["pmass"],
        1.0, 1.0, 2.0, precision="mixed")
    a64, du64 = O.derivs_constAV(sc["csr"], sc["pos"], sc["v"], sc["h"], sc["om"], sc["u"], sc["P"],
                                 sc["cs"], sc["pmass"], 1.0, 1.0, 2.0)
    same = lambda x, ref: torch.equal(x.cpu(), ref.cpu())
    for call in range(2):  # two calls in a row share (and reuse) the fixed staging
        rc, a, du, vs = _noalloc(lib, sc, csr_t, f)
        assert rc == _lib.GBSPH_OK, (call, rc)
        assert same(a, a_ref) and same(du, du_ref) and same(vs, vs_ref), call
        assert _norm_err(a.cpu().numpy().T, a64) <= 1e-5, call
        assert _norm_err(du.cpu().numpy(), du64) <= 1e-5, call
    # the merged count at the array's limit: the staging fills the whole array
    rc, a, du, vs = _noalloc(lib, sc, csr_t, _fields(sc, pad_to=MAX_MERGED), N=MAX_MERGED)
    assert rc == _lib.GBSPH_OK
    assert same(a, a_ref) and same(du, du_ref) and same(vs, vs_ref)
    ctx.close()


def test_noalloc_argument_checks():
    from shamrock_gb300 import _lib

    lib = _lib.load()
    sc = _scene()
    csr_t = {k: _dev(sc["csr"][k].astype(np.int64), torch.int32) for k in ("cnt", "scanned", "entries")}
    f = _fields(sc)
    # beyond the fixed array: refused before any argument is used
    null = None
    rc = lib.gbsph_derivs_constAV_mixed_noalloc(*([null] * 14), 1, MAX_MERGED + 1, 1.0, 1.0, 1.0,
                                                 2.0, *([null] * 5), None)
    assert rc == _lib.GBSPH_ERR_CAPACITY
    # more rows than merged particles
    rc, a, du, vs = _noalloc(lib, sc, csr_t, f, n=sc["N"] + 1, N=sc["N"])
    assert rc == _lib.GBSPH_ERR_ARG
    assert bool((a == -7.0).all()) and bool((du == -7.0).all())
    # no rows: nothing to do, outputs untouched
    rc, a, du, vs = _noalloc(lib, sc, csr_t, f, n=0)
    assert rc == _lib.GBSPH_OK
    assert bool((a == -7.0).all()) and bool((du == -7.0).all()) and bool((vs == -7.0).all())
