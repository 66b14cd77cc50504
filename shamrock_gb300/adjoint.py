"""Differentiable SPH rollout: a ``torch.autograd.Function`` over the C-ABI adjoint step.

The reference has no adjoint; this is the differentiable form of its step
(``Solver::evolve_once``, shammodels/sph/src/Solver.cpp:1942-3272) that the GB300 path adds.

``rollout(model, v0, u0, alpha, n_steps, checkpoint_every, dts=None)`` runs ``n_steps``
steps of ``model`` from its current positions, h, a and du with initial velocities
``v0`` (3, N), internal energies ``u0`` (N,) and the viscosity parameters ``alpha``, and
returns the final ``(x, v, u)``.  Gradients flow to ``v0``, ``u0``, ``alpha`` and the
initial positions ``x0`` when given.  ``alpha`` is alpha_AV (a scalar) for the constant
viscosity, and (alpha_min, alpha_max) for the varying ones (Cullen & Dehnen 2010, Morris &
Monaghan 1997), whose per-particle alpha_AV and stored sound speed are then part of the
state each step carries (their gradients, and that of sigma_decay, are kept in
``rollout.last_av_grads``).

What is differentiated: the step map with each step's dt, its number of corrector
evaluations and its neighbour cache held at the forward pass's values; h after each
step is the exact root of the density constraint (implicit differentiation).  The
forward pass records the dt sequence; pass it back as ``dts`` to replay the same map
(e.g. for finite-difference checks), since the CFL dt itself is not differentiated.

Memory: the state (x, v, a, h, u, du) is kept every ``checkpoint_every`` steps; the
backward pass recomputes each segment from its checkpoint once, each step with its tape
on a library context of its own (``gbsph_adjoint_record``: the context keeps the step's
tree, neighbour cache, h, Omega and tape, and the state after the step, which starts the
next one), then reverses the segment's steps in turn on those contexts
(``gbsph_adjoint_reverse``).  The model keeps ``checkpoint_every`` such contexts for
its later backward passes.  Past ``MAX_POOLED_PARTICLES`` particles times
``checkpoint_every`` the backward pass uses the model's own context alone: each segment's
start states rebuilt with plain steps, then each step recorded and reversed in turn.
"""

import ctypes as C

from . import _lib as L

STATE_KEYS = ("xyz", "vxyz", "axyz", "hpart", "uint", "duint")
AV_STATE_KEYS = ("alpha_AV", "soundspeed")


def _varying(model):
    return model.cfg.av["type"] in ("cd10", "mm97")


def _keys(model):
    return STATE_KEYS + (AV_STATE_KEYS if _varying(model) else ())


def _snapshot(model):
    d = model._to_device()
    return {k: d[k].clone() for k in _keys(model)}


def _restore(model, snap):
    d = model._to_device()
    for k in _keys(model):
        d[k].copy_(snap[k])


def _particles_of(snap):
    p = L.Particles()
    p.n = snap["hpart"].shape[0]
    for k in ("xyz", "vxyz", "axyz"):
        t = snap[k]
        setattr(p, k, L.Vec3(t[0].data_ptr(), t[1].data_ptr(), t[2].data_ptr(), 1, 0))
    p.hpart = snap["hpart"].data_ptr()
    p.uint = snap["uint"].data_ptr()
    p.duint = snap["duint"].data_ptr()
    p.omega = None
    if "alpha_AV" in snap:
        p.alpha_AV = snap["alpha_AV"].data_ptr()
        p.soundspeed = snap["soundspeed"].data_ptr()
    return p


def _cot_struct(cot):
    c = L.Cotangents()
    c.n = cot["gu"].shape[0]
    for name in ("gx", "gv", "ga"):
        t = cot[name]
        setattr(c, name, L.Vec3(t[0].data_ptr(), t[1].data_ptr(), t[2].data_ptr(), 1, 0))
    c.gu = cot["gu"].data_ptr()
    c.gdu = cot["gdu"].data_ptr()
    if "galpha" in cot:
        c.galpha = cot["galpha"].data_ptr()
        c.gsoundspeed = cot["gcs"].data_ptr()
    return c


def adjoint_step(model, start, t, dt, corrector_iters, cot, tier=None):
    """One reverse step (gbsph_adjoint_step): updates the cotangent dict ``cot`` in place
    from d/d(state after) to d/d(state before) and returns dL/d alpha_AV of the step.
    tier: the precision tier the forward step ran in (its log's "tier"; required when
    the configured precision is the error-controlled "mixed")."""
    import torch

    lib = model._lib()
    p = _particles_of(start)
    cfg = model._config_struct(tier)
    cs = _cot_struct(cot)
    g_alpha = C.c_double(0.0)
    torch.cuda.synchronize()
    lib.check(lib.lib.gbsph_adjoint_step(lib.handle, C.byref(p), C.byref(cfg), float(t),
                                         float(dt), int(corrector_iters), C.byref(cs),
                                         C.byref(g_alpha), None))
    if "g_av" in cot:
        cot["g_av"][0] += cs.g_alpha_min
        cot["g_av"][1] += cs.g_alpha_max
        cot["g_av"][2] += cs.g_sigma_decay
    return g_alpha.value


# Above this many particles times steps per segment the backward pass records and
# reverses on one context (a context holds the tree, cache slots and staging of one step:
# about 5 GB at 4M particles on the homogeneous set-up), else on one context per step.
MAX_POOLED_PARTICLES = 1 << 25


def _record_contexts(model, k):
    """k library contexts on the model's device for the steps of a segment (kept on the
    model, grown as needed)."""
    pool = getattr(model, "_adj_pool", None)
    if pool is None:
        pool = model._adj_pool = []
    dev = model._lib().device
    while len(pool) < k:
        pool.append(L.Context(dev))
    return pool


def _step(model, t, dt, tier=None):
    model.time = float(t)
    model.dt = float(dt)
    return model.evolve_once(tier=tier)


class _Rollout:
    """Forward bookkeeping shared by the autograd function and direct callers."""

    def __init__(self, model, n_steps, checkpoint_every, dts=None):
        self.model = model
        self.n_steps = int(n_steps)
        self.k = max(1, int(checkpoint_every))
        self.dts = None if dts is None else [float(v) for v in dts]
        self.records = []     # per step: (t, dt, corrector_iters, precision tier)
        self.checkpoints = {}  # step index -> state before that step

    def forward(self):
        m = self.model
        t = m.time
        for j in range(self.n_steps):
            if j % self.k == 0:
                self.checkpoints[j] = _snapshot(m)
            dt = self.dts[j] if self.dts is not None else m.dt
            log = _step(m, t, dt)
            self.records.append((t, dt, int(log["corrector_iters"]), int(log["tier"])))
            t = t + dt
            if self.dts is None:
                m.dt = log["next_dt"]
        return m

    def backward(self, cot):
        """cot: cotangents of the final state (dict gx, gv, ga, gu, gdu); updated in place
        to the cotangents of the initial state.  Returns dL/d alpha_AV."""
        n = int(cot["gu"].shape[0])
        if self.k > 1 and n * self.k > MAX_POOLED_PARTICLES:
            return self._backward_one_context(cot)
        return self._backward_pooled(cot)

    def _backward_one_context(self, cot):
        """The schedule for segments too large to keep a context per step: the segment's
        start states rebuilt from its checkpoint with plain steps, then each step recorded
        and reversed on the model's own context (gbsph_adjoint_step)."""
        import torch

        m = self.model
        saved = _snapshot(m)
        saved_time = (m.time, m.dt, m.cfl_mult)
        g_alpha = 0.0
        for s0 in reversed(sorted(self.checkpoints)):
            s1 = min(s0 + self.k, self.n_steps)
            _restore(m, self.checkpoints[s0])
            seg = []
            for j in range(s0, s1):
                seg.append(_snapshot(m))
                t, dt, _, tier = self.records[j]
                if j + 1 < s1:
                    _step(m, t, dt, tier)
            for j in reversed(range(s0, s1)):
                t, dt, kk, tier = self.records[j]
                g_alpha += adjoint_step(m, seg[j - s0], t, dt, kk, cot, tier)
        _restore(m, saved)
        m.time, m.dt, m.cfl_mult = saved_time
        torch.cuda.synchronize()
        return g_alpha

    def _backward_pooled(self, cot):
        import torch

        m = self.model
        pool = _record_contexts(m, self.k)
        g_alpha = 0.0
        starts = sorted(self.checkpoints)
        torch.cuda.synchronize()
        for s0 in reversed(starts):
            s1 = min(s0 + self.k, self.n_steps)
            # the segment recomputed once: step j recorded on pool[j - s0], from the state
            # the previous step's context holds after its step
            start = _particles_of(self.checkpoints[s0])
            rec = []
            for j in range(s0, s1):
                t, dt, kk, tier = self.records[j]
                cfg = m._config_struct(tier)
                after = L.Particles()
                ctx = pool[j - s0]
                ctx.check(ctx.lib.gbsph_adjoint_record(ctx.handle, C.byref(start), C.byref(cfg),
                                                       float(t), float(dt), int(kk),
                                                       C.byref(after), None))
                rec.append((start, cfg))
                start = after
            for j in reversed(range(s0, s1)):
                t, dt, kk, tier = self.records[j]
                start, cfg = rec[j - s0]
                ctx = pool[j - s0]
                cs = _cot_struct(cot)
                g = C.c_double(0.0)
                ctx.check(ctx.lib.gbsph_adjoint_reverse(ctx.handle, C.byref(start), C.byref(cfg),
                                                        float(dt), C.byref(cs), C.byref(g), None))
                if "g_av" in cot:
                    cot["g_av"][0] += cs.g_alpha_min
                    cot["g_av"][1] += cs.g_alpha_max
                    cot["g_av"][2] += cs.g_sigma_decay
                g_alpha += g.value
        torch.cuda.synchronize()
        return g_alpha


def _zero_cot(n, dev, varying=False):
    import torch

    z = lambda *s: torch.zeros(*s, dtype=torch.float64, device=dev)
    cot = dict(gx=z(3, n), gv=z(3, n), ga=z(3, n), gu=z(n), gdu=z(n))
    if varying:
        cot.update(galpha=z(n), gcs=z(n), g_av=[0.0, 0.0, 0.0])
    return cot


def rollout(model, v0, u0, alpha, n_steps, checkpoint_every=5, dts=None, x0=None):
    """Differentiable n-step rollout; returns (x_final, v_final, u_final) and records the
    dt sequence in ``rollout.last_dts``."""
    import torch

    class Fn(torch.autograd.Function):
        @staticmethod
        def forward(ctx, v0_, u0_, alpha_, x0_):
            d = model._to_device()
            if x0_ is not None:
                d["xyz"].copy_(x0_)
            d["vxyz"].copy_(v0_)
            d["uint"].copy_(u0_)
            if _varying(model):
                model.cfg.av["alpha_min"] = float(alpha_[0])
                model.cfg.av["alpha_max"] = float(alpha_[1])
            else:
                model.cfg.av["alpha_AV"] = float(alpha_)
            ro = _Rollout(model, n_steps, checkpoint_every, dts)
            ro.forward()
            ctx.ro = ro
            ctx.has_x0 = x0_ is not None
            rollout.last_dts = [r[1] for r in ro.records]
            rollout.last_records = list(ro.records)
            out = model._to_device()
            return out["xyz"].clone(), out["vxyz"].clone(), out["uint"].clone()

        @staticmethod
        def backward(ctx, gx, gv, gu):
            n = gu.shape[0] if gu is not None else model.get_total_part_count()
            dev = model._to_device()["hpart"].device
            var = _varying(model)
            cot = _zero_cot(n, dev, var)
            if gx is not None:
                cot["gx"].copy_(gx)
            if gv is not None:
                cot["gv"].copy_(gv)
            if gu is not None:
                cot["gu"].copy_(gu)
            g_alpha = ctx.ro.backward(cot)
            if var:
                ga = torch.tensor(cot["g_av"][:2], dtype=torch.float64)
                rollout.last_av_grads = dict(alpha_AV=cot["galpha"], soundspeed=cot["gcs"],
                                             sigma_decay=cot["g_av"][2])
            else:
                ga = torch.tensor(g_alpha, dtype=torch.float64)
            return cot["gv"], cot["gu"], ga, (cot["gx"] if ctx.has_x0 else None)

    alpha_t = alpha if isinstance(alpha, torch.Tensor) else torch.tensor(alpha, dtype=torch.float64)
    return Fn.apply(v0, u0, alpha_t, x0)


rollout.last_dts = None
rollout.last_records = None
rollout.last_av_grads = None
