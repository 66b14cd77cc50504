// Mixed-precision SPH pair kernels: the per-pair arithmetic of the h-rho Newton
// sums, Omega and the constant-AV derivatives runs in FP32 on hi/lo-split positions
// and velocities, with Kahan-compensated FP32 neighbour sums.  FP64 is kept for the
// absolute positions, the Newton update and its convergence test (eps_h), the
// leapfrog corrector and CFL, and the global totals.  Same physics and neighbour
// set as the FP64 kernels (sph64.cu); see those for the reference citations.
//
// Every neighbour costs one 256-bit load of its position record (density sums) or
// two (derivatives: position + hydro record).  Neighbour loops take CSR entries four
// at a time, issue all record loads of the four together and fetch the next four
// entries behind them, so each batch waits on one round trip.  Sums are accumulated
// per batch in plain FP32 and the batch sums are Kahan-compensated.  This unit is
// compiled with approximate FP32 division and square root (about 2 ulp).
//
// GB300 executes FP64 at a small fraction of its FP32 rate, so the per-particle work
// around the pair loops avoids FP64 wherever the result is stored in FP32 anyway or is
// dimensionless: hi/lo splits use integer operations (split64.cuh), 1/h is an FP32
// reciprocal, the Newton step and Omega are computed from the dimensionless ratios
// rho_sum / rho_h and h (d rho / dh) / rho_h, and the CFL step runs in FP32.  FP64 stays
// on the state (h, x, v, u, a) and on pressure, whose hi/lo pair carries it beyond FP32.

#include "df32.cuh"
#include "mixed_common.cuh"

namespace gbsph {

namespace {


// B.w carries fl32 of the neighbour-cache threshold ((h htol)^2) R^2 (computed in FP64
// in the reference's order) for the FP32 pre-test of the cache build; the corrector
// staging later overwrites it with c_s.
__global__ void k_stage_pos(u32 N, const f64 *__restrict__ sx, const f64 *__restrict__ sy,
                            const f64 *__restrict__ sz, const f64 *__restrict__ sh, f64 h_tol,
                            float4 *__restrict__ P) {
    u32 r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= N) return;
    float xh, xl, yh, yl, zh, zl;
    split64(sx[r], xh, xl);
    split64(sy[r], yh, yl);
    split64(sz[r], zh, zl);
    const f64 h = sh[r];
    f64 rint = __dmul_rn(h, h_tol);
    f64 thr  = __dmul_rn(__dmul_rn(rint, rint), kRkern * kRkern);
    P[2 * (size_t) r]     = make_float4(xh, yh, zh, __double2float_rn(rcp64(h)));
    P[2 * (size_t) r + 1] = make_float4(xl, yl, zl, __double2float_rn(thr));
}

// hydro staging from FP64 fields in the entry index space
__global__ void k_stage_hydro(u32 N, const f64 *__restrict__ x, const f64 *__restrict__ y,
                              const f64 *__restrict__ z, HydroSpace hs, f64 pmass,
                              float4 *__restrict__ P, float4 *__restrict__ H) {
    u32 r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= N) return;
    f64 h = hs.h[r], om = hs.omega[r], Pr = hs.P[r];
    f64 rho = rho_h64(pmass, h);
    float hinv = __double2float_rn(1.0 / h);
    size_t p2 = 2 * (size_t) r;
    if (x) {
        P[p2]     = make_float4(hi32(x[r]), hi32(y[r]), hi32(z[r]), hinv);
        P[p2 + 1] = make_float4(lo32(x[r]), lo32(y[r]), lo32(z[r]), __double2float_rn(hs.cs[r]));
    } else {
        ((float *) &P[p2])[3]     = hinv;
        ((float *) &P[p2 + 1])[3] = __double2float_rn(hs.cs[r]);
    }
    f64 vx = hs.vx[r], vy = hs.vy[r], vz = hs.vz[r];
    f64 sub = rho * rho * om;
    f64 c1  = (sub != 0 && sub == sub) ? 1. / sub : 0.;
    H[p2]     = make_float4(hi32(vx), hi32(vy), hi32(vz), __double2float_rn(hs.u[r]));
    H[p2 + 1] = make_float4(hi32(Pr), __double2float_rn(c1), pack_bf16x2(lo32(vx), lo32(vy)),
                            pack_bf16x2(lo32(vz), lo32(Pr)));
}

// EOS and hydro staging of the corrector loop in one pass (the FP64 path runs
// k_gather_eos into FP64 rank-ordered copies instead): per merged rank r, the source
// particle's fields (a local id, or a ghost's source), its pressure and sound speed,
// written as whole 32-byte position and hydro records.  Pressure and c_s follow
// ComputeEos.cpp (adiabatic: P = (gamma - 1) rho u, c_s = sqrt(gamma P / rho) =
// sqrt(gamma (gamma - 1) u); locally isothermal LP07: c_s^2 = cs0^2 (R^2/r0^2)^-q at the
// merged position, P = c_s^2 rho), and the FP64 h in rank order for the CFL step of the
// derivatives kernel.  c_s is stored in FP32, so it and the LP07 power are
// evaluated in FP32 (relative error ~2e-7, the size of the records' own rounding); rho,
// P and 1/(rho^2 Omega) stay FP64 until they are split into the record.
// varying viscosity: per rank a 32-byte record V of what the velocity gradients read
// besides positions, {vx_hi, vy_hi, vz_hi, ax | ay, az, bf16 (vx_lo, vy_lo), bf16 (vz_lo, 0)},
// the accelerations being those of the last evaluation in FP32 (ghosts copy their
// source), and the plain sound speed per rank (the records' c_s lane then carries
// alpha c_s)
struct StageAV {
    const f64 *ax, *ay, *az; // caller's local fields, stride of the caller's vectors
    float4 *V;               // 2 float4 per rank; null: constant viscosity
    float *cs_rank;
};

struct StageEos {
    u32 kind;       // 0 adiabatic, 1 locally isothermal LP07
    f64 gm1;        // gamma - 1
    f64 mh3;        // m hfact^3: rho = mh3 / h^3
    float gg;       // gamma (gamma - 1)
    float inv_r0sq; // 1 / r0^2
    float cs0sq, mq;
    f64 inv_r0sq64, cs0sq64, mq64; // the same in FP64 (compensated tier)
};

__global__ void k_gather_stage_mixed(const u32 *__restrict__ sort_index, u32 N, u32 n_local,
                                     const u32 *__restrict__ ghost_src, LocalFields lf,
                                     const f64 *__restrict__ omega, f64 pmass, StageEos eos,
                                     const f64 *__restrict__ sx, const f64 *__restrict__ sy,
                                     const f64 *__restrict__ sz, float4 *__restrict__ P,
                                     float4 *__restrict__ H, f64 *__restrict__ h_rank,
                                     StageAV av, float4 *__restrict__ E) {
    u32 r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= N) return;
    u32 id  = sort_index[r];
    u32 src = id < n_local ? id : ghost_src[id - n_local];
    size_t iv = (size_t) src * lf.vs;
    f64 hh = lf.h[src], uu = lf.u[src], om = omega[src];
    float xh, xl, yh, yl, zh, zl, vxh, vxl, vyh, vyl, vzh, vzl;
    split64(sx[r], xh, xl);
    split64(sy[r], yh, yl);
    split64(sz[r], zh, zl);
    split64(lf.vx[iv], vxh, vxl);
    split64(lf.vy[iv], vyh, vyl);
    split64(lf.vz[iv], vzh, vzl);
    h_rank[r] = hh;
    float u_hi, u_lo;
    split64(uu, u_hi, u_lo);
    float hinv_f, cs, c1, Ph, Pl;
    f64 hinv = 0, Pr = 0, sub = 0;
    if (!E) {
        // The FP32 tier's records need 1/h and c1 to FP32 and P to about 2^-32 (its hi
        // part and a bfloat16 residual): evaluated in double-float arithmetic on the FP32
        // pipes from the exact hi/lo splits of h, u, Omega and the constants, which keeps
        // this pass off GB300's scarce FP64 pipe.
        float h_hi, h_lo, m_hi, m_lo, o_hi, o_lo;
        split64(hh, h_hi, h_lo);
        split64(eos.mh3, m_hi, m_lo);
        split64(om, o_hi, o_lo);
        // 1/h: the FP32 reciprocal and one Newton step against the double-float h
        const float y0 = __frcp_rn(h_hi);
        const df hy    = df_mul_f(df{h_hi, h_lo}, y0);
        const df hi_df = fast_two_sum(y0, y0 * ((1.f - hy.hi) - hy.lo));
        hinv_f         = hi_df.hi;
        const df rho   = df_mul(df_mul(df_sqr(hi_df), hi_df), df{m_hi, m_lo});
        df P;
        if (eos.kind == 1) {
            const float ratio = (xh * xh + yh * yh + zh * zh) * eos.inv_r0sq;
            const float cs_sq = eos.cs0sq * powf(ratio, eos.mq);
            P  = df_mul_f(rho, cs_sq);
            cs = sqrtf(cs_sq);
        } else {
            float g_hi, g_lo;
            split64(eos.gm1, g_hi, g_lo);
            P  = df_mul(df_mul(df{g_hi, g_lo}, rho), df{u_hi, u_lo});
            cs = sqrtf(eos.gg * u_hi);
        }
        const df Pn = two_sum(P.hi, P.lo); // hi: the value rounded to FP32
        Ph = Pn.hi;
        Pl = Pn.lo;
        // c1 = inv_sat_zero(rho^2 Omega): the FP32 reciprocal refined once
        const df sd = df_mul(df_sqr(rho), df{o_hi, o_lo});
        c1          = 0.f;
        if (sd.hi != 0.f && isfinite(sd.hi)) {
            const float s0 = __frcp_rn(sd.hi);
            const df sy    = df_mul_f(sd, s0);
            c1             = s0 + s0 * ((1.f - sy.hi) - sy.lo);
        }
    } else {
        hinv   = rcp64(hh);
        hinv_f = __double2float_rn(hinv);
        const f64 rho = eos.mh3 * hinv * hinv * hinv;
        if (eos.kind == 1) {
            // compensated tier: the pressure to FP64 accuracy
            const f64 Rsq   = sx[r] * sx[r] + sy[r] * sy[r] + sz[r] * sz[r];
            const f64 cs_sq = eos.cs0sq64 * pow(Rsq * eos.inv_r0sq64, eos.mq64);
            Pr              = cs_sq * rho;
            cs              = (float) sqrt(cs_sq);
        } else {
            Pr = eos.gm1 * rho * uu;
            cs = sqrtf(eos.gg * u_hi);
        }
        sub = rho * rho * om;
        c1  = (sub != 0 && sub == sub) ? __double2float_rn(rcp64(sub)) : 0.f;
        split64(Pr, Ph, Pl);
    }
    size_t p2 = 2 * (size_t) r;
    P[p2]     = make_float4(xh, yh, zh, hinv_f);
    P[p2 + 1] = make_float4(xl, yl, zl, cs);
    H[p2]     = make_float4(vxh, vyh, vzh, u_hi);
    H[p2 + 1] = make_float4(Ph, c1, pack_bf16x2(vxl, vyl), pack_bf16x2(vzl, Pl));
    if (av.V) {
        float axh, axl, ayh, ayl, azh, azl;
        split64(av.ax[iv], axh, axl);
        split64(av.ay[iv], ayh, ayl);
        split64(av.az[iv], azh, azl);
        av.V[p2]     = make_float4(vxh, vyh, vzh, axh);
        av.V[p2 + 1] = make_float4(ayh, azh, pack_bf16x2(vxl, vyl), pack_bf16x2(vzl, 0.f));
        av.cs_rank[r] = cs;
    }
    if (E) {
        // X = P / (rho^2 Omega) (zero where the reference's inv_sat_zero gives zero), the
        // residuals of 1/h, P and u, and 1/h^4, as double-floats
        const f64 X = (sub != 0 && sub == sub) ? Pr * rcp64(sub) : 0.;
        float Xh, Xl, h4h, h4l;
        split64(X, Xh, Xl);
        const f64 hinv2 = hinv * hinv;
        split64(hinv2 * hinv2, h4h, h4l);
        const float hinv_lo = __double2float_rn(hinv - (f64) hinv_f);
        E[p2]     = make_float4(Xh, Xl, hinv_lo, Pl);
        E[p2 + 1] = make_float4(u_lo, h4h, h4l, 0.f);
    }
}

// sum_b f(q) and sum_b (3 f + q f') over the row, q = r / h_a.  The next four entries
// are fetched while the current four position records are in flight.
__device__ __forceinline__ void density_sums_f32(const RowSpace &rs, const MixedSpace &ms, u32 a,
                                                 u32 k0, u32 k1, float hinv, float &sf, float &sg) {
    const F8 pa    = ldg256(&ms.P[2 * (size_t) a]);
    const bool vec = rs.row_rank != nullptr;
    float cf = 0.f, cg = 0.f;
    sf = 0.f;
    sg = 0.f;
    float hinv2 = hinv * hinv;
    uint4 nx    = (k0 < k1) ? load_entries(rs.ent, k0, k1, vec, a) : make_uint4(a, a, a, a);
    for (u32 k = k0; k < k1; k += 4) {
        const u32 bb[4] = {nx.x, nx.y, nx.z, nx.w};
        F8 pb[4];
#pragma unroll
        for (int j = 0; j < 4; j++) pb[j] = ldg256(&ms.P[2 * (size_t) bb[j]]);
        if (k + 4 < k1) nx = load_entries(rs.ent, k + 4, k1, vec, a);
        float bf = 0.f, bg = 0.f;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            float dx = (pa.a.x - pb[j].a.x) + (pa.b.x - pb[j].b.x);
            float dy = (pa.a.y - pb[j].a.y) + (pa.b.y - pb[j].b.y);
            float dz = (pa.a.z - pb[j].a.z) + (pa.b.z - pb[j].b.z);
            float q2 = (dx * dx + dy * dy + dz * dz) * hinv2;
            if (k + j >= k1 || q2 > 4.f) continue;
            float q  = sqrt_approx(q2);
            float f  = m4_f32(q);
            float df = m4_df32(q);
            bf += f;
            bg += 3.f * f + q * df;
        }
        kahan_add(sf, cf, bf);
        kahan_add(sg, cg, bg);
    }
}

__global__ void __launch_bounds__(256, 4) k_h_iterate_mixed(RowSpace rs, MixedSpace ms,
                                                         const f64 *__restrict__ h_old,
                                                         f64 *__restrict__ h_new,
                                                         f64 *__restrict__ eps, f64 pmass,
                                                         f64 h_evol_max, f64 h_evol_iter_max,
                                                         u32 iters, f64 eps_p, Scalars *sc) {
    u32 t = blockIdx.x * blockDim.x + threadIdx.x;
    u64 emax = 0, emin = ~0ull;
    u32 used = 0;
    if (t < rs.n) {
        u32 a  = rs.row_rank ? rs.row_rank[t] : t;
        u32 k0 = rs.off[t], k1 = k0 + rs.cnt[t];
        // The Newton step of IterateSmoothingLengthDensity in dimensionless form:
        //   new_h = h - (rho_sum - rho_h) / (drho/dh + 3 rho_h / h) = h (1 - (A - 1) / (B + 3))
        // with A = rho_sum / rho_h and B = h (drho/dh) / rho_h, both FP32 sums times
        // kNorm3d / hfact^3; the relative update is FP32, h itself stays FP64.
        const float it_max = (float) h_evol_iter_max, it_min = 1.f / it_max;
        const f64 ha_0 = h_old[t], h_lim = ha_0 * h_evol_max;
        const float inv_h0 = __frcp_rn(__double2float_rn(ha_0));
        f64 h_a = h_new[t], e = eps[t];
        for (u32 it = 0; it < iters; it++) {
            if (!(e > eps_p)) break;
            used++;
            float sf, sg;
            const float hf = __double2float_rn(h_a);
            density_sums_f32(rs, ms, a, k0, k1, __double2float_rn(rcp64(h_a)), sf, sg);
            const float A = kDensRatio * sf, B = -kDensRatio * sg;
            float d = __fdiv_rn(A - 1.f, B + 3.f); // new_h = h (1 - d)
            float f = 1.f - d;
            if (f < it_min) d = 1.f - it_min;
            if (f > it_max) d = 1.f - it_max;
            const f64 new_h = h_a - h_a * (f64) d;
            if (new_h < h_lim) {
                e   = (f64) (fabsf(d) * hf * inv_h0);
                h_a = new_h;
            } else {
                h_a = h_lim;
                e   = -1;
            }
        }
        h_new[t] = h_a;
        eps[t]   = e;
        emax     = f64_to_ordered(e);
        emin     = emax;
    }
    emax   = block_reduce(emax, OpMaxU64{}, 0ull);
    emin   = block_reduce(emin, OpMinU64{}, ~0ull);
    u64 um = block_reduce((u64) used, OpMaxU64{}, 0ull);
    if (threadIdx.x == 0) {
        atomicMax((unsigned long long *) &sc->eps_max, (unsigned long long) emax);
        atomicMin((unsigned long long *) &sc->eps_min, (unsigned long long) emin);
        atomicMax(&sc->iters_max, (u32) um);
    }
}

// 1/h lane of the position records from the converged smoothing lengths (the records
// were staged with the h the neighbour cache was built with); the same value the
// corrector staging writes, so the compaction below and the corrector kernels test
// pairs alike.
__global__ void k_restage_hinv(const u32 *__restrict__ sort_index, u32 N, u32 n_local,
                               const u32 *__restrict__ ghost_src, const f64 *__restrict__ h,
                               float4 *__restrict__ P) {
    u32 r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= N) return;
    u32 id  = sort_index[r];
    u32 src = id < n_local ? id : ghost_src[id - n_local];
    ((float *) &P[2 * (size_t) r])[3] = __double2float_rn(rcp64(h[src]));
}

// Omega = 1 + B / 3, B = -kNorm3d / hfact^3 sum (3f + q f') (ComputeOmega.cpp:36-73 in
// the dimensionless form of the FP32 h iteration) and, in the same pass over the row,
// the row compacted in place to the entries the corrector kernels can use: pairs inside either particle's
// support at the converged h, the test of derivs_row_f32 (r^2 h_a^-2 > 4 and
// r^2 h_b^-2 > 4 drops a pair), coincident pairs and the particle itself kept (the
// density terms of the reverse pass include them).  About a quarter of a row lies
// beyond both supports (the cache holds pairs within 1.1 h).  Writes trail reads
// within the thread's own row (a group of four is written only after its four entries
// and the next four have been read), so the compaction is race-free.
__global__ void __launch_bounds__(256) k_omega_compact_mixed(RowSpace rs, MixedSpace ms,
                                                             const f64 *__restrict__ h_row,
                                                             f64 *__restrict__ omega_local,
                                                             u32 *ent_w, u32 *cnt_w, Scalars *sc) {
    u32 t = blockIdx.x * blockDim.x + threadIdx.x;
    u64 kept = 0;
    if (t < rs.n) {
        const u32 a  = rs.row_rank[t];
        const u32 k0 = rs.off[t], k1 = k0 + rs.cnt[t];
        const float hinv  = __double2float_rn(rcp64(h_row[t]));
        const float hinv2 = hinv * hinv;
        const F8 pa = ldg256(&ms.P[2 * (size_t) a]);
        float sg = 0.f, cg = 0.f;
        // kept entries are collected four at a time and written with one 128-bit store
        // (rows start on 16-byte boundaries and their slots are padded to four entries)
        u32 w = k0, p = 0;
        uint4 pend = make_uint4(a, a, a, a);
        uint4 nx = (k0 < k1) ? load_entries(rs.ent, k0, k1, true, a) : make_uint4(a, a, a, a);
        for (u32 k = k0; k < k1; k += 4) {
            const u32 bb[4] = {nx.x, nx.y, nx.z, nx.w};
            F8 pb[4];
    #pragma unroll
            for (int j = 0; j < 4; j++) pb[j] = ldg256(&ms.P[2 * (size_t) bb[j]]);
            if (k + 4 < k1) nx = load_entries(rs.ent, k + 4, k1, true, a);
            float bg = 0.f;
    #pragma unroll
            for (int j = 0; j < 4; j++) {
                if (k + j >= k1) continue;
                float dx = (pa.a.x - pb[j].a.x) + (pa.b.x - pb[j].b.x);
                float dy = (pa.a.y - pb[j].a.y) + (pa.b.y - pb[j].b.y);
                float dz = (pa.a.z - pb[j].a.z) + (pa.b.z - pb[j].b.z);
                float r2 = dx * dx + dy * dy + dz * dz;
                const float hib = pb[j].a.w;
                if (!(r2 * hinv2 > 4.f && r2 * (hib * hib) > 4.f)) {
                    const u32 b = bb[j];
                    pend.x = p == 0 ? b : pend.x;
                    pend.y = p == 1 ? b : pend.y;
                    pend.z = p == 2 ? b : pend.z;
                    pend.w = p == 3 ? b : pend.w;
                    if (++p == 4) {
                        *(uint4 *) (ent_w + w) = pend;
                        w += 4;
                        p = 0;
                    }
                }
                float q2 = r2 * hinv2;
                if (q2 > 4.f) continue;
                float q = sqrt_approx(q2);
                bg += 3.f * m4_f32(q) + q * m4_df32(q);
            }
            kahan_add(sg, cg, bg);
        }
        if (p) *(uint4 *) (ent_w + w) = pend; // the tail (slots past it hold stale entries)
        cnt_w[t] = w - k0 + p;
        kept     = w - k0 + p;
        omega_local[rs.row_local[t]] = (f64) (1.f - kDensRatio * sg * (1.f / 3.f));
    }
    kept = block_reduce(kept, OpAddU64{}, 0ull);
    if (threadIdx.x == 0) atomicAdd((unsigned long long *) &sc->csr_kept, (unsigned long long) kept);
}

// FP32 pair loop of the constant-AV derivatives; returns the bare sums
//   F = sum (ca Fa + cb Fb) r_hat   (acceleration = -m F)
//   U = sum [AVPa c1a Fa (v.r_hat) + 0.5 alpha_u vsig_u (u_a - u_b)(Fa c2a + Fb c2b)]
//   (du/dt = m U), and the v_sig maximum of the reference's separate v_sig kernel,
// with c1 = 1/(rho^2 Omega) and c2 = 1/(rho Omega) = c1 rho, rho = m (hfact/h)^3.
// Self and coincident pairs (r = 0) contribute nothing and are skipped, which also
// makes padding a partial batch of four with the row's own index harmless.
// cs_rank (varying viscosity): the records' c_s lane holds alpha c_s, p.alpha_AV is 1,
// and the plain c_s of the row for the v_sig maximum comes from cs_rank.
// Condition sums for the error estimate of the step (unused by the module kernels):
//   sa = sum |AVP_a c1a F_a + AVP_b c1b F_b|, the magnitudes of the pair forces whose sum
//        is F (their FP32 rounding, and that of the h behind them, errs in proportion);
//   su = sum |P-term| + |conductivity coefficient| (|u_a| + |u_b|), the du/dt terms with
//        the energy difference replaced by the magnitudes it is taken from.
template<bool COND = false>
__device__ __forceinline__ void derivs_row_f32(const RowSpace &rs, const MixedSpace &ms, u32 a,
                                               u32 k0, u32 k1, const MixedParams &p, float &Fx,
                                               float &Fy, float &Fz, float &U, float &vsig_max,
                                               float &sa, float &su,
                                               const float *__restrict__ cs_rank = nullptr) {
    const bool vec = rs.row_rank != nullptr;
    const F8 pa = ldg256(&ms.P[2 * (size_t) a]);
    const F8 ha = ldg256(&ms.H[2 * (size_t) a]);
    const float hia = pa.a.w, cs_a = pa.b.w, u_a = ha.a.w;
    const float hia2 = hia * hia;
    const float rho_a = p.mh3 * hia2 * hia;
    const float Pa_hi = ha.b.x, Pa_lo = bf_lo(ha.b.w), P_a = Pa_hi + Pa_lo;
    const float c1a = ha.b.y, c2a = c1a * rho_a;
    const float vla_x = bf_hi(ha.b.z), vla_y = bf_lo(ha.b.z), vla_z = bf_hi(ha.b.w);
    const float k4a = hia2 * hia2 * kNorm3dF;
    const float cs_sig = cs_rank ? cs_rank[a] : cs_a;
    float cx = 0.f, cy = 0.f, cz = 0.f, cu = 0.f;
    Fx = Fy = Fz = U = 0.f;
    vsig_max = 0.f;
    sa = su = 0.f;
    const float abs_ua = fabsf(u_a);
    uint4 nx = (k0 < k1) ? load_entries(rs.ent, k0, k1, vec, a) : make_uint4(a, a, a, a);
    for (u32 k = k0; k < k1; k += 4) {
        // both records of all four neighbours in one round trip, next entries behind them
        const u32 bb[4] = {nx.x, nx.y, nx.z, nx.w};
        F8 pb[4], hb[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            pb[j] = ldg256(&ms.P[2 * (size_t) bb[j]]);
            hb[j] = ldg256(&ms.H[2 * (size_t) bb[j]]);
        }
        if (k + 4 < k1) nx = load_entries(rs.ent, k + 4, k1, vec, a);
        float bx = 0.f, by = 0.f, bz = 0.f, bu = 0.f;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            float dx = (pa.a.x - pb[j].a.x) + (pa.b.x - pb[j].b.x);
            float dy = (pa.a.y - pb[j].a.y) + (pa.b.y - pb[j].b.y);
            float dz = (pa.a.z - pb[j].a.z) + (pa.b.z - pb[j].b.z);
            float r2 = dx * dx + dy * dy + dz * dz;
            const float hib = pb[j].a.w, cs_b = pb[j].b.w;
            const float hib2 = hib * hib;
            if (k + j >= k1 || r2 == 0.f || (r2 * hia2 > 4.f && r2 * hib2 > 4.f)) continue;
            const float hib3 = hib2 * hib;
            const float rho_b = p.mh3 * hib3;
            const float c1b = hb[j].b.y, c2b = c1b * rho_b;
            const float Pb_lo = bf_lo(hb[j].b.w), P_b = hb[j].b.x + Pb_lo;
            float rinv = rsqrtf(r2);
            float rab  = r2 * rinv;
            float Fa   = k4a * m4_df32(rab * hia);
            float Fb   = (hib2 * hib2) * kNorm3dF * m4_df32(rab * hib);
            float vx = (ha.a.x - hb[j].a.x) + (vla_x - bf_hi(hb[j].b.z));
            float vy = (ha.a.y - hb[j].a.y) + (vla_y - bf_lo(hb[j].b.z));
            float vz = (ha.a.z - hb[j].a.z) + (vla_z - bf_hi(hb[j].b.w));
            // r_hat = (dx, dy, dz) rinv applied once to v.r and once to the force
            float vr  = (vx * dx + vy * dy + vz * dz) * rinv;
            float avr = fabsf(vr);
            float vsig_a = p.alpha_AV * cs_a + p.beta_AV * avr;
            float vsig_b = p.alpha_AV * cs_b + p.beta_AV * avr;
            float dP     = (Pa_hi - hb[j].b.x) + (Pa_lo - Pb_lo);
            // sqrt(|dP| / mean rho) with the fast division (about 2 ulp)
            float vsig_u = sqrt_approx(fabsf(dP) * __fdividef(2.f, rho_a + rho_b));
            float qa = fmaxf(-0.5f * rho_a * vsig_a * vr, 0.f);
            float qb = fmaxf(-0.5f * rho_b * vsig_b * vr, 0.f);
            float AVPa = P_a + qa, AVPb = P_b + qb;
            float pf   = AVPa * c1a * Fa + AVPb * c1b * Fb;
            float f    = pf * rinv;
            bx += f * dx;
            by += f * dy;
            bz += f * dz;
            // the two du/dt terms rounded explicitly (no contraction, no sharing with the
            // force products), so that the instantiations with and without the condition
            // sums give the same bits
            const float tp = __fmul_rn(__fmul_rn(__fmul_rn(AVPa, c1a), Fa), vr);
            const float tc = __fmul_rn(__fmul_rn(0.5f * p.alpha_u, vsig_u),
                                       __fadd_rn(__fmul_rn(Fa, c2a), __fmul_rn(Fb, c2b)));
            bu += tp + tc * (u_a - hb[j].a.w);
            if (COND) {
                sa += fabsf(pf);
                su += fabsf(tp) + fabsf(tc) * (abs_ua + fabsf(hb[j].a.w));
            }
            vsig_max = fmaxf(vsig_max, cs_sig + 2.f * avr);
        }
        kahan_add(Fx, cx, bx);
        kahan_add(Fy, cy, by);
        kahan_add(Fz, cz, bz);
        kahan_add(U, cu, bu);
    }
}

__global__ void __launch_bounds__(128) k_derivs_mixed(RowSpace rs, MixedSpace ms, MixedParams p,
                                                      f64 pmass, f64 *__restrict__ ax,
                                                      f64 *__restrict__ ay, f64 *__restrict__ az,
                                                      f64 *__restrict__ du, f64 *__restrict__ vsig) {
    u32 t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= rs.n) return;
    u32 a  = rs.row_rank ? rs.row_rank[t] : t;
    u32 k0 = rs.off[t], k1 = k0 + rs.cnt[t];
    float Fx, Fy, Fz, U, vm, sa, su;
    derivs_row_f32(rs, ms, a, k0, k1, p, Fx, Fy, Fz, U, vm, sa, su);
    ax[t] = -pmass * (f64) Fx;
    ay[t] = -pmass * (f64) Fy;
    az[t] = -pmass * (f64) Fz;
    du[t] = pmass * (f64) U;
    if (vsig) vsig[t] = (f64) vm;
}

// COND: also the condition sums of the step's error estimate (first corrector
// evaluation of a step; the others skip their cost)
template<bool COND>
__global__ void __launch_bounds__(128) k_derivs_step_mixed(RowSpace rs, MixedSpace ms,
                                                           MixedParams p, f64 pmass,
                                                           const f64 *__restrict__ h_rank, f64 hdt,
                                                           f64 C_cour, f64 C_force, LocalFields lf,
                                                           ExtAccel ext, Scalars *sc,
                                                           const float *__restrict__ cs_rank) {
    u32 t = blockIdx.x * blockDim.x + threadIdx.x;
    u64 ev2 = 0, dtm = ~0ull;
    float v2 = 0.f;
    float c_fa = 0.f, c_fu = 0.f, c_a = 0.f, c_du = 0.f; // condition sums and magnitudes
    if (t < rs.n) {
        u32 a  = rs.row_rank[t];
        u32 k0 = rs.off[t], k1 = k0 + rs.cnt[t];
        float Fx, Fy, Fz, U, vm, sa, su;
        derivs_row_f32<COND>(rs, ms, a, k0, k1, p, Fx, Fy, Fz, U, vm, sa, su, cs_rank);
        if (COND) {
            c_fa = sa;
            c_fu = su;
            c_a  = sqrtf(Fx * Fx + Fy * Fy + Fz * Fz);
            c_du = fabsf(U);
        }
        f64 fx = -pmass * (f64) Fx, fy = -pmass * (f64) Fy, fz = -pmass * (f64) Fz;
        f64 tdu = pmass * (f64) U;
        u32 i     = rs.row_local[t];
        if (ext.x) {
            fx = fx + ext.x[i];
            fy = fy + ext.y[i];
            fz = fz + ext.z[i];
        }
        size_t iv = (size_t) i * lf.vs;
        f64 ox = lf.ax[iv], oy = lf.ay[iv], oz = lf.az[iv], odu = lf.du[i];
        lf.ax[iv] = fx;
        lf.ay[iv] = fy;
        lf.az[iv] = fz;
        lf.du[i]  = tdu;
        f64 ix = hdt * (fx - ox), iy = hdt * (fy - oy), iz = hdt * (fz - oz);
        f64 nvx = lf.vx[iv] + ix, nvy = lf.vy[iv] + iy, nvz = lf.vz[iv] + iz;
        lf.vx[iv] = nvx;
        lf.vy[iv] = nvy;
        lf.vz[iv] = nvz;
        lf.u[i]   = lf.u[i] + hdt * (tdu - odu);
        // the rerun test, the mean |v|^2 and the CFL step only need FP32 (they feed a
        // 1e-2 threshold, a normalisation and a time step)
        const float fix = (float) ix, fiy = (float) iy, fiz = (float) iz;
        ev2 = f64_to_ordered((f64) (fix * fix + fiy * fiy + fiz * fiz));
        const float fvx = (float) nvx, fvy = (float) nvy, fvz = (float) nvz;
        v2 = fvx * fvx + fvy * fvy + fvz * fvz;
        const float hf  = (float) h_rank[a];
        const float ffx = (float) fx, ffy = (float) fy, ffz = (float) fz;
        const float abs_a = sqrtf(ffx * ffx + ffy * ffy + ffz * ffz);
        float dt = fminf(__int_as_float(0x7f800000), (float) C_cour * hf / vm);
        dt       = fminf(dt, (float) C_force * sqrtf(hf / abs_a));
        dtm      = f64_to_ordered((f64) dt);
    }
    ev2 = block_reduce(ev2, OpMaxU64{}, 0ull);
    dtm = block_reduce(dtm, OpMinU64{}, ~0ull);
    v2  = block_reduce(v2, OpAddF32{}, 0.f);
    if (COND) cond_reduce(sc, c_fa, c_fu, c_a, c_du);
    if (threadIdx.x == 0) {
        atomicMax((unsigned long long *) &sc->epsv2_max, (unsigned long long) ev2);
        atomicMin((unsigned long long *) &sc->dt_min, (unsigned long long) dtm);
        atomicAdd(&sc->sum_v2, (f64) v2);
    }
}

// ---- varying viscosity, FP32 pair arithmetic: div v, curl v (SPH estimates) and
// d(div v)/dt = tr(G(a)) - tr(G(v) G(v)) with the corrected gradients G = R^-1 D, the
// mass factoring out of R^-1 D.  Positions and velocities from the hi/lo records,
// accelerations from the V records (64 bytes per pair with the position records); FP32
// sums (the results feed the viscosity switch, not the state).  The same sums as
// k_velgrad64, arranged for FP32:
//  - only pairs inside a's kernel support are visited (the cache also holds pairs inside
//    b's only, whose dW(r, h_a) is zero);
//  - R = -sum r (x) g is symmetric (g is parallel to r): six sums;
//  - div v and curl v are read off Dv = -sum g (x) v: sum v.g = -tr Dv and
//    sum (v x g)_i = eps_ijk Dv[k][j] (the SPH sums are the same terms as Dv's).
__device__ __forceinline__ void inv33f(const float m[3][3], float r[3][3]) {
    const float a00 = m[0][0], a01 = m[0][1], a02 = m[0][2];
    const float a10 = m[1][0], a11 = m[1][1], a12 = m[1][2];
    const float a20 = m[2][0], a21 = m[2][1], a22 = m[2][2];
    const float det = (((((-a02 * a11) * a20 + (a01 * a12) * a20) + (a02 * a10) * a21)
                        - (a00 * a12) * a21) - (a01 * a10) * a22) + (a00 * a11) * a22;
    const float id = __frcp_rn(det);
    r[0][0] = (-a12 * a21 + a11 * a22) * id;
    r[0][1] = (a02 * a21 - a01 * a22) * id;
    r[0][2] = (-a02 * a11 + a01 * a12) * id;
    r[1][0] = (a12 * a20 - a10 * a22) * id;
    r[1][1] = (-a02 * a20 + a00 * a22) * id;
    r[1][2] = (a02 * a10 - a00 * a12) * id;
    r[2][0] = (-a11 * a20 + a10 * a21) * id;
    r[2][1] = (a01 * a20 - a00 * a21) * id;
    r[2][2] = (-a01 * a10 + a00 * a11) * id;
}

__global__ void __launch_bounds__(128) k_velgrad_mixed(RowSpace rs, MixedSpace ms,
                                                       const float4 *__restrict__ V,
                                                       const f64 *__restrict__ omega_local,
                                                       f64 pmass, float mh3,
                                                       f64 *__restrict__ divv, f64 *__restrict__ cx,
                                                       f64 *__restrict__ cy, f64 *__restrict__ cz,
                                                       u32 cvs, f64 *__restrict__ dtdivv,
                                                       float *__restrict__ sums) {
    u32 t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= rs.n) return;
    const u32 a  = rs.row_rank[t];
    const u32 k0 = rs.off[t], k1 = k0 + rs.cnt[t];
    const F8 pa = ldg256(&ms.P[2 * (size_t) a]);
    const F8 va = ldg256(&V[2 * (size_t) a]);
    const float hia = pa.a.w, hia2 = hia * hia;
    const float k4a = hia2 * hia2 * kNorm3dF;
    const float vla[3] = {bf_hi(va.b.z), bf_lo(va.b.z), bf_hi(va.b.w)};
    const float aa[3]  = {va.a.w, va.b.x, va.b.y};
    float R00 = 0.f, R01 = 0.f, R02 = 0.f, R11 = 0.f, R12 = 0.f, R22 = 0.f;
    float Dv[3][3] = {}, Da[3][3] = {};
    // entries four at a time (pipeline rows are padded to 4), all records of the four
    // neighbours requested together, the next four entries fetched behind them
    uint4 nx = (k0 < k1) ? load_entries(rs.ent, k0, k1, true, a) : make_uint4(a, a, a, a);
    for (u32 k = k0; k < k1; k += 4) {
        const u32 bb[4] = {nx.x, nx.y, nx.z, nx.w};
        F8 pb[4], vb[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            pb[q] = ldg256(&ms.P[2 * (size_t) bb[q]]);
            vb[q] = ldg256(&V[2 * (size_t) bb[q]]);
        }
        if (k + 4 < k1) nx = load_entries(rs.ent, k + 4, k1, true, a);
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const float r[3] = {(pa.a.x - pb[q].a.x) + (pa.b.x - pb[q].b.x),
                                (pa.a.y - pb[q].a.y) + (pa.b.y - pb[q].b.y),
                                (pa.a.z - pb[q].a.z) + (pa.b.z - pb[q].b.z)};
            const float r2  = (r[0] * r[0] + r[1] * r[1]) + r[2] * r[2];
            if (k + q >= k1 || r2 * hia2 > 4.f) continue;
            const float inv  = (r2 < 1e-18f) ? 0.f : rsqrtf(r2); // 1/r, 0 for coincident pairs
            const float rab  = r2 * inv;
            const float v[3] = {(va.a.x - vb[q].a.x) + (vla[0] - bf_hi(vb[q].b.z)),
                                (va.a.y - vb[q].a.y) + (vla[1] - bf_lo(vb[q].b.z)),
                                (va.a.z - vb[q].a.z) + (vla[2] - bf_hi(vb[q].b.w))};
            const float w[3] = {aa[0] - vb[q].a.w, aa[1] - vb[q].b.x, aa[2] - vb[q].b.y};
            const float F    = k4a * m4_df32(rab * hia) * inv; // dW(r, h_a) / r
            const float g[3] = {F * r[0], F * r[1], F * r[2]};
            R00 = R00 - r[0] * g[0];
            R01 = R01 - r[0] * g[1];
            R02 = R02 - r[0] * g[2];
            R11 = R11 - r[1] * g[1];
            R12 = R12 - r[1] * g[2];
            R22 = R22 - r[2] * g[2];
#pragma unroll
            for (int i = 0; i < 3; i++)
#pragma unroll
                for (int j = 0; j < 3; j++) {
                    Dv[j][i] = Dv[j][i] - v[i] * g[j];
                    Da[j][i] = Da[j][i] - w[i] * g[j];
                }
        }
    }
    const u32 i = rs.row_local[t];
    if (sums) {
        // recorded for the reverse pass (by local id, 24 per row): R (xx xy xz yy yz zz),
        // Dv and Da row-major, the bare sums (without the pair mass)
        float *o = sums + 24 * (size_t) i;
        o[0] = R00;
        o[1] = R01;
        o[2] = R02;
        o[3] = R11;
        o[4] = R12;
        o[5] = R22;
#pragma unroll
        for (int j = 0; j < 3; j++)
#pragma unroll
            for (int k2 = 0; k2 < 3; k2++) {
                o[6 + 3 * j + k2]  = Dv[j][k2];
                o[15 + 3 * j + k2] = Da[j][k2];
            }
    }
    const float rho_a = mh3 * hia2 * hia;
    const float f = -(float) pmass / (__double2float_rn(omega_local[i]) * rho_a);
    divv[i] = (f64) (-f * ((Dv[0][0] + Dv[1][1]) + Dv[2][2]));
    cx[(size_t) i * cvs] = (f64) (f * (Dv[1][2] - Dv[2][1]));
    cy[(size_t) i * cvs] = (f64) (f * (Dv[2][0] - Dv[0][2]));
    cz[(size_t) i * cvs] = (f64) (f * (Dv[0][1] - Dv[1][0]));
    const float R[3][3] = {{R00, R01, R02}, {R01, R11, R12}, {R02, R12, R22}};
    float Ri[3][3], G[3][3];
    inv33f(R, Ri);
    float div_a = 0.f;
#pragma unroll
    for (int j = 0; j < 3; j++) div_a += (Ri[j][0] * Da[0][j] + Ri[j][1] * Da[1][j]) + Ri[j][2] * Da[2][j];
#pragma unroll
    for (int i2 = 0; i2 < 3; i2++)
#pragma unroll
        for (int j = 0; j < 3; j++) G[i2][j] = (Ri[i2][0] * Dv[0][j] + Ri[i2][1] * Dv[1][j]) + Ri[i2][2] * Dv[2][j];
    float tens = 0.f;
#pragma unroll
    for (int i2 = 0; i2 < 3; i2++)
#pragma unroll
        for (int j = 0; j < 3; j++) tens += G[j][i2] * G[i2][j];
    dtdivv[i] = (f64) (div_a - tens);
}

// P.b.w (c_s) times the updated alpha of each rank's source particle
__global__ void k_stage_alpha(const u32 *__restrict__ sort_index, u32 N, u32 n_local,
                              const u32 *__restrict__ ghost_src, const f64 *__restrict__ alpha,
                              float4 *__restrict__ P) {
    u32 r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= N) return;
    u32 id  = sort_index[r];
    u32 src = id < n_local ? id : ghost_src[id - n_local];
    float *w = &((float *) &P[2 * (size_t) r + 1])[3];
    *w       = *w * __double2float_rn(alpha[src]);
}

__global__ void k_cs_to_local(u32 n, const u32 *__restrict__ row_rank,
                              const u32 *__restrict__ row_local, const float *__restrict__ cs_rank,
                              f64 *__restrict__ dst) {
    u32 t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    dst[row_local[t]] = (f64) cs_rank[row_rank[t]];
}


// f_pos holds 2N float4 (position records), f_aux0 2N float4 (hydro records)
MixedSpace mixed_space(Ctx &c, u32 N) {
    return MixedSpace{c.f_pos.as<float4>(), c.f_aux0.as<float4>()};
}

cudaError_t ensure_mixed(Ctx &c, u32 N) {
    cudaError_t e;
    if ((e = c.f_pos.ensure(2 * sizeof(float4) * (size_t) N, c.stream)) != cudaSuccess) return e;
    return c.f_aux0.ensure(2 * sizeof(float4) * (size_t) N, c.stream);
}

} // namespace

const float4 *mixed_positions(Ctx &c) { return c.f_pos.as<float4>(); }

cudaError_t stage_positions_mixed(Ctx &c, u32 N, f64 h_tol) {
    cudaError_t e = ensure_mixed(c, N);
    if (e != cudaSuccess) return e;
    ProfScope ps(c, kProfTree, N);
    { k_stage_pos<<<div_up(N, 256), 256, 0, c.stream>>>(N, c.sx.as<f64>(), c.sy.as<f64>(),
                                                      c.sz.as<f64>(), c.sh.as<f64>(), h_tol,
                                                      c.f_pos.as<float4>()); GBSPH_COUNTED; }
    return cudaGetLastError();
}

cudaError_t h_iterate_mixed(Ctx &c, const RowSpace &rs, const f64 *h_old, f64 *h_new, f64 *eps,
                            f64 pmass, f64 h_evol_max, f64 h_evol_iter_max, u32 iters, f64 eps_p) {
    ProfScope ps(c, kProfHIter, rs.n);
    MixedSpace ms = mixed_space(c, c.n_obj);
    { k_h_iterate_mixed<<<div_up(rs.n, 256), 256, 0, c.stream>>>(
        rs, ms, h_old, h_new, eps, pmass, h_evol_max, h_evol_iter_max, iters, eps_p,
        c.d_scalars.as<Scalars>()); GBSPH_COUNTED; }
    return cudaGetLastError();
}

cudaError_t omega_compact_mixed(Ctx &c, const RowSpace &rs, u32 N, u32 n_local, const f64 *h_local,
                                const f64 *h_row, f64 *omega_local) {
    ProfScope ps(c, kProfOmega, rs.n);
    MixedSpace ms = mixed_space(c, c.n_obj);
    { k_restage_hinv<<<div_up(N, 256), 256, 0, c.stream>>>(c.sort_index.as<u32>(), N, n_local,
                                                         c.ghost_src.as<u32>(), h_local,
                                                         c.f_pos.as<float4>()); GBSPH_COUNTED; }
    { k_omega_compact_mixed<<<div_up(rs.n, 256), 256, 0, c.stream>>>(
        rs, ms, h_row, omega_local, c.csr_ent.as<u32>(), c.csr_cnt.as<u32>(),
        c.d_scalars.as<Scalars>()); GBSPH_COUNTED; }
    // the cache no longer holds the reference's pair set
    c.cache_valid = false;
    return cudaGetLastError();
}

cudaError_t gather_stage_mixed(Ctx &c, u32 N, u32 n_local, const LocalFields &lf,
                               const f64 *omega_local, f64 pmass, const EosParams &eos,
                               bool varying_av, bool compensated) {
    float4 *E = nullptr;
    if (compensated) {
        cudaError_t e = c.f_comp.ensure(2 * sizeof(float4) * (size_t) N, c.stream);
        if (e != cudaSuccess) return e;
        E = c.f_comp.as<float4>();
    }
    StageAV av{lf.ax, lf.ay, lf.az, nullptr, nullptr};
    if (varying_av) {
        cudaError_t e;
        if ((e = c.f_aux1.ensure(2 * sizeof(float4) * (size_t) N, c.stream)) != cudaSuccess) return e;
        if ((e = c.f_aux2.ensure(sizeof(float) * (size_t) N, c.stream)) != cudaSuccess) return e;
        av.V       = c.f_aux1.as<float4>();
        av.cs_rank = c.f_aux2.as<float>();
    }
    StageEos se{eos.kind, eos.gamma - 1, pmass * kHfact * kHfact * kHfact,
                (float) (eos.gamma * (eos.gamma - 1)), (float) (1.0 / (eos.r0 * eos.r0)),
                (float) (eos.cs0 * eos.cs0), (float) -eos.q, 1.0 / (eos.r0 * eos.r0),
                eos.cs0 * eos.cs0, -eos.q};
    ProfScope ps(c, kProfGatherEos, N);
    { k_gather_stage_mixed<<<div_up(N, 256), 256, 0, c.stream>>>(
        c.sort_index.as<u32>(), N, n_local, c.ghost_src.as<u32>(), lf, omega_local, pmass, se,
        c.sx.as<f64>(), c.sy.as<f64>(), c.sz.as<f64>(), c.f_pos.as<float4>(),
        c.f_aux0.as<float4>(), c.sh2.as<f64>(), av, E); GBSPH_COUNTED; }
    return cudaGetLastError();
}

cudaError_t derivs_step_mixed(Ctx &c, const RowSpace &rs, f64 pmass, f64 alpha_u, f64 alpha_AV,
                              f64 beta_AV, f64 hdt, f64 C_cour, f64 C_force,
                              const LocalFields &lf, const ExtAccel &ext, bool varying_av,
                              bool cond) {
    MixedSpace ms = mixed_space(c, c.n_obj);
    MixedParams p = mixed_params(pmass, alpha_u, varying_av ? 1.0 : alpha_AV, beta_AV);
    const float *cs_rank = varying_av ? c.f_aux2.as<float>() : nullptr;
    ProfScope ps(c, kProfDerivs, rs.n);
    auto kern = cond ? k_derivs_step_mixed<true> : k_derivs_step_mixed<false>;
    { kern<<<div_up(rs.n, 128), 128, 0, c.stream>>>(rs, ms, p, pmass, c.sh2.as<f64>(), hdt, C_cour,
                                                    C_force, lf, ext, c.d_scalars.as<Scalars>(),
                                                    cs_rank); GBSPH_COUNTED; }
    return cudaGetLastError();
}

cudaError_t velgrad_mixed(Ctx &c, const RowSpace &rs, const f64 *omega_local, f64 pmass,
                          f64 *divv, f64 *cx, f64 *cy, f64 *cz, u32 cvs, f64 *dtdivv,
                          float *sums) {
    MixedSpace ms = mixed_space(c, c.n_obj);
    ProfScope ps(c, kProfVelGrad, rs.n);
    { k_velgrad_mixed<<<div_up(rs.n, 128), 128, 0, c.stream>>>(
        rs, ms, c.f_aux1.as<float4>(), omega_local, pmass, (float) (pmass * kHfact * kHfact * kHfact),
        divv, cx, cy, cz, cvs, dtdivv, sums); GBSPH_COUNTED; }
    return cudaGetLastError();
}

cudaError_t stage_alpha_mixed(Ctx &c, u32 N, u32 n_local, const f64 *alpha_local) {
    { k_stage_alpha<<<div_up(N, 256), 256, 0, c.stream>>>(c.sort_index.as<u32>(), N, n_local,
                                                         c.ghost_src.as<u32>(), alpha_local,
                                                         c.f_pos.as<float4>()); GBSPH_COUNTED; }
    return cudaGetLastError();
}

cudaError_t cs_to_local_mixed(Ctx &c, u32 n, f64 *dst) {
    { k_cs_to_local<<<div_up(n, 256), 256, 0, c.stream>>>(n, c.row_rank.as<u32>(), c.row_local.as<u32>(),
                                                         c.f_aux2.as<float>(), dst); GBSPH_COUNTED; }
    return cudaGetLastError();
}

cudaError_t derivs_mixed_module(Ctx &c, const RowSpace &rs, const HydroSpace &hs, f64 pmass,
                                f64 alpha_u, f64 alpha_AV, f64 beta_AV, f64 *ax, f64 *ay, f64 *az,
                                f64 *du, f64 *vsig) {
    // the caller's merged arrays hold c.n_obj entries (set from n_merged)
    u32 N = c.n_obj;
    cudaError_t e = ensure_mixed(c, N);
    if (e != cudaSuccess) return e;
    MixedSpace ms = mixed_space(c, N);
    { k_stage_hydro<<<div_up(N, 256), 256, 0, c.stream>>>(N, rs.x, rs.y, rs.z, hs, pmass,
                                                        c.f_pos.as<float4>(),
                                                        c.f_aux0.as<float4>()); GBSPH_COUNTED; }
    MixedParams p = mixed_params(pmass, alpha_u, alpha_AV, beta_AV);
    { k_derivs_mixed<<<div_up(rs.n, 128), 128, 0, c.stream>>>(rs, ms, p, pmass, ax, ay, az, du, vsig); GBSPH_COUNTED; }
    return cudaGetLastError();
}

// ---------------------------------------------------------------- allocation-free variant
// For callers that cannot allocate device memory: a host framework whose own pool owns
// every device byte, a solver loop that must not allocate once it is running, code that
// runs where the CUDA allocator may not be called.  They cannot create a gbsph_ctx (its
// scratch arena is allocated), so this entry point keeps the FP32 staging of the
// mixed-precision derivatives in a fixed device array that is part of the library image.
namespace {

// Largest merged (locals + ghosts) particle count the fixed staging holds.
constexpr u32 kNoAllocMaxMerged = 1u << 16;
// Four float4 per merged particle: 65,536 x 64 B = 4 MiB, reserved on every GPU that
// loads the library and kept until the process exits.
static __device__ __align__(256) float4 g_noalloc_staging[4 * kNoAllocMaxMerged];

} // namespace

} // namespace gbsph

extern "C" int gbsph_derivs_constAV_mixed_noalloc(
    const uint32_t *cnt, const uint32_t *scanned, const uint32_t *entries, const double *x,
    const double *y, const double *z, const double *vx, const double *vy, const double *vz,
    const double *h, const double *omega, const double *u, const double *P, const double *cs,
    uint32_t n_local, uint32_t n_merged, double pmass, double alpha_u, double alpha_AV,
    double beta_AV, double *ax, double *ay, double *az, double *du, double *vsig, void *stream) {
    using namespace gbsph;
    if (n_merged > kNoAllocMaxMerged) return GBSPH_ERR_CAPACITY; // beyond the fixed staging
    if (n_local > n_merged) return GBSPH_ERR_ARG;
    if (n_local == 0) return GBSPH_OK;
    // Set-up, on every call, with the caller's device current: in host code the array's
    // name is only a host-side handle, the kernels need its device address.  The address
    // belongs to the module loaded in the current context, so it is looked up each time
    // (a table lookup once the module is loaded) rather than cached per device: a cached
    // address would go stale after cudaDeviceReset or under another driver-API context on
    // the same device, and the lookup needs no host-side shared state.  The first call in
    // a context loads the module, which must not happen inside a stream capture.
    void *base    = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&base, g_noalloc_staging);
    if (e != cudaSuccess || !base) return GBSPH_ERR_CUDA;
    float4 *b     = (float4 *) base;
    u32 N         = n_merged;
    // N position records (2N float4) then N hydro records (2N float4)
    MixedSpace ms{b, b + 2 * (size_t) N};
    RowSpace rs{n_local, nullptr, nullptr, cnt, scanned, entries, x, y, z};
    HydroSpace hs{h, u, vx, vy, vz, omega, P, cs};
    cudaStream_t s = (cudaStream_t) stream;
    // every staging entry the pair kernel reads is rewritten first: nothing to clear
    { k_stage_hydro<<<div_up(N, 256), 256, 0, s>>>(N, x, y, z, hs, pmass, b, b + 2 * (size_t) N); GBSPH_COUNTED; }
    MixedParams p = mixed_params(pmass, alpha_u, alpha_AV, beta_AV);
    { k_derivs_mixed<<<div_up(n_local, 128), 128, 0, s>>>(rs, ms, p, pmass, ax, ay, az, du, vsig); GBSPH_COUNTED; }
    return cudaGetLastError() == cudaSuccess ? GBSPH_OK : GBSPH_ERR_CUDA;
}
