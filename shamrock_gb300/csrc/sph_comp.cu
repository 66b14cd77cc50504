// Compensated tier of the mixed-precision path: the sums that cancel are evaluated in
// double-float arithmetic on the FP32 pipes (df32.cuh), the rest stays FP32.
//
// Why: with a large uniform background pressure P0 (a sound wave, a cold disc at rest
// against its own pressure) the net force is a small residue of O(P0) pair terms.  The
// FP32 pair loop then errs by ~1e-7 times the sum of the term magnitudes, and, worse, an
// h carried to only ~1e-8 relative (the root of an FP32 density sum) moves rho, P and
// Omega of every neighbour by that much, which the cancellation amplifies alike.  On the
// 64^3 sound wave (P0 = 1, dP ~ 1e-4) the two give ~4e-3 relative force error, and a
// relative h noise of 1e-9 alone gives 1.6e-5.  This tier therefore
//   - finishes h with one Newton step from double-float density sums (the FP32 Newton
//     iteration leaves h within ~1e-7 of the root, one more step brings it to ~1e-14),
//     and computes Omega at that h from double-float sums (IterateSmoothingLengthDensity
//     .cpp:52-119 and ComputeOmega.cpp:36-73 evaluated exactly enough);
//   - stages per particle X = P / (rho^2 Omega), 1/h, 1/h^4, the pressure and the energy
//     as double-floats (FP64 arithmetic per particle, not per pair);
//   - splits the pressure force of UpdateDerivs.cpp:176-271 (forces.hpp:24-226) as
//       sum_b [(P_a + q_a) c1_a F_a + (P_b + q_b) c1_b F_b] r_hat
//         = X_a sum_b (F_a + F_b) r_hat
//         + sum_b [(X_b - X_a) F_b + q_a c1_a F_a + q_b c1_b F_b] r_hat,
//     the first (cancelling, geometric) sum in double-float, the second (small) one in
//     FP32, with X_b - X_a, P_a - P_b and u_a - u_b formed from the double-floats.
// On the 64^3 sound wave the tier agrees with the FP64 path to 2e-13 in h and 1e-6 in a
// and du/dt (what remains is the FP32 rounding of the remainder sum).
#include "df32.cuh"
#include "mixed_common.cuh"

namespace gbsph {

namespace {

constexpr f64 kDensRatio64 = kNorm3d / (kHfact * kHfact * kHfact);

__device__ __forceinline__ df df_from_f64(f64 v) {
    float hi, lo;
    split64(v, hi, lo);
    return df{hi, lo};
}

// component a - b of the separation of two hi/lo positions, as a double-float
__device__ __forceinline__ df sep_df(float ah, float al, float bh, float bl) {
    return df_add_f(two_sum(ah, -bh), al - bl);
}

__device__ __forceinline__ df r2_df(df dx, df dy, df dz) {
    return df_add(df_add(df_sqr(dx), df_sqr(dy)), df_sqr(dz));
}

// M4 over one row in double-float: S = sum f(q), G = sum (3 f + q f'), q = r / h_a,
// every neighbour with r <= 2 h_a including the particle itself (the reference's
// rab2 > h^2 R^2 exclusion).  With t = 2 - q:
//   q < 1:  f = 1 - 1.5 q^2 + 0.75 q^3,  3 f + q f' = 3 - 7.5 q^2 + 4.5 q^3
//   q < 2:  f = t^3 / 4,                  3 f + q f' = 1.5 t^2 (1 - q)
__device__ __forceinline__ void density_sums_df(const RowSpace &rs, const MixedSpace &ms, u32 a,
                                                u32 k0, u32 k1, df hinv2, df &S, df &G) {
    const F8 pa = ldg256(&ms.P[2 * (size_t) a]);
    S = G = df{0.f, 0.f};
    uint4 nx = (k0 < k1) ? load_entries(rs.ent, k0, k1, true, a) : make_uint4(a, a, a, a);
    for (u32 k = k0; k < k1; k += 4) {
        const u32 bb[4] = {nx.x, nx.y, nx.z, nx.w};
        F8 pb[4];
#pragma unroll
        for (int j = 0; j < 4; j++) pb[j] = ldg256(&ms.P[2 * (size_t) bb[j]]);
        if (k + 4 < k1) nx = load_entries(rs.ent, k + 4, k1, true, a);
#pragma unroll
        for (int j = 0; j < 4; j++) {
            if (k + j >= k1) continue;
            const df dx = sep_df(pa.a.x, pa.b.x, pb[j].a.x, pb[j].b.x);
            const df dy = sep_df(pa.a.y, pa.b.y, pb[j].a.y, pb[j].b.y);
            const df dz = sep_df(pa.a.z, pa.b.z, pb[j].a.z, pb[j].b.z);
            const df q2 = df_mul(r2_df(dx, dy, dz), hinv2);
            if (q2.hi > 4.f || (q2.hi == 4.f && q2.lo > 0.f)) continue;
            const df q = (q2.hi > 0.f) ? df_mul(q2, df_rsqrt(q2)) : df{0.f, 0.f};
            df f, g;
            if (q.hi < 1.f) {
                const df q3 = df_mul(q2, q);
                f = df_add_f(df_add(df_mul_f(q3, 0.75f), df_mul_f(q2, -1.5f)), 1.f);
                g = df_add_f(df_add(df_mul_f(q3, 4.5f), df_mul_f(q2, -7.5f)), 3.f);
            } else {
                const df t  = df_add_f(df_neg(q), 2.f);
                const df t2 = df_sqr(t);
                f = df_mul_f(df_mul(t2, t), 0.25f);
                g = df_mul_f(df_mul(t2, df_add_f(df_neg(q), 1.f)), 1.5f);
            }
            S = df_add(S, f);
            G = df_add(G, g);
        }
    }
}

// One Newton step of h from double-float sums (skipped for rows whose iteration did
// not converge, eps < 0), then Omega at the resulting h.  In the dimensionless form of
// the FP32 iteration: A = rho_sum / rho_h, B = h (d rho / dh) / rho_h,
// new_h = h (1 - (A - 1) / (B + 3)) with the reference's per-step and total limits, and
// Omega = 1 + B / 3.
__global__ void __launch_bounds__(256) k_dens_polish_df(RowSpace rs, MixedSpace ms,
                                                        const f64 *__restrict__ h_old,
                                                        f64 *__restrict__ h_row,
                                                        const f64 *__restrict__ eps,
                                                        f64 h_evol_max, f64 h_evol_iter_max,
                                                        f64 *__restrict__ omega_local) {
    u32 t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= rs.n) return;
    const u32 a  = rs.row_rank[t];
    const u32 k0 = rs.off[t], k1 = k0 + rs.cnt[t];
    f64 h = h_row[t];
    df S, G;
    if (!(eps[t] < 0)) {
        const f64 hinv = 1.0 / h;
        density_sums_df(rs, ms, a, k0, k1, df_from_f64(hinv * hinv), S, G);
        const f64 A = kDensRatio64 * df_to_f64(S), B = -kDensRatio64 * df_to_f64(G);
        f64 d = (A - 1) / (B + 3);
        const f64 f = 1 - d;
        if (f < 1 / h_evol_iter_max) d = 1 - 1 / h_evol_iter_max;
        if (f > h_evol_iter_max) d = 1 - h_evol_iter_max;
        const f64 new_h = h - h * d;
        if (new_h < h_old[t] * h_evol_max) h = new_h;
        h_row[t] = h;
    }
    const f64 hinv = 1.0 / h;
    density_sums_df(rs, ms, a, k0, k1, df_from_f64(hinv * hinv), S, G);
    omega_local[rs.row_local[t]] = 1 - kDensRatio64 * df_to_f64(G) / 3;
}

// m4_df(q) / r in double-float for q = r / h: h^-1 (-3 + 2.25 q) below 1,
// -0.75 (2 - q)^2 / r below 2, else 0
__device__ __forceinline__ df m4_df_over_r(df q, df hinv, df rinv) {
    if (q.hi < 1.f) return df_mul(hinv, df_add_f(df_mul_f(q, 2.25f), -3.f));
    if (q.hi < 2.f) return df_mul(df_mul_f(df_sqr(df_add_f(df_neg(q), 2.f)), -0.75f), rinv);
    return df{0.f, 0.f};
}

// Compensated constant-AV derivatives of one row (same pair set, v_sig and records as
// derivs_row_f32, plus the E records {X_hi, X_lo, (1/h)_lo, P_lo}{u_lo, (1/h^4)_hi,
// (1/h^4)_lo, 0}).  Returns the bare force F = X_a G / pi + R with G the double-float
// geometric sum sum_b (h_a^-4 m4'(q_a) + h_b^-4 m4'(q_b)) (r_ab / r) and R the FP32
// remainder, the bare du/dt sum U, the v_sig maximum and the condition sums of the FP32
// tier (as derivs_row_f32, so the step can tell when that tier would do).
template<bool COND>
__device__ __forceinline__ void derivs_row_comp(const RowSpace &rs, const MixedSpace &ms,
                                                const float4 *__restrict__ E, u32 a, u32 k0,
                                                u32 k1, const MixedParams &p, f64 &Fx, f64 &Fy,
                                                f64 &Fz, float &U, float &vsig_max, float &sa,
                                                float &su, const float *__restrict__ cs_rank) {
    const F8 pa = ldg256(&ms.P[2 * (size_t) a]);
    const F8 ha = ldg256(&ms.H[2 * (size_t) a]);
    const F8 ea = ldg256(&E[2 * (size_t) a]);
    const float hia = pa.a.w, cs_a = pa.b.w;
    const float hia2 = hia * hia;
    const float rho_a = p.mh3 * hia2 * hia;
    const df X_a     = df{ea.a.x, ea.a.y};
    const df hinv_a  = df{hia, ea.a.z};
    const df h4_a    = df{ea.b.y, ea.b.z};
    const float Pa_hi = ha.b.x, Pa_lo = ea.a.w;
    const float ua_hi = ha.a.w, ua_lo = ea.b.x;
    const float c1a = ha.b.y, c2a = c1a * rho_a;
    const float vla_x = bf_hi(ha.b.z), vla_y = bf_lo(ha.b.z), vla_z = bf_hi(ha.b.w);
    const float k4a = hia2 * hia2 * kNorm3dF;
    const float cs_sig = cs_rank ? cs_rank[a] : cs_a;
    const float abs_ua = fabsf(ua_hi);
    df Gx{0.f, 0.f}, Gy{0.f, 0.f}, Gz{0.f, 0.f};
    float Rx = 0.f, Ry = 0.f, Rz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f, cu = 0.f;
    U = 0.f;
    vsig_max = 0.f;
    sa = su = 0.f;
    uint4 nx = (k0 < k1) ? load_entries(rs.ent, k0, k1, true, a) : make_uint4(a, a, a, a);
    for (u32 k = k0; k < k1; k += 4) {
        const u32 bb[4] = {nx.x, nx.y, nx.z, nx.w};
        float bx = 0.f, by = 0.f, bz = 0.f, bu = 0.f;
#pragma unroll
        for (int half = 0; half < 2; half++) {
            // two neighbours' three records per round trip (96 registers for four)
            F8 pb[2], hb[2], eb[2];
#pragma unroll
            for (int j = 0; j < 2; j++) {
                const size_t r2i = 2 * (size_t) bb[2 * half + j];
                pb[j] = ldg256(&ms.P[r2i]);
                hb[j] = ldg256(&ms.H[r2i]);
                eb[j] = ldg256(&E[r2i]);
            }
            if (half == 0 && k + 4 < k1) nx = load_entries(rs.ent, k + 4, k1, true, a);
#pragma unroll
            for (int j = 0; j < 2; j++) {
                const df dx = sep_df(pa.a.x, pa.b.x, pb[j].a.x, pb[j].b.x);
                const df dy = sep_df(pa.a.y, pa.b.y, pb[j].a.y, pb[j].b.y);
                const df dz = sep_df(pa.a.z, pa.b.z, pb[j].a.z, pb[j].b.z);
                const float fdx = dx.hi, fdy = dy.hi, fdz = dz.hi;
                const float r2 = fdx * fdx + fdy * fdy + fdz * fdz;
                const float hib = pb[j].a.w, cs_b = pb[j].b.w;
                const float hib2 = hib * hib;
                if (k + 2 * half + j >= k1 || r2 == 0.f || (r2 * hia2 > 4.f && r2 * hib2 > 4.f))
                    continue;
                // ---- geometric sum in double-float
                const df r2d  = r2_df(dx, dy, dz);
                const df rinv = df_rsqrt(r2d);
                const df r    = df_mul(r2d, rinv);
                const df hinv_b = df{hib, eb[j].a.z};
                const df Ta = m4_df_over_r(df_mul(r, hinv_a), hinv_a, rinv);
                const df Tb = m4_df_over_r(df_mul(r, hinv_b), hinv_b, rinv);
                const df K  = df_add(df_mul(h4_a, Ta), df_mul(df{eb[j].b.y, eb[j].b.z}, Tb));
                Gx = df_add(Gx, df_mul(K, dx));
                Gy = df_add(Gy, df_mul(K, dy));
                Gz = df_add(Gz, df_mul(K, dz));
                // ---- FP32 remainder: (X_b - X_a) F_b and the viscous parts
                const float rinvf = rinv.hi;
                const float rab   = r.hi;
                const float rho_b = p.mh3 * hib2 * hib;
                const float c1b = hb[j].b.y, c2b = c1b * rho_b;
                float Fa = k4a * m4_df32(rab * hia);
                float Fb = (hib2 * hib2) * kNorm3dF * m4_df32(rab * hib);
                float vx = (ha.a.x - hb[j].a.x) + (vla_x - bf_hi(hb[j].b.z));
                float vy = (ha.a.y - hb[j].a.y) + (vla_y - bf_lo(hb[j].b.z));
                float vz = (ha.a.z - hb[j].a.z) + (vla_z - bf_hi(hb[j].b.w));
                float vr  = (vx * fdx + vy * fdy + vz * fdz) * rinvf;
                float avr = fabsf(vr);
                float vsig_a = p.alpha_AV * cs_a + p.beta_AV * avr;
                float vsig_b = p.alpha_AV * cs_b + p.beta_AV * avr;
                float dP     = (Pa_hi - hb[j].b.x) + (Pa_lo - eb[j].a.w);
                float vsig_u = sqrt_approx(fabsf(dP) * __fdividef(2.f, rho_a + rho_b));
                float qa = fmaxf(-0.5f * rho_a * vsig_a * vr, 0.f);
                float qb = fmaxf(-0.5f * rho_b * vsig_b * vr, 0.f);
                float dX = (eb[j].a.x - X_a.hi) + (eb[j].a.y - X_a.lo);
                float pf = dX * Fb + qa * c1a * Fa + qb * c1b * Fb;
                float f  = pf * rinvf;
                bx += f * fdx;
                by += f * fdy;
                bz += f * fdz;
                const float du_ab = (ua_hi - hb[j].a.w) + (ua_lo - eb[j].b.x);
                const float tp = (X_a.hi + qa * c1a) * Fa * vr;
                const float tc = 0.5f * p.alpha_u * vsig_u * (Fa * c2a + Fb * c2b);
                bu += tp + tc * du_ab;
                vsig_max = fmaxf(vsig_max, cs_sig + 2.f * avr);
                if (COND) {
                    sa += fabsf(X_a.hi * (Fa + Fb) + pf);
                    su += fabsf(tp) + fabsf(tc) * (abs_ua + fabsf(hb[j].a.w));
                }
            }
        }
        kahan_add(Rx, cx, bx);
        kahan_add(Ry, cy, by);
        kahan_add(Rz, cz, bz);
        kahan_add(U, cu, bu);
    }
    Fx = df_to_f64(df_mul(X_a, Gx)) * kNorm3d + (f64) Rx;
    Fy = df_to_f64(df_mul(X_a, Gy)) * kNorm3d + (f64) Ry;
    Fz = df_to_f64(df_mul(X_a, Gz)) * kNorm3d + (f64) Rz;
}

// Compensated derivatives + v_sig + leapfrog corrector + CFL, the counterpart of
// k_derivs_step_mixed (same outputs and reductions)
template<bool COND>
__global__ void __launch_bounds__(128) k_derivs_step_comp(RowSpace rs, MixedSpace ms,
                                                          const float4 *__restrict__ E,
                                                          MixedParams p, f64 pmass,
                                                          const f64 *__restrict__ h_rank, f64 hdt,
                                                          f64 C_cour, f64 C_force, LocalFields lf,
                                                          ExtAccel ext, Scalars *sc,
                                                          const float *__restrict__ cs_rank) {
    u32 t = blockIdx.x * blockDim.x + threadIdx.x;
    u64 ev2 = 0, dtm = ~0ull;
    float v2 = 0.f;
    float c_fa = 0.f, c_fu = 0.f, c_a = 0.f, c_du = 0.f;
    if (t < rs.n) {
        u32 a  = rs.row_rank[t];
        u32 k0 = rs.off[t], k1 = k0 + rs.cnt[t];
        f64 Fx, Fy, Fz;
        float U, vm, sa, su;
        derivs_row_comp<COND>(rs, ms, E, a, k0, k1, p, Fx, Fy, Fz, U, vm, sa, su, cs_rank);
        if (COND) {
            c_fa = sa;
            c_fu = su;
            c_a  = (float) sqrt(Fx * Fx + Fy * Fy + Fz * Fz);
            c_du = fabsf(U);
        }
        f64 fx = -pmass * Fx, fy = -pmass * Fy, fz = -pmass * Fz;
        f64 tdu = pmass * (f64) U;
        u32 i   = rs.row_local[t];
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

} // namespace

cudaError_t dens_polish_df(Ctx &c, const RowSpace &rs, const f64 *h_old, f64 *h_row, const f64 *eps,
                           f64 h_evol_max, f64 h_evol_iter_max, f64 *omega_local) {
    ProfScope ps(c, kProfOmega, rs.n);
    MixedSpace ms{c.f_pos.as<float4>(), c.f_aux0.as<float4>()};
    { k_dens_polish_df<<<div_up(rs.n, 256), 256, 0, c.stream>>>(rs, ms, h_old, h_row, eps, h_evol_max,
                                                               h_evol_iter_max, omega_local); GBSPH_COUNTED; }
    return cudaGetLastError();
}

cudaError_t derivs_step_comp(Ctx &c, const RowSpace &rs, f64 pmass, f64 alpha_u, f64 alpha_AV,
                             f64 beta_AV, f64 hdt, f64 C_cour, f64 C_force, const LocalFields &lf,
                             const ExtAccel &ext, bool varying_av, bool cond) {
    MixedSpace ms{c.f_pos.as<float4>(), c.f_aux0.as<float4>()};
    MixedParams p = mixed_params(pmass, alpha_u, varying_av ? 1.0 : alpha_AV, beta_AV);
    const float *cs_rank = varying_av ? c.f_aux2.as<float>() : nullptr;
    ProfScope ps(c, kProfDerivs, rs.n);
    auto kern = cond ? k_derivs_step_comp<true> : k_derivs_step_comp<false>;
    { kern<<<div_up(rs.n, 128), 128, 0, c.stream>>>(
        rs, ms, c.f_comp.as<float4>(), p, pmass, c.sh2.as<f64>(), hdt, C_cour, C_force, lf, ext,
        c.d_scalars.as<Scalars>(), cs_rank); GBSPH_COUNTED; }
    return cudaGetLastError();
}

} // namespace gbsph
