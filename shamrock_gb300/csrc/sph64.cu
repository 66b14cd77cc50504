// FP64 SPH pair kernels and integrator.  This translation unit is compiled with
// fused multiply-add disabled so that every expression rounds exactly as the cited
// reference line (and the oracle) evaluates it; the FP64 path is bit-identical to
// the oracle for the same neighbour order.
//
//   h-rho Newton step  shammodels/sph/src/modules/IterateSmoothingLengthDensity.cpp:52-119
//                      shammodels/sph/include/shammodels/sph/math/density.hpp:22-41
//   Omega              shammodels/sph/src/modules/ComputeOmega.cpp:36-73
//   EOS (adiabatic)    shammodels/sph/src/modules/ComputeEos.cpp:162-172,219-236
//   derivatives        shammodels/sph/src/modules/UpdateDerivs.cpp:176-271,
//                      shammodels/sph/include/shammodels/sph/math/forces.hpp:24-226, q_ab.hpp:36-39
//   v_sig              shammodels/sph/src/Solver.cpp:2716-2788
//   CFL                ComputeCFLCourant.hpp:45-60, ComputeCFLForce.hpp:50-62
//   corrector          shamrock/src/math/integrators.cpp:88-120, Solver.cpp:2506-2616
//   predictor + wrap   Solver.cpp:390-524, ForwardEuler.hpp:62-84, integrators.cpp:207-237

#include "gbsph_ctx.cuh"
#include "sph_kernels.cuh"

namespace gbsph {

namespace {

// ---------------------------------------------------------------- M4 (FP64)
__device__ __forceinline__ f64 m4_f(f64 q) {
    f64 t1 = 2 - q;
    f64 t2 = 1 - q;
    t1     = t1 * t1 * t1;
    t2     = t2 * t2 * t2;
    const f64 div1_4 = (1. / 4.);
    t1 *= div1_4;
    t2 *= -1;
    if (q < 1) return t1 + t2;
    else if (q < 2) return t1;
    return 0;
}
__device__ __forceinline__ f64 m4_df(f64 q) {
    const f64 div9_4 = (9. / 4.);
    const f64 div3_4 = (3. / 4.);
    if (q < 1) return -3 * q + div9_4 * q * q;
    else if (q < 2) return -3 + 3 * q - div3_4 * q * q;
    return 0;
}
__device__ __forceinline__ f64 W_3d(f64 r, f64 h) { return kNorm3d * m4_f(r / h) / (h * h * h); }
__device__ __forceinline__ f64 dW_3d(f64 r, f64 h) {
    return kNorm3d * m4_df(r / h) / (h * h * h * h);
}
__device__ __forceinline__ f64 dhW_3d(f64 r, f64 h) {
    return -(kNorm3d) * (3 * m4_f(r / h) + (r / h) * m4_df(r / h)) / (h * h * h * h);
}
__device__ __forceinline__ f64 rho_h(f64 m, f64 h) {
    return m * (kHfact / h) * (kHfact / h) * (kHfact / h);
}
__device__ __forceinline__ f64 inv_sat_positive(f64 v) { return (v >= 1e-9) ? 1. / v : 0.; }
__device__ __forceinline__ f64 inv_sat_zero(f64 v) { return (v != 0 && v == v) ? 1. / v : 0.; }

// ---------------------------------------------------------------- density sums
__device__ __forceinline__ void density_sums(const RowSpace &rs, u32 a, u32 k0, u32 k1, f64 h_a,
                                             f64 pmass, f64 &rho_sum, f64 &sumdWdh) {
    f64 xa = rs.x[a], ya = rs.y[a], za = rs.z[a];
    f64 dint = h_a * h_a * kRkern * kRkern;
    rho_sum  = 0;
    sumdWdh  = 0;
    for (u32 k = k0; k < k1; k++) {
        u32 b    = rs.ent[k];
        f64 dx   = xa - rs.x[b], dy = ya - rs.y[b], dz = za - rs.z[b];
        f64 rab2 = dx * dx + dy * dy + dz * dz;
        if (rab2 > dint) continue;
        f64 rab = sqrt(rab2);
        rho_sum += pmass * W_3d(rab, h_a);
        sumdWdh += pmass * dhW_3d(rab, h_a);
    }
}

// ITERS Newton iterations per row (the reference's global loop is equivalent per
// particle: a particle's update reads only its own h, so it iterates until its own
// eps <= eps_p (1e-6 in the reference), becomes -1, or the iteration cap is reached).
__global__ void __launch_bounds__(256) k_h_iterate(RowSpace rs, const f64 *__restrict__ h_old,
                                                   f64 *__restrict__ h_new, f64 *__restrict__ eps,
                                                   f64 pmass, f64 h_evol_max, f64 h_evol_iter_max,
                                                   u32 iters, f64 eps_p, Scalars *sc) {
    u32 t = blockIdx.x * blockDim.x + threadIdx.x;
    u64 emax = 0, emin = ~0ull;
    u32 used = 0;
    if (t < rs.n) {
        u32 a  = rs.row_rank ? rs.row_rank[t] : t;
        u32 k0 = rs.off[t], k1 = k0 + rs.cnt[t];
        const f64 h_max_tot_max_evol = h_evol_max;
        const f64 h_max_evol_p       = h_evol_iter_max;
        const f64 h_max_evol_m       = 1 / h_evol_iter_max;
        f64 ha_0 = h_old[t];
        f64 h_a  = h_new[t];
        f64 e    = eps[t];
        for (u32 it = 0; it < iters; it++) {
            if (!(e > eps_p)) break;
            used++;
            f64 rho_sum, sumdWdh;
            density_sums(rs, a, k0, k1, h_a, pmass, rho_sum, sumdWdh);
            f64 rho_ha  = rho_h(pmass, h_a);
            f64 f_iter  = rho_sum - rho_ha;
            f64 df_iter = sumdWdh + 3 * rho_ha / h_a;
            f64 new_h   = h_a - f_iter / df_iter;
            if (new_h < h_a * h_max_evol_m) new_h = h_max_evol_m * h_a;
            if (new_h > h_a * h_max_evol_p) new_h = h_max_evol_p * h_a;
            if (new_h < ha_0 * h_max_tot_max_evol) {
                e   = fabs(new_h - h_a) / ha_0;
                h_a = new_h;
            } else {
                h_a = ha_0 * h_max_tot_max_evol;
                e   = -1;
            }
        }
        h_new[t] = h_a;
        eps[t]   = e;
        emax     = f64_to_ordered(e);
        emin     = emax;
    }
    emax = block_reduce(emax, OpMaxU64{}, 0ull);
    emin = block_reduce(emin, OpMinU64{}, ~0ull);
    u32 um = block_reduce((u64) used, OpMaxU64{}, 0ull);
    if (threadIdx.x == 0) {
        atomicMax((unsigned long long *) &sc->eps_max, (unsigned long long) emax);
        atomicMin((unsigned long long *) &sc->eps_min, (unsigned long long) emin);
        atomicMax(&sc->iters_max, um);
    }
}

__global__ void __launch_bounds__(256) k_omega(RowSpace rs, const f64 *__restrict__ h_row,
                                               f64 pmass, f64 *__restrict__ omega_out,
                                               const u32 *__restrict__ out_index) {
    u32 t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= rs.n) return;
    u32 a  = rs.row_rank ? rs.row_rank[t] : t;
    u32 k0 = rs.off[t], k1 = k0 + rs.cnt[t];
    f64 h_a = h_row[t];
    f64 rho_sum, part_omega_sum;
    density_sums(rs, a, k0, k1, h_a, pmass, rho_sum, part_omega_sum);
    f64 rho_ha  = rho_h(pmass, h_a);
    f64 omega_a = 1 + (h_a / (3 * rho_ha)) * part_omega_sum;
    omega_out[out_index ? out_index[t] : t] = omega_a;
}

// gather h, u, v, omega of locals and ghosts into rank order + adiabatic EOS
__global__ void k_gather_eos(const u32 *__restrict__ sort_index, u32 N, u32 n_local,
                             const u32 *__restrict__ ghost_src, const f64 *__restrict__ h,
                             const f64 *__restrict__ u, const f64 *__restrict__ vx,
                             const f64 *__restrict__ vy, const f64 *__restrict__ vz, u32 vs,
                             const f64 *__restrict__ omega, f64 pmass, EosParams eos,
                             const f64 *__restrict__ sx, const f64 *__restrict__ sy,
                             const f64 *__restrict__ sz,
                             f64 *__restrict__ sh, f64 *__restrict__ su, f64 *__restrict__ svx,
                             f64 *__restrict__ svy, f64 *__restrict__ svz, f64 *__restrict__ som,
                             f64 *__restrict__ sP, f64 *__restrict__ scs, f64 *__restrict__ srho,
                             f64 *__restrict__ sinv, f64 *__restrict__ srom) {
    u32 r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= N) return;
    u32 id  = sort_index[r];
    u32 src = id < n_local ? id : ghost_src[id - n_local];
    f64 hh = h[src], uu = u[src];
    sh[r]  = hh;
    su[r]  = uu;
    svx[r] = vx[(size_t) src * vs];
    svy[r] = vy[(size_t) src * vs];
    svz[r] = vz[(size_t) src * vs];
    const f64 om = omega[src];
    som[r] = om;
    f64 rho = rho_h(pmass, hh);
    if (srho) {
        // the pair loop's per-neighbour factors, in its own expressions (derivs_row)
        srho[r] = rho;
        sinv[r] = inv_sat_zero((rho * rho) * om);
        srom[r] = rho * om;
    }
    if (eos.kind == 1) {
        // LP07 at the merged (rank-ordered) position
        f64 x = sx[r], y = sy[r], z = sz[r];
        f64 Rsq   = x * x + y * y + z * z;
        f64 cs_sq = (eos.cs0 * eos.cs0) * pow(Rsq / (eos.r0 * eos.r0), -eos.q);
        sP[r]     = cs_sq * rho;
        scs[r]    = sqrt(cs_sq);
    } else {
        f64 P  = (eos.gamma - 1) * rho * uu;
        sP[r]  = P;
        scs[r] = sqrt(eos.gamma * P / rho);
    }
}

__global__ void k_eos_lp07(u32 n, const f64 *__restrict__ x, const f64 *__restrict__ y,
                           const f64 *__restrict__ z, u32 vs, const f64 *__restrict__ h, f64 pmass,
                           f64 cs0, f64 r0, f64 q, f64 *__restrict__ P, f64 *__restrict__ cs) {
    u32 i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    size_t iv = (size_t) i * vs;
    f64 a = x[iv], b = y[iv], c = z[iv];
    f64 Rsq   = a * a + b * b + c * c;
    f64 cs_sq = (cs0 * cs0) * pow(Rsq / (r0 * r0), -q);
    P[i]      = cs_sq * rho_h(pmass, h[i]);
    cs[i]     = sqrt(cs_sq);
}

__global__ void k_eos(u32 n, const f64 *__restrict__ h, const f64 *__restrict__ u, f64 pmass,
                      f64 gamma, f64 *__restrict__ P, f64 *__restrict__ cs) {
    u32 i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    f64 rho = rho_h(pmass, h[i]);
    f64 Pa  = (gamma - 1) * rho * u[i];
    P[i]    = Pa;
    cs[i]   = sqrt(gamma * Pa / rho);
}

// ---------------------------------------------------------------- derivatives
struct DerivParams {
    f64 pmass, alpha_u, alpha_AV, beta_AV;
    f64 hdt;             // dt / 2 for the corrector
    f64 C_cour, C_force; // CFL factors (already x cfl multiplier)
    ExtAccel ext;        // external acceleration added to the hydro one (may be null)
};

// PRE: the neighbour's rho, inv_sat_zero(rho^2 Omega) and rho Omega are read from the
// staged per-particle factors (hs.rho, hs.inv_sub, hs.rho_om) instead of recomputed per
// pair: the same expressions evaluated once, so the same bits, and two FP64 divisions and
// five multiplications fewer per pair on GB300's scarce FP64 pipe.
template<bool VSIG, bool PRE = false>
__device__ __forceinline__ void derivs_row(const RowSpace &rs, const HydroSpace &hs, u32 a, u32 k0,
                                           u32 k1, const DerivParams &p, f64 &fx, f64 &fy, f64 &fz,
                                           f64 &tdu, f64 &vsig_max) {
    const f64 Rker2 = kRkern * kRkern;
    f64 h_a = hs.h[a];
    f64 xa = rs.x[a], ya = rs.y[a], za = rs.z[a];
    f64 vxa = hs.vx[a], vya = hs.vy[a], vza = hs.vz[a];
    f64 P_a = hs.P[a], omega_a = hs.omega[a];
    const f64 u_a         = hs.u[a];
    f64 rho_a             = rho_h(p.pmass, h_a);
    f64 rho_a_sq          = rho_a * rho_a;
    f64 rho_a_inv         = 1. / rho_a;
    f64 omega_a_rho_a_inv = 1 / (omega_a * rho_a);
    f64 cs_a              = hs.cs[a];
    const f64 alpha_a     = hs.alpha ? hs.alpha[a] : p.alpha_AV;
    fx = fy = fz = tdu = 0;
    vsig_max           = 0;
    for (u32 k = k0; k < k1; k++) {
        u32 b    = rs.ent[k];
        f64 dx   = xa - rs.x[b], dy = ya - rs.y[b], dz = za - rs.z[b];
        f64 rab2 = dx * dx + dy * dy + dz * dz;
        f64 h_b  = hs.h[b];
        if (rab2 > h_a * h_a * Rker2 && rab2 > h_b * h_b * Rker2) continue;
        f64 rab       = sqrt(rab2);
        const f64 u_b = hs.u[b];
        f64 rho_b   = PRE ? hs.rho[b] : rho_h(p.pmass, h_b);
        f64 P_b     = hs.P[b];
        f64 cs_b    = hs.cs[b];
        f64 Fab_a   = dW_3d(rab, h_a);
        f64 Fab_b   = dW_3d(rab, h_b);
        f64 vx = vxa - hs.vx[b], vy = vya - hs.vy[b], vz = vza - hs.vz[b];
        f64 inv = inv_sat_positive(rab);
        f64 rx = dx * inv, ry = dy * inv, rz = dz * inv;
        f64 v_ab_r_ab     = vx * rx + vy * ry + vz * rz;
        f64 abs_v_ab_r_ab = fabs(v_ab_r_ab);
        // varying AV: alpha_a, alpha_b per particle (NodeUpdateDerivsVaryingAlphaAV.cpp:95-96)
        const f64 alpha_b = hs.alpha ? hs.alpha[b] : p.alpha_AV;
        f64 vsig_a  = alpha_a * cs_a + p.beta_AV * abs_v_ab_r_ab;
        f64 vsig_b  = alpha_b * cs_b + p.beta_AV * abs_v_ab_r_ab;
        f64 rho_avg = (rho_a + rho_b) * 0.5;
        f64 abs_dp  = fabs(P_a - P_b);
        f64 vsig_u  = sqrt(abs_dp / rho_avg);
        f64 qa_ab   = fmax(-f64(0.5) * rho_a * vsig_a * v_ab_r_ab, f64(0));
        f64 qb_ab   = fmax(-f64(0.5) * rho_b * vsig_b * v_ab_r_ab, f64(0));
        f64 AV_P_a  = P_a + qa_ab;
        f64 AV_P_b  = P_b + qb_ab;
        f64 sub_fact_a = rho_a_sq * omega_a;
        f64 ca = AV_P_a * inv_sat_zero(sub_fact_a);
        f64 cb;
        if (PRE) {
            cb = AV_P_b * hs.inv_sub[b];
        } else {
            f64 sub_fact_b = (rho_b * rho_b) * hs.omega[b];
            cb = AV_P_b * inv_sat_zero(sub_fact_b);
        }
        f64 nax = rx * Fab_a, nay = ry * Fab_a, naz = rz * Fab_a;
        f64 nbx = rx * Fab_b, nby = ry * Fab_b, nbz = rz * Fab_b;
        f64 mb = -p.pmass;
        fx += mb * (ca * nax + cb * nbx);
        fy += mb * (ca * nay + cb * nby);
        fz += mb * (ca * naz + cb * nbz);
        f64 dotvg = vx * nax + vy * nay + vz * naz;
        tdu += AV_P_a * (omega_a_rho_a_inv * rho_a_inv) * p.pmass * dotvg;
        f64 Fa = Fab_a * omega_a_rho_a_inv;
        f64 Fb = Fab_b / (PRE ? hs.rho_om[b] : rho_b * hs.omega[b]);
        tdu += p.pmass * p.alpha_u * vsig_u * (u_a - u_b) * f64(0.5) * (Fa + Fb);
        if (VSIG) {
            // separate v_sig kernel of the reference: r_hat = dr / r, zero below 1e-9,
            // alpha = 1, beta = 2 fixed
            f64 ux = dx / rab, uy = dy / rab, uz = dz / rab;
            if (rab < 1e-9) ux = uy = uz = 0;
            f64 vr = vx * ux + vy * uy + vz * uz;
            f64 vs = 1.0 * cs_a + 2.0 * fabs(vr);
            vsig_max = fmax(vsig_max, vs);
        }
    }
}

// module form: reference CSR, outputs a, du (and vsig) by row
__global__ void __launch_bounds__(128) k_derivs(RowSpace rs, HydroSpace hs, DerivParams p,
                                                f64 *__restrict__ ax, f64 *__restrict__ ay,
                                                f64 *__restrict__ az, f64 *__restrict__ du,
                                                f64 *__restrict__ vsig) {
    u32 t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= rs.n) return;
    u32 a  = rs.row_rank ? rs.row_rank[t] : t;
    u32 k0 = rs.off[t], k1 = k0 + rs.cnt[t];
    f64 fx, fy, fz, tdu, vm;
    if (vsig) derivs_row<true>(rs, hs, a, k0, k1, p, fx, fy, fz, tdu, vm);
    else derivs_row<false>(rs, hs, a, k0, k1, p, fx, fy, fz, tdu, vm);
    ax[t] = fx;
    ay[t] = fy;
    az[t] = fz;
    du[t] = tdu;
    if (vsig) vsig[t] = vm;
}

// pipeline form: derivatives + v_sig + leapfrog corrector + CFL, outputs to the
// caller's local arrays.  Neighbour velocities come from the rank-ordered copy
// taken before the corrector, so correcting the caller's v here is race-free.
template<bool PRE>
__global__ void __launch_bounds__(128) k_derivs_step(RowSpace rs, HydroSpace hs, DerivParams p,
                                                     LocalFields lf, Scalars *sc) {
    u32 t = blockIdx.x * blockDim.x + threadIdx.x;
    u64 ev2 = 0, dtm = ~0ull;
    f64 v2  = 0;
    if (t < rs.n) {
        u32 a  = rs.row_rank[t];
        u32 k0 = rs.off[t], k1 = k0 + rs.cnt[t];
        f64 fx, fy, fz, tdu, vm;
        derivs_row<true, PRE>(rs, hs, a, k0, k1, p, fx, fy, fz, tdu, vm);
        u32 i  = rs.row_local[t];
        size_t iv = (size_t) i * lf.vs;
        if (p.ext.x) {
            // axyz += axyz_ext (ExternalForces.cpp:342-359)
            fx = fx + p.ext.x[i];
            fy = fy + p.ext.y[i];
            fz = fz + p.ext.z[i];
        }
        f64 ox = lf.ax[iv], oy = lf.ay[iv], oz = lf.az[iv], odu = lf.du[i];
        lf.ax[iv] = fx;
        lf.ay[iv] = fy;
        lf.az[iv] = fz;
        lf.du[i]  = tdu;
        // corrector (integrators.cpp:88-120): incr = hdt * (new - old)
        f64 ix = p.hdt * (fx - ox), iy = p.hdt * (fy - oy), iz = p.hdt * (fz - oz);
        f64 nvx = lf.vx[iv] + ix, nvy = lf.vy[iv] + iy, nvz = lf.vz[iv] + iz;
        lf.vx[iv] = nvx;
        lf.vy[iv] = nvy;
        lf.vz[iv] = nvz;
        f64 iu    = p.hdt * (tdu - odu);
        lf.u[i]   = lf.u[i] + iu;
        ev2       = f64_to_ordered(ix * ix + iy * iy + iz * iz);
        v2        = nvx * nvx + nvy * nvy + nvz * nvz;
        // CFL with the new acceleration
        f64 h_a  = hs.h[a];
        f64 dt   = __longlong_as_double(0x7ff0000000000000ll);
        f64 dt_c = p.C_cour * h_a / vm;
        dt       = fmin(dt, dt_c);
        f64 abs_a = sqrt(fx * fx + fy * fy + fz * fz);
        f64 dt_f  = p.C_force * sqrt(h_a / abs_a);
        dt        = fmin(dt, dt_f);
        dtm       = f64_to_ordered(dt);
    }
    ev2 = block_reduce(ev2, OpMaxU64{}, 0ull);
    dtm = block_reduce(dtm, OpMinU64{}, ~0ull);
    v2  = block_reduce(v2, OpAddF64{}, 0.0);
    if (threadIdx.x == 0) {
        atomicMax((unsigned long long *) &sc->epsv2_max, (unsigned long long) ev2);
        atomicMin((unsigned long long *) &sc->dt_min, (unsigned long long) dtm);
        atomicAdd(&sc->sum_v2, v2);
    }
}

// leapfrog predictor (half kick, drift, half kick) + periodic wrap, one pass
// fmod(r, d) for d > 0.  fmod is exact (its result is r - n d, which is representable),
// so any exact evaluation gives the same bits: within one period of the box, the
// remainder is r itself or r -+ d (exact by Sterbenz's lemma: d <= |r| <= 2 d); further
// out, and for NaN or infinities, the library fmod decides.  A zero result takes the sign
// of r, as fmod's does.
__device__ __forceinline__ f64 fmod_wrap(f64 r, f64 d) {
    if (fabs(r) < d) return r;
    if (r >= d && r < 2 * d) return r - d;
    if (r <= -d && r > -2 * d) {
        const f64 t = r + d;
        return t == 0 ? -0.0 : t;
    }
    return fmod(r, d);
}

__global__ void k_predict(LocalFields lf, u32 n, f64 dt, int periodic, f64 b0, f64 b1, f64 b2,
                          f64 e0, f64 e1, f64 e2, f64 mGM, f64 *__restrict__ ext_x,
                          f64 *__restrict__ ext_y, f64 *__restrict__ ext_z) {
    u32 i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    size_t iv   = (size_t) i * lf.vs;
    f64 dt_half = dt / 2;
    f64 ax = lf.ax[iv], ay = lf.ay[iv], az = lf.az[iv], dd = lf.du[i];
    f64 vx = lf.vx[iv], vy = lf.vy[iv], vz = lf.vz[iv], u = lf.u[i];
    vx = vx + dt_half * ax;
    vy = vy + dt_half * ay;
    vz = vz + dt_half * az;
    u  = u + dt_half * dd;
    f64 x = lf.x[iv] + dt * vx, y = lf.y[iv] + dt * vy, z = lf.z[iv] + dt * vz;
    vx = vx + dt_half * ax;
    vy = vy + dt_half * ay;
    vz = vz + dt_half * az;
    u  = u + dt_half * dd;
    if (ext_x) {
        // central point mass at the drifted position, before the wrap
        f64 r  = sqrt(x * x + y * y + z * z);
        f64 r3 = r * r * r;
        ext_x[i] = mGM * x / r3;
        ext_y[i] = mGM * y / r3;
        ext_z[i] = mGM * z / r3;
    }
    if (periodic) {
        f64 bmin[3] = {b0, b1, b2}, bmax[3] = {e0, e1, e2};
        f64 p[3]    = {x, y, z};
        for (int c = 0; c < 3; c++) {
            f64 delt = bmax[c] - bmin[c];
            f64 r    = p[c] - bmin[c];
            r        = fmod_wrap(r, delt);
            r += delt;
            r = fmod_wrap(r, delt);
            r += bmin[c];
            p[c] = r;
        }
        x = p[0];
        y = p[1];
        z = p[2];
    }
    lf.x[iv]  = x;
    lf.y[iv]  = y;
    lf.z[iv]  = z;
    lf.vx[iv] = vx;
    lf.vy[iv] = vy;
    lf.vz[iv] = vz;
    lf.u[i]   = u;
}

// ---------------------------------------------------------------- conservation totals
// ConservativeCheck::check_conservation (shammodels/sph/src/modules/ConservativeCheck.cpp:
// 56-180): sum v, sum a, sum (u + v.v / 2) and sum (v.a + du), each times the particle
// mass, in FP64.  Per-block partial sums in a fixed tree order, then one block adds the
// partials in block order: the totals are the same from run to run.
constexpr u32 kConsBlock = 256;

__global__ void __launch_bounds__(kConsBlock) k_cons_partial(LocalFields lf, u32 n,
                                                            f64 *__restrict__ part) {
    __shared__ f64 sm[8][kConsBlock];
    const u32 t = threadIdx.x;
    f64 v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (u32 i = blockIdx.x * kConsBlock + t; i < n; i += gridDim.x * kConsBlock) {
        const size_t iv = (size_t) i * lf.vs;
        const f64 vx = lf.vx[iv], vy = lf.vy[iv], vz = lf.vz[iv];
        const f64 ax = lf.ax[iv], ay = lf.ay[iv], az = lf.az[iv];
        v[0] += vx;
        v[1] += vy;
        v[2] += vz;
        v[3] += ax;
        v[4] += ay;
        v[5] += az;
        v[6] += lf.u[i] + 0.5 * ((vx * vx + vy * vy) + vz * vz);
        v[7] += ((vx * ax + vy * ay) + vz * az) + lf.du[i];
    }
#pragma unroll
    for (int k = 0; k < 8; k++) sm[k][t] = v[k];
    __syncthreads();
    for (u32 s = kConsBlock / 2; s > 0; s >>= 1) {
        if (t < s)
#pragma unroll
            for (int k = 0; k < 8; k++) sm[k][t] += sm[k][t + s];
        __syncthreads();
    }
    if (t < 8) part[(size_t) blockIdx.x * 8 + t] = sm[t][0];
}

__global__ void k_cons_final(const f64 *__restrict__ part, u32 nb, f64 pmass,
                             f64 *__restrict__ out) {
    const u32 k = threadIdx.x;
    if (k >= 8) return;
    f64 s = 0;
    for (u32 b = 0; b < nb; b++) s += part[(size_t) b * 8 + k];
    out[k] = pmass * s;
}

// ---------------------------------------------------------------- varying AV (CD10)
// div v and curl v (DiffOperator.cpp:95-140, 200-245) and d(div v)/dt from the linearly
// corrected gradients (DiffOperatorDtDivv.cpp:116-210) in one pass over the row; each
// sum in the reference's order, so the values equal the three separate kernels'.
__device__ __forceinline__ void inv33(const f64 m[3][3], f64 r[3][3]) {
    const f64 a00 = m[0][0], a01 = m[0][1], a02 = m[0][2];
    const f64 a10 = m[1][0], a11 = m[1][1], a12 = m[1][2];
    const f64 a20 = m[2][0], a21 = m[2][1], a22 = m[2][2];
    const f64 det = (((((-a02 * a11) * a20 + (a01 * a12) * a20) + (a02 * a10) * a21)
                      - (a00 * a12) * a21) - (a01 * a10) * a22) + (a00 * a11) * a22;
    r[0][0] = (-a12 * a21 + a11 * a22) / det;
    r[0][1] = (a02 * a21 - a01 * a22) / det;
    r[0][2] = (-a02 * a11 + a01 * a12) / det;
    r[1][0] = (a12 * a20 - a10 * a22) / det;
    r[1][1] = (-a02 * a20 + a00 * a22) / det;
    r[1][2] = (a02 * a10 - a00 * a12) / det;
    r[2][0] = (-a11 * a20 + a10 * a21) / det;
    r[2][1] = (a01 * a20 - a00 * a21) / det;
    r[2][2] = (-a01 * a10 + a00 * a11) / det;
}
__device__ __forceinline__ void mul33(const f64 a[3][3], const f64 b[3][3], f64 c[3][3]) {
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) c[i][j] = (a[i][0] * b[0][j] + a[i][1] * b[1][j]) + a[i][2] * b[2][j];
}

__global__ void __launch_bounds__(128) k_velgrad64(RowSpace rs, HydroSpace hs,
                                                   const f64 *__restrict__ axr,
                                                   const f64 *__restrict__ ayr,
                                                   const f64 *__restrict__ azr, f64 pmass,
                                                   f64 *__restrict__ divv, f64 *__restrict__ cx,
                                                   f64 *__restrict__ cy, f64 *__restrict__ cz,
                                                   u32 cvs, f64 *__restrict__ dtdivv) {
    u32 t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= rs.n) return;
    const u32 a  = rs.row_rank[t];
    const u32 k0 = rs.off[t], k1 = k0 + rs.cnt[t];
    const f64 Rker2 = kRkern * kRkern;
    const f64 h_a   = hs.h[a];
    const f64 xa[3] = {rs.x[a], rs.y[a], rs.z[a]};
    const f64 va[3] = {hs.vx[a], hs.vy[a], hs.vz[a]};
    const f64 aa[3] = {axr[a], ayr[a], azr[a]};
    const f64 rho_a = rho_h(pmass, h_a);
    const f64 inv_rho_omega_a = 1. / (hs.omega[a] * rho_a);
    f64 sdiv = 0, sc[3] = {0, 0, 0};
    f64 R[3][3] = {}, Dv[3][3] = {}, Da[3][3] = {};
    for (u32 k = k0; k < k1; k++) {
        const u32 b    = rs.ent[k];
        const f64 r[3] = {xa[0] - rs.x[b], xa[1] - rs.y[b], xa[2] - rs.z[b]};
        const f64 rab2 = (r[0] * r[0] + r[1] * r[1]) + r[2] * r[2];
        const f64 h_b  = hs.h[b];
        if (rab2 > h_a * h_a * Rker2 && rab2 > h_b * h_b * Rker2) continue;
        const f64 rab  = sqrt(rab2);
        const f64 v[3] = {va[0] - hs.vx[b], va[1] - hs.vy[b], va[2] - hs.vz[b]};
        const f64 w[3] = {aa[0] - axr[b], aa[1] - ayr[b], aa[2] - azr[b]};
        f64 e[3] = {r[0] / rab, r[1] / rab, r[2] / rab};
        if (rab < 1e-9) e[0] = e[1] = e[2] = 0;
        const f64 F    = dW_3d(rab, h_a);
        const f64 g[3] = {F * e[0], F * e[1], F * e[2]};
        sdiv  = sdiv + pmass * ((v[0] * g[0] + v[1] * g[1]) + v[2] * g[2]);
        sc[0] = sc[0] + pmass * (v[1] * g[2] - v[2] * g[1]);
        sc[1] = sc[1] + pmass * (v[2] * g[0] - v[0] * g[2]);
        sc[2] = sc[2] + pmass * (v[0] * g[1] - v[1] * g[0]);
        const f64 mg[3] = {g[0] * pmass, g[1] * pmass, g[2] * pmass};
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) {
                R[i][j]  = R[i][j] - r[i] * mg[j];
                Dv[j][i] = Dv[j][i] - v[i] * mg[j];
                Da[j][i] = Da[j][i] - w[i] * mg[j];
            }
    }
    const u32 i = rs.row_local[t];
    divv[i]     = -inv_rho_omega_a * sdiv;
    cx[(size_t) i * cvs] = -inv_rho_omega_a * sc[0];
    cy[(size_t) i * cvs] = -inv_rho_omega_a * sc[1];
    cz[(size_t) i * cvs] = -inv_rho_omega_a * sc[2];
    f64 Ri[3][3], Gv[3][3], Ga[3][3];
    inv33(R, Ri);
    mul33(Ri, Dv, Gv);
    mul33(Ri, Da, Ga);
    const f64 div_a = (Ga[0][0] + Ga[1][1]) + Ga[2][2];
    const f64 tens  = ((((((((Gv[0][0] * Gv[0][0] + Gv[1][0] * Gv[0][1]) + Gv[2][0] * Gv[0][2])
                            + Gv[0][1] * Gv[1][0]) + Gv[1][1] * Gv[1][1]) + Gv[2][1] * Gv[1][2])
                         + Gv[0][2] * Gv[2][0]) + Gv[1][2] * Gv[2][1]) + Gv[2][2] * Gv[2][2]);
    dtdivv[i] = div_a - tens;
}

// Cullen & Dehnen (2010) switch, one implicit-Euler step (UpdateViscosity.cpp:170-215);
// max / min as comparisons, as in the oracle
// T = f64: the reference's FP64 switch, bit for bit.  T = float: the same expressions in
// FP32 for the mixed path (its velocity gradients are FP32 sums already; the switch's
// divisions would otherwise make this pass FP64-pipe bound on GB300).
template<class T>
__global__ void k_cd10(u32 n, const f64 *__restrict__ divv, const f64 *__restrict__ cx,
                       const f64 *__restrict__ cy, const f64 *__restrict__ cz, u32 cvs,
                       const f64 *__restrict__ dtdivv, const f64 *__restrict__ cs,
                       const f64 *__restrict__ h, const f64 *__restrict__ alpha, f64 dt_,
                       f64 sigma_decay_, f64 alpha_min_, f64 alpha_max_, f64 *__restrict__ alpha_new) {
    u32 i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const T eps  = (T) 2.220446049250313e-16; // DBL_EPSILON
    const T dt = (T) dt_, sigma_decay = (T) sigma_decay_, alpha_min = (T) alpha_min_,
            alpha_max = (T) alpha_max_;
    const T cs_a = (T) cs[i], h_a = (T) h[i], alpha_a = (T) alpha[i];
    const T inv_tau = cs_a * sigma_decay / h_a;
    const T fact_t  = dt * inv_tau;
    const T euler   = 1 / (1 + fact_t);
    const T md = -(T) divv[i];
    T fac      = (md > 0) ? md : T(0);
    fac        = fac * fac;
    const size_t iv = (size_t) i * cvs;
    const T cxi = (T) cx[iv], cyi = (T) cy[iv], czi = (T) cz[iv];
    const T traceS  = (cxi * cxi + cyi * cyi) + czi * czi;
    const T balsara = (fac + traceS > eps) ? fac / (fac + traceS) : T(1);
    const T mdt     = -(T) dtdivv[i];
    const T A       = balsara * ((mdt > 0) ? mdt : T(0));
    const T temp    = cs_a * cs_a;
    T alpha_loc     = (cs_a > 0) ? 10 * h_a * h_a * A / temp : alpha_min;
    alpha_loc       = (alpha_loc < alpha_max) ? alpha_loc : alpha_max;
    alpha_loc       = (temp > eps) ? alpha_loc : alpha_min;
    T na = (alpha_a + alpha_loc * fact_t) * euler;
    if (alpha_loc > alpha_a) na = alpha_loc;
    alpha_new[i] = (f64) na;
}

// Morris & Monaghan (1997) switch (UpdateViscosity.cpp:53-118), comparisons as in the oracle
template<class T>
__global__ void k_mm97(u32 n, const f64 *__restrict__ divv, const f64 *__restrict__ cs,
                       const f64 *__restrict__ h, const f64 *__restrict__ alpha, f64 dt_,
                       f64 sigma_decay_, f64 alpha_min_, f64 alpha_max_, f64 *__restrict__ alpha_new) {
    u32 i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const T dt = (T) dt_, alpha_min = (T) alpha_min_, alpha_max = (T) alpha_max_;
    const T inv_tau = (T) cs[i] * (T) sigma_decay_ / (T) h[i];
    const T fact_t  = dt * inv_tau;
    const T euler   = 1 / (1 + fact_t);
    const T md      = -(T) divv[i];
    const T source  = (md > 0) ? md : T(0);
    const T na      = ((T) alpha[i] + source * dt + fact_t * alpha_min) * euler;
    alpha_new[i]    = (f64) ((na < alpha_max) ? na : alpha_max);
}

__global__ void k_gather_merged(const u32 *__restrict__ sort_index, u32 N, u32 n_local,
                                const u32 *__restrict__ ghost_src, const f64 *__restrict__ src,
                                u32 stride, f64 *__restrict__ dst) {
    u32 r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= N) return;
    u32 id  = sort_index[r];
    u32 s   = id < n_local ? id : ghost_src[id - n_local];
    dst[r]  = src[(size_t) s * stride];
}

__global__ void k_rank_to_local(u32 n, const u32 *__restrict__ row_rank,
                                const u32 *__restrict__ row_local, const f64 *__restrict__ src,
                                f64 *__restrict__ dst) {
    u32 t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    dst[row_local[t]] = src[row_rank[t]];
}

__global__ void k_scatter_rows(u32 n, const u32 *__restrict__ row_local, const f64 *__restrict__ src,
                               f64 *__restrict__ dst) {
    u32 t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    dst[row_local[t]] = src[t];
}

__global__ void k_gather_rows(u32 n, const u32 *__restrict__ row_rank, const f64 *__restrict__ src,
                              f64 *__restrict__ dst, f64 *__restrict__ dst2) {
    u32 t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    f64 v  = src[row_rank[t]];
    dst[t] = v;
    if (dst2) dst2[t] = v;
}

__global__ void k_fill(u32 n, f64 *__restrict__ dst, f64 v) {
    u32 t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) dst[t] = v;
}

} // namespace

// ---------------------------------------------------------------- host wrappers
cudaError_t h_iterate64(Ctx &c, const RowSpace &rs, const f64 *h_old, f64 *h_new, f64 *eps,
                        f64 pmass, f64 hev, f64 hevi, u32 iters, f64 eps_p) {
    ProfScope ps(c, kProfHIter, rs.n);
    { k_h_iterate<<<div_up(rs.n, 256), 256, 0, c.stream>>>(rs, h_old, h_new, eps, pmass, hev, hevi,
                                                         iters, eps_p, c.d_scalars.as<Scalars>()); GBSPH_COUNTED; }
    return cudaGetLastError();
}
cudaError_t omega64(Ctx &c, const RowSpace &rs, const f64 *h_row, f64 pmass, f64 *out,
                    const u32 *out_index) {
    ProfScope ps(c, kProfOmega, rs.n);
    { k_omega<<<div_up(rs.n, 256), 256, 0, c.stream>>>(rs, h_row, pmass, out, out_index); GBSPH_COUNTED; }
    return cudaGetLastError();
}
cudaError_t eos64(Ctx &c, u32 n, const f64 *h, const f64 *u, f64 pmass, f64 gamma, f64 *P, f64 *cs) {
    { k_eos<<<div_up(n, 256), 256, 0, c.stream>>>(n, h, u, pmass, gamma, P, cs); GBSPH_COUNTED; }
    return cudaGetLastError();
}
cudaError_t gather_eos64(Ctx &c, u32 N, u32 n_local, const LocalFields &lf, const f64 *omega_local,
                         f64 pmass, const EosParams &eos) {
    ProfScope ps(c, kProfGatherEos, N);
    { k_gather_eos<<<div_up(N, 256), 256, 0, c.stream>>>(
        c.sort_index.as<u32>(), N, n_local, c.ghost_src.as<u32>(), lf.h, lf.u, lf.vx, lf.vy, lf.vz,
        lf.vs, omega_local, pmass, eos, c.sx.as<f64>(), c.sy.as<f64>(), c.sz.as<f64>(),
        c.sh2.as<f64>(), c.su.as<f64>(), c.svx.as<f64>(), c.svy.as<f64>(), c.svz.as<f64>(),
        c.som.as<f64>(), c.sP.as<f64>(), c.scs.as<f64>(), c.srho.as<f64>(), c.sinv.as<f64>(),
        c.srom.as<f64>()); GBSPH_COUNTED; }
    return cudaGetLastError();
}
cudaError_t eos_lp07(Ctx &c, u32 n, const f64 *x, const f64 *y, const f64 *z, u32 vs, const f64 *h,
                     f64 pmass, f64 cs0, f64 r0, f64 q, f64 *P, f64 *cs) {
    { k_eos_lp07<<<div_up(n, 256), 256, 0, c.stream>>>(n, x, y, z, vs, h, pmass, cs0, r0, q, P, cs); GBSPH_COUNTED; }
    return cudaGetLastError();
}
cudaError_t derivs64(Ctx &c, const RowSpace &rs, const HydroSpace &hs, f64 pmass, f64 alpha_u,
                     f64 alpha_AV, f64 beta_AV, f64 *ax, f64 *ay, f64 *az, f64 *du, f64 *vsig) {
    DerivParams p{pmass, alpha_u, alpha_AV, beta_AV, 0, 0, 0, ExtAccel{nullptr, nullptr, nullptr}};
    { k_derivs<<<div_up(rs.n, 128), 128, 0, c.stream>>>(rs, hs, p, ax, ay, az, du, vsig); GBSPH_COUNTED; }
    return cudaGetLastError();
}
cudaError_t derivs_step64(Ctx &c, const RowSpace &rs, const HydroSpace &hs, f64 pmass, f64 alpha_u,
                          f64 alpha_AV, f64 beta_AV, f64 hdt, f64 C_cour, f64 C_force,
                          const LocalFields &lf, const ExtAccel &ext) {
    DerivParams p{pmass, alpha_u, alpha_AV, beta_AV, hdt, C_cour, C_force, ext};
    ProfScope ps(c, kProfDerivs, rs.n);
    if (hs.rho && hs.inv_sub && hs.rho_om) {
        k_derivs_step<true><<<div_up(rs.n, 128), 128, 0, c.stream>>>(rs, hs, p, lf, c.d_scalars.as<Scalars>()); GBSPH_COUNTED;
    } else {
        k_derivs_step<false><<<div_up(rs.n, 128), 128, 0, c.stream>>>(rs, hs, p, lf, c.d_scalars.as<Scalars>()); GBSPH_COUNTED;
    }
    return cudaGetLastError();
}
// leapfrog corrector (integrators.cpp:88-120): v += dt/2 (a_new - a_old), u likewise;
// max |dv|^2 and sum |v|^2 for the eps_v rerun test (Solver.cpp:2580-2616)
__global__ void k_kdk_correct(LocalFields lf, u32 n, const f64 *__restrict__ aox,
                              const f64 *__restrict__ aoy, const f64 *__restrict__ aoz, u32 avs,
                              const f64 *__restrict__ du_old, f64 hdt, Scalars *sc) {
    u32 i   = blockIdx.x * blockDim.x + threadIdx.x;
    u64 ev2 = 0;
    f64 v2  = 0;
    if (i < n) {
        size_t iv = (size_t) i * lf.vs, io = (size_t) i * avs;
        f64 ix = hdt * (lf.ax[iv] - aox[io]);
        f64 iy = hdt * (lf.ay[iv] - aoy[io]);
        f64 iz = hdt * (lf.az[iv] - aoz[io]);
        f64 vx = lf.vx[iv] + ix, vy = lf.vy[iv] + iy, vz = lf.vz[iv] + iz;
        lf.vx[iv] = vx;
        lf.vy[iv] = vy;
        lf.vz[iv] = vz;
        lf.u[i]   = lf.u[i] + hdt * (lf.du[i] - du_old[i]);
        ev2       = f64_to_ordered(__dadd_rn(__dadd_rn(ix * ix, iy * iy), iz * iz));
        v2        = __dadd_rn(__dadd_rn(vx * vx, vy * vy), vz * vz);
    }
    ev2 = block_reduce(ev2, OpMaxU64{}, 0ull);
    v2  = block_reduce(v2, OpAddF64{}, 0.0);
    if (threadIdx.x == 0) {
        atomicMax((unsigned long long *) &sc->epsv2_max, (unsigned long long) ev2);
        atomicAdd(&sc->sum_v2, v2);
    }
}

// CFL (ComputeCFLCourant.hpp:45-60, ComputeCFLForce.hpp:50-62) and its minimum
__global__ void k_cfl(u32 n, const f64 *__restrict__ h, const f64 *__restrict__ vsig,
                      const f64 *__restrict__ ax, const f64 *__restrict__ ay,
                      const f64 *__restrict__ az, u32 avs, f64 C_cour, f64 C_force,
                      f64 *__restrict__ dt_part, Scalars *sc) {
    u32 i   = blockIdx.x * blockDim.x + threadIdx.x;
    u64 dtm = ~0ull;
    if (i < n) {
        size_t io = (size_t) i * avs;
        f64 dt    = __longlong_as_double(0x7ff0000000000000ll);
        dt        = fmin(dt, C_cour * h[i] / vsig[i]);
        f64 a0 = ax[io], a1 = ay[io], a2 = az[io];
        f64 abs_a = sqrt(a0 * a0 + a1 * a1 + a2 * a2);
        dt        = fmin(dt, C_force * sqrt(h[i] / abs_a));
        if (dt_part) dt_part[i] = dt;
        dtm = f64_to_ordered(dt);
    }
    dtm = block_reduce(dtm, OpMinU64{}, ~0ull);
    if (threadIdx.x == 0) atomicMin((unsigned long long *) &sc->dt_min, (unsigned long long) dtm);
}

cudaError_t kdk_correct64(Ctx &c, const LocalFields &lf, u32 n, const f64 *aox, const f64 *aoy,
                          const f64 *aoz, u32 avs, const f64 *du_old, f64 dt) {
    { k_kdk_correct<<<div_up(n, 256), 256, 0, c.stream>>>(lf, n, aox, aoy, aoz, avs, du_old, dt / 2,
                                                         c.d_scalars.as<Scalars>()); GBSPH_COUNTED; }
    return cudaGetLastError();
}
cudaError_t cfl64(Ctx &c, u32 n, const f64 *h, const f64 *vsig, const f64 *ax, const f64 *ay,
                  const f64 *az, u32 avs, f64 C_cour, f64 C_force, f64 *dt_part) {
    { k_cfl<<<div_up(n, 256), 256, 0, c.stream>>>(n, h, vsig, ax, ay, az, avs, C_cour, C_force,
                                                 dt_part, c.d_scalars.as<Scalars>()); GBSPH_COUNTED; }
    return cudaGetLastError();
}

cudaError_t predict64(Ctx &c, const LocalFields &lf, u32 n, f64 dt, int periodic, const f64 *bmin,
                      const f64 *bmax, f64 mGM, f64 *ext_x, f64 *ext_y, f64 *ext_z) {
    ProfScope ps(c, kProfPredict, n);
    { k_predict<<<div_up(n, 256), 256, 0, c.stream>>>(lf, n, dt, periodic, bmin[0], bmin[1], bmin[2],
                                                   bmax[0], bmax[1], bmax[2], mGM, ext_x, ext_y,
                                                   ext_z); GBSPH_COUNTED; }
    return cudaGetLastError();
}
cudaError_t velgrad64(Ctx &c, const RowSpace &rs, const HydroSpace &hs, const f64 *ax,
                      const f64 *ay, const f64 *az, f64 pmass, f64 *divv, f64 *cx, f64 *cy,
                      f64 *cz, u32 cvs, f64 *dtdivv) {
    ProfScope ps(c, kProfVelGrad, rs.n);
    { k_velgrad64<<<div_up(rs.n, 128), 128, 0, c.stream>>>(rs, hs, ax, ay, az, pmass, divv, cx, cy,
                                                         cz, cvs, dtdivv); GBSPH_COUNTED; }
    return cudaGetLastError();
}
cudaError_t cd10_update(Ctx &c, u32 n, const f64 *divv, const f64 *cx, const f64 *cy,
                        const f64 *cz, u32 cvs, const f64 *dtdivv, const f64 *cs, const f64 *h,
                        const f64 *alpha, f64 dt, f64 sigma_decay, f64 alpha_min, f64 alpha_max,
                        f64 *alpha_new, bool fp32) {
    if (fp32) {
        k_cd10<float><<<div_up(n, 256), 256, 0, c.stream>>>(n, divv, cx, cy, cz, cvs, dtdivv, cs, h,
                                                           alpha, dt, sigma_decay, alpha_min,
                                                           alpha_max, alpha_new); GBSPH_COUNTED;
    } else {
        k_cd10<f64><<<div_up(n, 256), 256, 0, c.stream>>>(n, divv, cx, cy, cz, cvs, dtdivv, cs, h,
                                                         alpha, dt, sigma_decay, alpha_min,
                                                         alpha_max, alpha_new); GBSPH_COUNTED;
    }
    return cudaGetLastError();
}
cudaError_t mm97_update(Ctx &c, u32 n, const f64 *divv, const f64 *cs, const f64 *h,
                        const f64 *alpha, f64 dt, f64 sigma_decay, f64 alpha_min, f64 alpha_max,
                        f64 *alpha_new, bool fp32) {
    if (fp32) {
        k_mm97<float><<<div_up(n, 256), 256, 0, c.stream>>>(n, divv, cs, h, alpha, dt, sigma_decay,
                                                           alpha_min, alpha_max, alpha_new); GBSPH_COUNTED;
    } else {
        k_mm97<f64><<<div_up(n, 256), 256, 0, c.stream>>>(n, divv, cs, h, alpha, dt, sigma_decay,
                                                         alpha_min, alpha_max, alpha_new); GBSPH_COUNTED;
    }
    return cudaGetLastError();
}
cudaError_t conservation64(Ctx &c, const LocalFields &lf, u32 n, f64 pmass, f64 *out_dev,
                           f64 *scratch) {
    const u32 nb = 1024;
    { k_cons_partial<<<nb, kConsBlock, 0, c.stream>>>(lf, n, scratch); GBSPH_COUNTED; }
    { k_cons_final<<<1, 32, 0, c.stream>>>(scratch, nb, pmass, out_dev); GBSPH_COUNTED; }
    return cudaGetLastError();
}
cudaError_t gather_merged64(Ctx &c, u32 N, u32 n_local, const f64 *src, u32 stride, f64 *dst) {
    { k_gather_merged<<<div_up(N, 256), 256, 0, c.stream>>>(c.sort_index.as<u32>(), N, n_local,
                                                           c.ghost_src.as<u32>(), src, stride,
                                                           dst); GBSPH_COUNTED; }
    return cudaGetLastError();
}
cudaError_t rank_to_local64(Ctx &c, u32 n, const f64 *src_rank, f64 *dst) {
    { k_rank_to_local<<<div_up(n, 256), 256, 0, c.stream>>>(n, c.row_rank.as<u32>(),
                                                           c.row_local.as<u32>(), src_rank,
                                                           dst); GBSPH_COUNTED; }
    return cudaGetLastError();
}
cudaError_t scatter_rows(Ctx &c, u32 n, const f64 *src, f64 *dst) {
    { k_scatter_rows<<<div_up(n, 256), 256, 0, c.stream>>>(n, c.row_local.as<u32>(), src, dst); GBSPH_COUNTED; }
    return cudaGetLastError();
}
cudaError_t gather_rows(Ctx &c, u32 n, const f64 *src_rank, f64 *dst, f64 *dst2) {
    { k_gather_rows<<<div_up(n, 256), 256, 0, c.stream>>>(n, c.row_rank.as<u32>(), src_rank, dst, dst2); GBSPH_COUNTED; }
    return cudaGetLastError();
}
cudaError_t fill64(Ctx &c, u32 n, f64 *dst, f64 v) {
    { k_fill<<<div_up(n, 256), 256, 0, c.stream>>>(n, dst, v); GBSPH_COUNTED; }
    return cudaGetLastError();
}

} // namespace gbsph
