// Adjoint (reverse mode) of one SPH step with the neighbour cache, dt and the number of
// corrector evaluations frozen from the forward pass.
//
// Forward map of one step (the leapfrog of integrators.cpp:27-120, Solver.cpp:390-524,
// 2506-2616), with A_0 = a, D_0 = du:
//   v_2 = v + dt a,  u_2 = u + dt du,  x' = x + dt v + dt^2/2 a           (predictor)
//   h'  solves  sum_b m W(r_ab, h_a) = rho(h_a) = m (hfact / h_a)^3         (density)
//   Omega_a = 1 + h_a / (3 rho_a) sum_b m dW/dh(r_ab, h_a)
//   for k = 1..K:  (A_k, D_k) = derivs(x', v_{k+1}, u_{k+1}, h', Omega)
//                  v_{k+2} = v_{k+1} + dt/2 (A_k - A_{k-1}),  u likewise
//   state after the step: x', v_{K+2}, u_{K+2}, a' = A_K, du' = D_K.
// h' is differentiated as the exact root of the density constraint (implicit function:
// dC_a/dh_a = 3 rho_a Omega_a / h_a), so the gradient is that of the converged solve.
//
// Pair sums are reversed without atomics.  The neighbour relation is symmetric (the
// cache test max(r_a, r_b) is, and a ghost pair (a, b + L) mirrors (b, a - L)), so the
// contribution of the pair {c, b} to particle c's cotangents is the derivative, with
// respect to c's inputs, of the two-row pair term
//   L_cb = (lambda_c - lambda_b) . f_cb + mu_c g_cb + mu_b g_bc,
// which row c evaluates with its neighbour's cotangents gathered by rank.
// FP64 throughout (the reference gradient).

#include "adjoint.cuh"

namespace gbsph {

namespace {

constexpr f64 kSig = kNorm3d;

// M4 shape f(q) and its first two derivatives (sphkernels.hpp:29-72)
__device__ __forceinline__ f64 m4_f(f64 q) {
    f64 t1 = 2 - q, t2 = 1 - q;
    t1 = 0.25 * t1 * t1 * t1;
    if (q < 1) return t1 - t2 * t2 * t2;
    return q < 2 ? t1 : 0.0;
}
__device__ __forceinline__ f64 m4_d1(f64 q) {
    if (q < 1) return -3 * q + 2.25 * q * q;
    return q < 2 ? -3 + 3 * q - 0.75 * q * q : 0.0;
}
__device__ __forceinline__ f64 m4_d2(f64 q) {
    if (q < 1) return -3 + 4.5 * q;
    return q < 2 ? 3 - 1.5 * q : 0.0;
}
__device__ __forceinline__ f64 rho_of_h(f64 m, f64 h) {
    return m * (kHfact / h) * (kHfact / h) * (kHfact / h);
}

// -------------------------------------------------------------- gathers into rank order
// Per rank (ghosts read their source particle): velocity and energy of the corrector
// evaluation being reversed, h, Omega and the cotangents (lambda, mu) of its outputs.
__global__ void k_adj_gather(u32 N, u32 n, const u32 *__restrict__ sort_index,
                             const u32 *__restrict__ ghost_src, const f64 *__restrict__ vx,
                             const f64 *__restrict__ vy, const f64 *__restrict__ vz,
                             const f64 *__restrict__ u, const f64 *__restrict__ h,
                             const f64 *__restrict__ om, const f64 *__restrict__ lx,
                             const f64 *__restrict__ ly, const f64 *__restrict__ lz,
                             const f64 *__restrict__ mu, f64 *__restrict__ R) {
    u32 r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= N) return;
    u32 id  = sort_index[r];
    u32 src = id < n ? id : ghost_src[id - n];
    size_t N_ = N;
    R[0 * N_ + r] = vx[src];
    R[1 * N_ + r] = vy[src];
    R[2 * N_ + r] = vz[src];
    R[3 * N_ + r] = u[src];
    R[4 * N_ + r] = h[src];
    R[5 * N_ + r] = om[src];
    R[6 * N_ + r] = lx[src];
    R[7 * N_ + r] = ly[src];
    R[8 * N_ + r] = lz[src];
    R[9 * N_ + r] = mu[src];
}
__global__ void k_adj_gather2(u32 N, u32 n, const u32 *__restrict__ sort_index,
                              const u32 *__restrict__ ghost_src, const f64 *__restrict__ a,
                              const f64 *__restrict__ b, f64 *__restrict__ ra,
                              f64 *__restrict__ rb) {
    u32 r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= N) return;
    u32 id  = sort_index[r];
    u32 src = id < n ? id : ghost_src[id - n];
    ra[r]   = a[src];
    rb[r]   = b[src];
}

struct RankFields {
    const f64 *vx, *vy, *vz, *u, *h, *om, *lx, *ly, *lz, *mu;
};
RankFields rank_fields(const f64 *R, u32 N) {
    size_t N_ = N;
    return RankFields{R, R + N_, R + 2 * N_, R + 3 * N_, R + 4 * N_,
                      R + 5 * N_, R + 6 * N_, R + 7 * N_, R + 8 * N_, R + 9 * N_};
}

// Local accumulators of the reverse pass (SoA, n each).
struct AdjLocal {
    f64 *lam[3], *mu;       // cotangent of A_k, D_k (corrector evaluation being reversed)
    f64 *lamp[3], *mup;     // share of A_{k-1}, D_{k-1}
    f64 *lv[3], *lu;        // cotangent of v_{k+1}, u_{k+1}
    f64 *gx[3];             // cotangent of x'
    f64 *gh, *gom;          // cotangent of h', Omega
    f64 *nu, *lom;          // density-constraint multiplier, Omega cotangent x h/(3 rho)
};

// -------------------------------------------------------------- reverse of derivs
__global__ void __launch_bounds__(128) k_adj_derivs(RowSpace rs, RankFields f, AdjParams p,
                                                    AdjLocal L, f64 *g_alpha) {
    u32 t      = blockIdx.x * blockDim.x + threadIdx.x;
    f64 galpha = 0;
    if (t < rs.n) {
        const f64 m = p.pmass, gm1 = p.gamma - 1, Rk2 = kRkern * kRkern;
        const u32 c = rs.row_rank[t], i = rs.row_local[t];
        const f64 xc = rs.x[c], yc = rs.y[c], zc = rs.z[c];
        const f64 vxc = f.vx[c], vyc = f.vy[c], vzc = f.vz[c];
        const f64 uc = f.u[c], hc = f.h[c], omc = f.om[c];
        const f64 lxc = f.lx[c], lyc = f.ly[c], lzc = f.lz[c], muc = f.mu[c];
        const f64 rhoc = rho_of_h(m, hc), Pc = gm1 * rhoc * uc, csc = sqrt(p.gamma * gm1 * uc);
        const f64 subc = rhoc * rhoc * omc;
        const f64 kc = (subc != 0 && subc == subc) ? 1 / subc : 0, jc = 1 / (rhoc * omc);
        f64 gxr = 0, gyr = 0, gzr = 0, gvx = 0, gvy = 0, gvz = 0;
        f64 sP = 0, scs = 0, srho = 0, sk = 0, sj = 0, su = 0, shF = 0;
        const u32 k0 = rs.off[t], k1 = k0 + rs.cnt[t];
        for (u32 k = k0; k < k1; k++) {
            const u32 b = rs.ent[k];
            const f64 dx = xc - rs.x[b], dy = yc - rs.y[b], dz = zc - rs.z[b];
            const f64 r2 = dx * dx + dy * dy + dz * dz;
            const f64 hb = f.h[b];
            if (r2 > hc * hc * Rk2 && r2 > hb * hb * Rk2) continue;
            if (r2 == 0) continue; // self pair: no contribution and no dependence
            const f64 r = sqrt(r2), ir = 1 / r;
            const f64 ex = dx * ir, ey = dy * ir, ez = dz * ir;
            const f64 ub = f.u[b], omb = f.om[b];
            const f64 rhob = rho_of_h(m, hb), Pb = gm1 * rhob * ub, csb = sqrt(p.gamma * gm1 * ub);
            const f64 subb = rhob * rhob * omb;
            const f64 kb = (subb != 0 && subb == subb) ? 1 / subb : 0, jb = 1 / (rhob * omb);
            const f64 ihc = 1 / hc, ihb = 1 / hb;
            const f64 qc = r * ihc, qb = r * ihb;
            const f64 ihc4 = ihc * ihc * ihc * ihc, ihb4 = ihb * ihb * ihb * ihb;
            const f64 d1c = m4_d1(qc), d1b = m4_d1(qb), d2c = m4_d2(qc), d2b = m4_d2(qb);
            const f64 Fc = kSig * d1c * ihc4, Fb = kSig * d1b * ihb4;        // dW/dr
            const f64 Frc = kSig * d2c * ihc4 * ihc, Frb = kSig * d2b * ihb4 * ihb; // d2W/dr2
            const f64 Fhc = -kSig * (qc * d2c + 4 * d1c) * ihc4 * ihc;       // d(dW/dr)/dh_c
            const f64 vabx = vxc - f.vx[b], vaby = vyc - f.vy[b], vabz = vzc - f.vz[b];
            const f64 w = vabx * ex + vaby * ey + vabz * ez, aw = fabs(w);
            const f64 vsc = p.alpha_AV * csc + p.beta_AV * aw, vsb = p.alpha_AV * csb + p.beta_AV * aw;
            const f64 tc = -0.5 * rhoc * vsc * w, tb = -0.5 * rhob * vsb * w;
            const bool actc = tc > 0, actb = tb > 0;
            const f64 Ac = Pc + (actc ? tc : 0), Ab = Pb + (actb ? tb : 0);
            const f64 dP = Pc - Pb, rbar = 0.5 * (rhoc + rhob);
            const f64 vsu = sqrt(fabs(dP) / rbar);
            const f64 J = Fc * jc + Fb * jb;
            const f64 S = Ac * kc * Fc + Ab * kb * Fb;
            const f64 Lx = lxc - f.lx[b], Ly = lyc - f.ly[b], Lz = lzc - f.lz[b];
            const f64 Le = Lx * ex + Ly * ey + Lz * ez;
            const f64 mub = f.mu[b];
            const f64 du_ = uc - ub, dmu = muc - mub;
            const f64 cond = 0.5 * m * p.alpha_u * dmu * vsu * du_; // multiplies J
            // d q / d w where the viscous pressure is active
            const f64 dqcw = actc ? -0.5 * rhoc * (vsc + p.beta_AV * aw) : 0;
            const f64 dqbw = actb ? -0.5 * rhob * (vsb + p.beta_AV * aw) : 0;
            const f64 dSw  = kc * Fc * dqcw + kb * Fb * dqbw;
            const f64 E    = muc * Ac * kc * Fc + mub * Ab * kb * Fb;
            const f64 dLw  = -m * Le * dSw + m * E + m * w * (muc * kc * Fc * dqcw + mub * kb * Fb * dqbw);
            const f64 dLr  = -m * Le * (Ac * kc * Frc + Ab * kb * Frb)
                            + m * w * (muc * Ac * kc * Frc + mub * Ab * kb * Frb)
                            + cond * (Frc * jc + Frb * jb);
            // dL/de (e free), then the projection of r_vec -> (r, e)
            const f64 dex = -m * S * Lx + dLw * vabx, dey = -m * S * Ly + dLw * vaby,
                      dez = -m * S * Lz + dLw * vabz;
            const f64 ede = dex * ex + dey * ey + dez * ez;
            gxr += dLr * ex + (dex - ede * ex) * ir;
            gyr += dLr * ey + (dey - ede * ey) * ir;
            gzr += dLr * ez + (dez - ede * ez) * ir;
            gvx += dLw * ex;
            gvy += dLw * ey;
            gvz += dLw * ez;
            // particle-c scalars
            const f64 dLAc  = -m * Le * kc * Fc + m * w * muc * kc * Fc;
            const f64 dLvsu = 0.5 * m * p.alpha_u * dmu * du_ * J;
            const f64 dvsuP = vsu > 0 ? (dP > 0 ? 1.0 : -1.0) / (2 * rbar * vsu) : 0;
            const f64 dvsur = vsu > 0 ? -vsu / (4 * rbar) : 0;
            sP += dLAc + dLvsu * dvsuP;
            if (actc) scs += dLAc * (-0.5 * rhoc * p.alpha_AV * w);
            srho += (actc ? dLAc * (tc / rhoc) : 0) + dLvsu * dvsur;
            sk += -m * Le * Ac * Fc + m * w * muc * Ac * Fc;
            sj += cond * Fc;
            su += 0.5 * m * p.alpha_u * dmu * vsu * J;
            shF += (-m * Le * Ac * kc + m * w * muc * Ac * kc + cond * jc) * Fhc;
            // alpha_AV: this row's own pair term only (lambda_c . f_cb + mu_c g_cb)
            const f64 dqca = actc ? -0.5 * rhoc * csc * w : 0;
            const f64 dqba = actb ? -0.5 * rhob * csb * w : 0;
            const f64 lce  = lxc * ex + lyc * ey + lzc * ez;
            galpha += -m * lce * (kc * Fc * dqca + kb * Fb * dqba) + muc * m * w * kc * Fc * dqca;
        }
        const f64 gu   = sP * gm1 * rhoc + (csc > 0 ? scs * p.gamma * gm1 / (2 * csc) : 0) + su;
        const f64 grho = sP * gm1 * uc + srho + sk * (-2 * kc / rhoc) + sj * (-jc / rhoc);
        const f64 gh   = grho * (-3 * rhoc / hc) + shF;
        const f64 gom  = sk * (-kc / omc) + sj * (-jc / omc);
        L.lv[0][i] += gvx;
        L.lv[1][i] += gvy;
        L.lv[2][i] += gvz;
        L.lu[i] += gu;
        L.gx[0][i] += gxr;
        L.gx[1][i] += gyr;
        L.gx[2][i] += gzr;
        L.gh[i] += gh;
        L.gom[i] += gom;
    }
    galpha = block_reduce(galpha, OpAddF64{}, 0.0);
    if (threadIdx.x == 0) atomicAdd(g_alpha, galpha);
}

// -------------------------------------------------------------- reverse of Omega and h'
// nu_c = -(gh_c + gom_c dOmega_c/dh_c) h_c / (3 rho_c Omega_c), and lom_c = gom_c h_c/(3 rho_c).
__global__ void __launch_bounds__(256) k_adj_omega_a(RowSpace rs, const f64 *__restrict__ rh,
                                                     const f64 *__restrict__ rom, f64 pmass,
                                                     AdjLocal L) {
    u32 t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= rs.n) return;
    const u32 c = rs.row_rank[t], i = rs.row_local[t];
    const f64 hc = rh[c], ihc = 1 / hc, omc = rom[c];
    const f64 xc = rs.x[c], yc = rs.y[c], zc = rs.z[c];
    const f64 rhoc = rho_of_h(pmass, hc);
    f64 S = 0, Sh = 0; // sum m dW/dh, sum m d2W/dh2 (self pair included)
    const u32 k0 = rs.off[t], k1 = k0 + rs.cnt[t];
    for (u32 k = k0; k < k1; k++) {
        const u32 b = rs.ent[k];
        const f64 dx = xc - rs.x[b], dy = yc - rs.y[b], dz = zc - rs.z[b];
        const f64 r  = sqrt(dx * dx + dy * dy + dz * dz);
        const f64 q  = r * ihc;
        if (q >= 2) continue;
        const f64 f0 = m4_f(q), f1 = m4_d1(q), f2 = m4_d2(q);
        const f64 ih4 = ihc * ihc * ihc * ihc;
        S += -kSig * (3 * f0 + q * f1) * ih4;
        Sh += kSig * (12 * f0 + 8 * q * f1 + q * q * f2) * ih4 * ihc;
    }
    S *= pmass;
    Sh *= pmass;
    const f64 coef  = hc / (3 * rhoc); // Omega = 1 + coef S, coef = h^4 / (3 m hfact^3)
    const f64 dOmdh = 4 * coef * ihc * S + coef * Sh;
    const f64 gom   = L.gom[i];
    const f64 ghtot = L.gh[i] + gom * dOmdh;
    L.nu[i]  = -ghtot * hc / (3 * rhoc * omc);
    L.lom[i] = gom * coef;
}

// gx_c += sum_b e_cb m [lom_c dG/dr(h_c) + lom_b dG/dr(h_b) + nu_c dW/dr(h_c) + nu_b dW/dr(h_b)]
__global__ void __launch_bounds__(256) k_adj_omega_b(RowSpace rs, const f64 *__restrict__ rh,
                                                     const f64 *__restrict__ rnu,
                                                     const f64 *__restrict__ rlom, f64 pmass,
                                                     AdjLocal L) {
    u32 t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= rs.n) return;
    const u32 c = rs.row_rank[t], i = rs.row_local[t];
    const f64 hc = rh[c], ihc = 1 / hc, nuc = rnu[c], lomc = rlom[c];
    const f64 xc = rs.x[c], yc = rs.y[c], zc = rs.z[c];
    f64 gx = 0, gy = 0, gz = 0;
    const u32 k0 = rs.off[t], k1 = k0 + rs.cnt[t];
    for (u32 k = k0; k < k1; k++) {
        const u32 b = rs.ent[k];
        const f64 dx = xc - rs.x[b], dy = yc - rs.y[b], dz = zc - rs.z[b];
        const f64 r2 = dx * dx + dy * dy + dz * dz;
        if (r2 == 0) continue;
        const f64 r = sqrt(r2), ir = 1 / r;
        const f64 hb = rh[b], ihb = 1 / hb;
        const f64 qc = r * ihc, qb = r * ihb;
        if (qc >= 2 && qb >= 2) continue;
        const f64 d1c = m4_d1(qc), d2c = m4_d2(qc), d1b = m4_d1(qb), d2b = m4_d2(qb);
        const f64 ihc5 = ihc * ihc * ihc * ihc * ihc, ihb5 = ihb * ihb * ihb * ihb * ihb;
        const f64 Grc = -kSig * (4 * d1c + qc * d2c) * ihc5, Grb = -kSig * (4 * d1b + qb * d2b) * ihb5;
        const f64 Fc = kSig * d1c * ihc5 * hc, Fb = kSig * d1b * ihb5 * hb;
        const f64 s = pmass * (lomc * Grc + rlom[b] * Grb + nuc * Fc + rnu[b] * Fb) * ir;
        gx += s * dx;
        gy += s * dy;
        gz += s * dz;
    }
    L.gx[0][i] += gx;
    L.gx[1][i] += gy;
    L.gx[2][i] += gz;
}

// -------------------------------------------------------------- linear steps
// mode 0 (before reversing evaluation k): lam += hdt lv, mu += hdt lu, lamp = -hdt lv,
//        mup = -hdt lu
// mode 1 (after it): lam = lamp, mu = mup
__global__ void k_adj_lin(u32 n, int mode, f64 hdt, AdjLocal L) {
    u32 i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (mode == 0) {
#pragma unroll
        for (int d = 0; d < 3; d++) {
            L.lam[d][i] += hdt * L.lv[d][i];
            L.lamp[d][i] = -hdt * L.lv[d][i];
        }
        L.mu[i] += hdt * L.lu[i];
        L.mup[i] = -hdt * L.lu[i];
    } else {
#pragma unroll
        for (int d = 0; d < 3; d++) L.lam[d][i] = L.lamp[d][i];
        L.mu[i] = L.mup[i];
    }
}

// user cotangents (strided vectors) <-> accumulators
__global__ void k_adj_load(u32 n, CotState cs, u32 vs, AdjLocal L) {
    u32 i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    size_t iv = (size_t) i * vs;
#pragma unroll
    for (int d = 0; d < 3; d++) {
        L.lam[d][i] = cs.a[d][iv];
        L.lv[d][i]  = cs.v[d][iv];
        L.gx[d][i]  = cs.x[d][iv];
    }
    L.mu[i]  = cs.du[i];
    L.lu[i]  = cs.u[i];
    L.gh[i]  = 0;
    L.gom[i] = 0;
}
// predictor reverse: x' = x + dt v + dt^2/2 a, v_2 = v + dt a, u_2 = u + dt du
__global__ void k_adj_store(u32 n, f64 dt, AdjLocal L, CotState cs, u32 vs) {
    u32 i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    size_t iv = (size_t) i * vs;
#pragma unroll
    for (int d = 0; d < 3; d++) {
        f64 gx = L.gx[d][i], lv = L.lv[d][i];
        cs.x[d][iv] = gx;
        cs.v[d][iv] = lv + dt * gx;
        cs.a[d][iv] = L.lam[d][i] + dt * lv + 0.5 * dt * dt * gx;
    }
    cs.u[i]  = L.lu[i];
    cs.du[i] = L.mu[i] + dt * L.lu[i];
}

} // namespace

cudaError_t adjoint_backward(Ctx &c, const RowSpace &rs, u32 n, const f64 *h_local,
                             const f64 *omega_local, const StepTape &tape, const AdjParams &p,
                             const CotState &cot, f64 *g_alpha) {
    cudaStream_t s = c.stream;
    cudaError_t e;
    const u32 N   = n + c.n_ghost;
    const u32 K   = tape.iters;
    const f64 hdt = p.dt / 2;
    if ((e = c.adj_loc.ensure(sizeof(f64) * 21 * (size_t) n, s)) != cudaSuccess) return e;
    if ((e = c.adj_rank.ensure(sizeof(f64) * 12 * (size_t) N, s)) != cudaSuccess) return e;
    f64 *B = c.adj_loc.as<f64>();
    size_t n_ = n;
    AdjLocal L;
    for (int d = 0; d < 3; d++) {
        L.lam[d]  = B + (0 + d) * n_;
        L.lamp[d] = B + (3 + d) * n_;
        L.lv[d]   = B + (6 + d) * n_;
        L.gx[d]   = B + (9 + d) * n_;
    }
    L.mu  = B + 12 * n_;
    L.mup = B + 13 * n_;
    L.lu  = B + 14 * n_;
    L.gh  = B + 15 * n_;
    L.gom = B + 16 * n_;
    L.nu  = B + 17 * n_;
    L.lom = B + 18 * n_;
    f64 *R   = c.adj_rank.as<f64>();
    f64 *rnu = R + 10 * (size_t) N, *rlom = R + 11 * (size_t) N;
    const u32 vs = cot.vs;
    const u32 gb = div_up(n, 256), gN = div_up(N, 256);
    { k_adj_load<<<gb, 256, 0, s>>>(n, cot, vs, L); GBSPH_COUNTED; }
    const f64 *snap = tape.snap->as<f64>();
    for (u32 k = K; k >= 1; k--) {
        { k_adj_lin<<<gb, 256, 0, s>>>(n, 0, hdt, L); GBSPH_COUNTED; }
        const f64 *sv = snap + (size_t) (k - 1) * 4 * n_;
        { k_adj_gather<<<gN, 256, 0, s>>>(N, n, c.sort_index.as<u32>(), c.ghost_src.as<u32>(), sv,
                                        sv + n_, sv + 2 * n_, sv + 3 * n_, h_local, omega_local,
                                        L.lam[0], L.lam[1], L.lam[2], L.mu, R); GBSPH_COUNTED; }
        { k_adj_derivs<<<div_up(n, 128), 128, 0, s>>>(rs, rank_fields(R, N), p, L, g_alpha); GBSPH_COUNTED; }
        { k_adj_lin<<<gb, 256, 0, s>>>(n, 1, hdt, L); GBSPH_COUNTED; }
    }
    // Omega and the density constraint
    { k_adj_gather2<<<gN, 256, 0, s>>>(N, n, c.sort_index.as<u32>(), c.ghost_src.as<u32>(), h_local,
                                     omega_local, R + 4 * (size_t) N, R + 5 * (size_t) N); GBSPH_COUNTED; }
    { k_adj_omega_a<<<gb, 256, 0, s>>>(rs, R + 4 * (size_t) N, R + 5 * (size_t) N, p.pmass, L); GBSPH_COUNTED; }
    { k_adj_gather2<<<gN, 256, 0, s>>>(N, n, c.sort_index.as<u32>(), c.ghost_src.as<u32>(), L.nu,
                                     L.lom, rnu, rlom); GBSPH_COUNTED; }
    { k_adj_omega_b<<<gb, 256, 0, s>>>(rs, R + 4 * (size_t) N, rnu, rlom, p.pmass, L); GBSPH_COUNTED; }
    { k_adj_store<<<gb, 256, 0, s>>>(n, p.dt, L, cot, vs); GBSPH_COUNTED; }
    return cudaGetLastError();
}

} // namespace gbsph
