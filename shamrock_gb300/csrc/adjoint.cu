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
// Two precisions: FP64 arrays (the reference gradient) and FP32 pair arithmetic on
// hi/lo-split position and velocity records (the mixed-precision path), with the
// per-particle chain rule and all accumulators in FP64.

#include "adjoint.cuh"

#include <type_traits>

namespace gbsph {

namespace {

// M4 shape f(q) and its first two derivatives (sphkernels.hpp:29-72)
template<class T>
__device__ __forceinline__ T m4_f(T q) {
    T t1 = T(2) - q, t2 = T(1) - q;
    t1 = T(0.25) * t1 * t1 * t1;
    if (q < T(1)) return t1 - t2 * t2 * t2;
    return q < T(2) ? t1 : T(0);
}
template<class T>
__device__ __forceinline__ T m4_d1(T q) {
    if (q < T(1)) return T(-3) * q + T(2.25) * q * q;
    return q < T(2) ? T(-3) + T(3) * q - T(0.75) * q * q : T(0);
}
template<class T>
__device__ __forceinline__ T m4_d2(T q) {
    if (q < T(1)) return T(-3) + T(4.5) * q;
    return q < T(2) ? T(3) - T(1.5) * q : T(0);
}
// Division and square root of the pair loops: exact in FP64 (the reference gradient),
// the hardware approximations in FP32 (about 2 ulp: the FP32 reverse pass is checked
// against central differences at the 1e-6 level, and the correctly rounded forms cost
// many more instructions per pair)
template<class T>
__device__ __forceinline__ T pdiv(T a, T b) { return a / b; }
template<>
__device__ __forceinline__ float pdiv<float>(float a, float b) { return __fdividef(a, b); }
template<class T>
__device__ __forceinline__ T psqrt(T x) { return sqrt(x); }
template<>
__device__ __forceinline__ float psqrt<float>(float x) { return x > 0.f ? x * rsqrtf(x) : 0.f; }

template<class T>
__device__ __forceinline__ T rho_of_h(T m, T h) {
    const T r = T(kHfact) / h;
    return m * r * r * r;
}

// Local accumulators of the reverse pass (SoA, n each, FP64).
struct AdjLocal {
    f64 *lam[3], *mu;       // cotangent of A_k, D_k (corrector evaluation being reversed)
    f64 *lamp[3], *mup;     // share of A_{k-1}, D_{k-1}
    f64 *lv[3], *lu;        // cotangent of v_{k+1}, u_{k+1}
    f64 *gx[3];             // cotangent of x'
    f64 *gh, *gom;          // cotangent of h', Omega
    f64 *nu, *lom;          // density-constraint multiplier, Omega cotangent x h/(3 rho)
    // varying viscosity: cotangent of the switched alpha of the evaluation being reversed,
    // of the step's input alpha_AV and stored sound speed
    f64 *gal, *gain, *gcsin;
};

// -------------------------------------------------------------- particle sources
// A source gives, per rank, what the reverse pair loops read: the row's own values and,
// for a neighbour, its differences to the row (positions, velocities, cotangents) and
// its scalars.  Ghost ranks carry their source particle's values (positions shifted).

// FP64 rank-ordered arrays: the reference gradient.
struct Src64 {
    using T = f64;
    const f64 *x, *y, *z;                           // rank positions
    const f64 *vx, *vy, *vz, *u, *h, *om, *lx, *ly, *lz, *mu;
    const f64 *nu, *lom;                            // density / Omega multipliers
    const f64 *al;                                  // per-rank alpha (varying viscosity)
    struct Row {
        f64 x, y, z, vx, vy, vz, u, h, om, lx, ly, lz, mu;
    };
    struct Nb {
        f64 dx, dy, dz, dvx, dvy, dvz, u, h, om, lx, ly, lz, mu, rsq, al;
    };
    __device__ Row row(u32 c) const {
        return Row{x[c], y[c], z[c], vx[c], vy[c], vz[c], u[c], h[c], om[c], lx[c], ly[c], lz[c], mu[c]};
    }
    __device__ Nb nb(u32 b, const Row &r) const {
        const f64 xb = x[b], yb = y[b], zb = z[b];
        return Nb{r.x - xb, r.y - yb, r.z - zb, r.vx - vx[b], r.vy - vy[b], r.vz - vz[b],
                  u[b],     h[b],     om[b],    lx[b],        ly[b],        lz[b],
                  mu[b],    xb * xb + yb * yb + zb * zb, al ? al[b] : 0.0};
    }
    __device__ void apos(const Row &r, f64 &ax, f64 &ay, f64 &az) const {
        ax = r.x;
        ay = r.y;
        az = r.z;
    }
    __device__ void pos(u32 c, f64 &px, f64 &py, f64 &pz, f64 &ph) const {
        px = x[c];
        py = y[c];
        pz = z[c];
        ph = h[c];
    }
    __device__ void dpos(u32 b, f64 px, f64 py, f64 pz, f64 &dx, f64 &dy, f64 &dz, f64 &hb) const {
        dx = px - x[b];
        dy = py - y[b];
        dz = pz - z[b];
        hb = h[b];
    }
    __device__ void mult(u32 b, f64 &nub, f64 &lomb) const {
        nub  = nu[b];
        lomb = lom[b];
    }
};

// FP32 records (rank order), differences taken on hi/lo pairs:
//   P[2r..2r+1] = {x_hi, y_hi, z_hi, h | x_lo, y_lo, z_lo, Omega}
//   V[2r..2r+1] = {v_hi, u | v_lo, mu},   Lr[r] = {lambda, alpha},   M[r] = {nu, lom}
// (alpha: the per-particle viscosity of the varying forms, 0 for the constant one)
struct Src32 {
    using T = float;
    const float4 *P, *V, *Lr;
    const float2 *M;
    struct Row {
        F8 p, v;
        float4 l;
    };
    struct Nb {
        float dx, dy, dz, dvx, dvy, dvz, u, h, om, lx, ly, lz, mu, rsq, al;
    };
    __device__ Row row(u32 c) const {
        return Row{ldg256(&P[2 * (size_t) c]), ldg256(&V[2 * (size_t) c]), __ldg(&Lr[c])};
    }
    __device__ Nb nb(u32 b, const Row &r) const {
        const F8 p = ldg256(&P[2 * (size_t) b]), v = ldg256(&V[2 * (size_t) b]);
        const float4 l = __ldg(&Lr[b]);
        const float xb = p.a.x + p.b.x, yb = p.a.y + p.b.y, zb = p.a.z + p.b.z;
        return Nb{(r.p.a.x - p.a.x) + (r.p.b.x - p.b.x), (r.p.a.y - p.a.y) + (r.p.b.y - p.b.y),
                  (r.p.a.z - p.a.z) + (r.p.b.z - p.b.z), (r.v.a.x - v.a.x) + (r.v.b.x - v.b.x),
                  (r.v.a.y - v.a.y) + (r.v.b.y - v.b.y), (r.v.a.z - v.a.z) + (r.v.b.z - v.b.z),
                  v.a.w, p.a.w, p.b.w, l.x, l.y, l.z, v.b.w, xb * xb + yb * yb + zb * zb, l.w};
    }
    __device__ void apos(const Row &r, float &ax, float &ay, float &az) const {
        ax = r.p.a.x + r.p.b.x;
        ay = r.p.a.y + r.p.b.y;
        az = r.p.a.z + r.p.b.z;
    }
    __device__ void pos(u32 c, F8 &pc, float &ph) const {
        pc = ldg256(&P[2 * (size_t) c]);
        ph = pc.a.w;
    }
    __device__ void dpos(u32 b, const F8 &pc, float &dx, float &dy, float &dz, float &hb) const {
        const F8 p = ldg256(&P[2 * (size_t) b]);
        dx = (pc.a.x - p.a.x) + (pc.b.x - p.b.x);
        dy = (pc.a.y - p.a.y) + (pc.b.y - p.b.y);
        dz = (pc.a.z - p.a.z) + (pc.b.z - p.b.z);
        hb = p.a.w;
    }
    __device__ void mult(u32 b, float &nub, float &lomb) const {
        const float2 v = __ldg(&M[b]);
        nub  = v.x;
        lomb = v.y;
    }
};

// -------------------------------------------------------------- staging
// FP64: per rank (ghosts read their source particle) velocity and energy of the
// corrector evaluation being reversed, h, Omega and the cotangents (lambda, mu).
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

__device__ __forceinline__ float hi32(f64 v) { return __double2float_rn(v); }
__device__ __forceinline__ float lo32(f64 v) { return __double2float_rn(v - (f64) __double2float_rn(v)); }

// FP32 records of one corrector evaluation (positions from the rank-ordered copies,
// which already hold the ghosts' shifted positions).
__global__ void k_adj_stage32(u32 N, u32 n, const u32 *__restrict__ sort_index,
                              const u32 *__restrict__ ghost_src, const f64 *__restrict__ sx,
                              const f64 *__restrict__ sy, const f64 *__restrict__ sz,
                              const f64 *__restrict__ vx, const f64 *__restrict__ vy,
                              const f64 *__restrict__ vz, const f64 *__restrict__ u,
                              const f64 *__restrict__ h, const f64 *__restrict__ om,
                              const f64 *__restrict__ lx, const f64 *__restrict__ ly,
                              const f64 *__restrict__ lz, const f64 *__restrict__ mu,
                              const f64 *__restrict__ al, float4 *__restrict__ P,
                              float4 *__restrict__ V, float4 *__restrict__ Lr) {
    u32 r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= N) return;
    u32 id  = sort_index[r];
    u32 src = id < n ? id : ghost_src[id - n];
    f64 x = sx[r], y = sy[r], z = sz[r];
    size_t r2 = 2 * (size_t) r;
    P[r2]     = make_float4(hi32(x), hi32(y), hi32(z), hi32(h[src]));
    P[r2 + 1] = make_float4(lo32(x), lo32(y), lo32(z), hi32(om[src]));
    f64 a = vx[src], b = vy[src], c = vz[src];
    V[r2]     = make_float4(hi32(a), hi32(b), hi32(c), hi32(u[src]));
    V[r2 + 1] = make_float4(lo32(a), lo32(b), lo32(c), hi32(mu[src]));
    Lr[r]     = make_float4(hi32(lx[src]), hi32(ly[src]), hi32(lz[src]), al ? hi32(al[src]) : 0.f);
}
__global__ void k_adj_stage32m(u32 N, u32 n, const u32 *__restrict__ sort_index,
                               const u32 *__restrict__ ghost_src, const f64 *__restrict__ nu,
                               const f64 *__restrict__ lom, float2 *__restrict__ M) {
    u32 r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= N) return;
    u32 id  = sort_index[r];
    u32 src = id < n ? id : ghost_src[id - n];
    M[r]    = make_float2(hi32(nu[src]), hi32(lom[src]));
}

// -------------------------------------------------------------- reverse of derivs
template<class Src, bool LP07>
__global__ void __launch_bounds__(128) k_adj_derivs(RowSpace rs, Src src, AdjParams p,
                                                    AdjLocal L, f64 *g_alpha) {
    using T    = typename Src::T;
    u32 t      = blockIdx.x * blockDim.x + threadIdx.x;
    f64 galpha = 0;
    if (t < rs.n) {
        const T m = T(p.pmass), gm1 = T(p.gamma - 1), gam = T(p.gamma), Rk2 = T(kRkern * kRkern);
        const T aAV = T(p.alpha_AV), bAV = T(p.beta_AV), au = T(p.alpha_u), sig = T(kNorm3d);
        const T half = T(0.5);
        const u32 c = rs.row_rank[t], i = rs.row_local[t];
        const auto rc = src.row(c);
        const auto self = src.nb(c, rc); // the row's own scalars (differences are zero)
        const T uc = self.u, hc = self.h, omc = self.om;
        const T lxc = self.lx, lyc = self.ly, lzc = self.lz, muc = self.mu;
        // viscosity of the row: the constant alpha_AV, or the row's switched alpha
        const bool var = p.av_kind != 0;
        const T alc = var ? self.al : aAV;
        constexpr bool lp07 = LP07;
        const T cs0sq = T(p.cs0 * p.cs0), ir0sq = T(1 / (p.r0 * p.r0)), mq = T(-p.q);
        const T rhoc = rho_of_h(m, hc);
        // adiabatic: P = (gamma - 1) rho u; LP07: c_s^2 = cs0^2 (R^2 / r0^2)^(-q), P = c_s^2 rho
        const T csqc = lp07 ? cs0sq * pow(self.rsq * ir0sq, mq) : gam * gm1 * uc;
        const T Pc   = lp07 ? csqc * rhoc : gm1 * rhoc * uc;
        const T csc  = sqrt(csqc);
        const T subc = rhoc * rhoc * omc;
        const T kc = (subc != T(0) && subc == subc) ? T(1) / subc : T(0), jc = T(1) / (rhoc * omc);
        const T ihc = T(1) / hc, ihc4 = ihc * ihc * ihc * ihc;
        T gxr = 0, gyr = 0, gzr = 0, gvx = 0, gvy = 0, gvz = 0;
        T sP = 0, scs = 0, srho = 0, sk = 0, sj = 0, su = 0, shF = 0, ga = 0;
        const u32 k0 = rs.off[t], k1 = k0 + rs.cnt[t];
        for (u32 k = k0; k < k1; k++) {
            const u32 b = rs.ent[k];
            const auto nb = src.nb(b, rc);
            const T dx = nb.dx, dy = nb.dy, dz = nb.dz;
            const T r2 = dx * dx + dy * dy + dz * dz;
            const T hb = nb.h;
            if (r2 > hc * hc * Rk2 && r2 > hb * hb * Rk2) continue;
            if (r2 == T(0)) continue; // self pair: no contribution and no dependence
            const T r = psqrt(r2), ir = pdiv(T(1), r);
            const T ex = dx * ir, ey = dy * ir, ez = dz * ir;
            const T ub = nb.u, omb = nb.om;
            const T rhob = rho_of_h(m, hb);
            const T csqb = lp07 ? cs0sq * pow(nb.rsq * ir0sq, mq) : gam * gm1 * ub;
            const T Pb   = lp07 ? csqb * rhob : gm1 * rhob * ub;
            const T csb  = psqrt(csqb);
            const T subb = rhob * rhob * omb;
            const T kb = (subb != T(0) && subb == subb) ? pdiv(T(1), subb) : T(0),
                    jb = pdiv(T(1), rhob * omb);
            const T ihb = pdiv(T(1), hb);
            const T qc = r * ihc, qb = r * ihb;
            const T ihb4 = ihb * ihb * ihb * ihb;
            const T d1c = m4_d1(qc), d1b = m4_d1(qb), d2c = m4_d2(qc), d2b = m4_d2(qb);
            const T Fc = sig * d1c * ihc4, Fb = sig * d1b * ihb4;               // dW/dr
            const T Frc = sig * d2c * ihc4 * ihc, Frb = sig * d2b * ihb4 * ihb; // d2W/dr2
            const T Fhc = -sig * (qc * d2c + T(4) * d1c) * ihc4 * ihc;         // d(dW/dr)/dh_c
            const T vabx = nb.dvx, vaby = nb.dvy, vabz = nb.dvz;
            const T w = vabx * ex + vaby * ey + vabz * ez, aw = fabs(w);
            const T alb = var ? nb.al : aAV;
            const T vsc = alc * csc + bAV * aw, vsb = alb * csb + bAV * aw;
            const T tc = -half * rhoc * vsc * w, tb = -half * rhob * vsb * w;
            const bool actc = tc > T(0), actb = tb > T(0);
            // weight of the active branch of max(t, 0): 1, 0, or 1/2 exactly at the kink
            // (w = 0), the symmetric derivative that central differences measure
            const T wc = actc ? T(1) : (tc == T(0) ? half : T(0));
            const T wb = actb ? T(1) : (tb == T(0) ? half : T(0));
            const T Ac = Pc + (actc ? tc : T(0)), Ab = Pb + (actb ? tb : T(0));
            const T dP = Pc - Pb, rbar = half * (rhoc + rhob);
            const T vsu = psqrt(pdiv(fabs(dP), rbar));
            const T J = Fc * jc + Fb * jb;
            const T S = Ac * kc * Fc + Ab * kb * Fb;
            const T Lx = lxc - nb.lx, Ly = lyc - nb.ly, Lz = lzc - nb.lz;
            const T Le = Lx * ex + Ly * ey + Lz * ez;
            const T mub = nb.mu;
            const T du_ = uc - ub, dmu = muc - mub;
            const T cond = half * m * au * dmu * vsu * du_; // multiplies J
            // d q / d w where the viscous pressure is active
            const T dqcw = wc * (-half * rhoc * (vsc + bAV * aw));
            const T dqbw = wb * (-half * rhob * (vsb + bAV * aw));
            const T dSw  = kc * Fc * dqcw + kb * Fb * dqbw;
            const T E    = muc * Ac * kc * Fc + mub * Ab * kb * Fb;
            const T dLw  = -m * Le * dSw + m * E + m * w * (muc * kc * Fc * dqcw + mub * kb * Fb * dqbw);
            const T dLr  = -m * Le * (Ac * kc * Frc + Ab * kb * Frb)
                          + m * w * (muc * Ac * kc * Frc + mub * Ab * kb * Frb)
                          + cond * (Frc * jc + Frb * jb);
            // dL/de (e free), then the projection of r_vec -> (r, e)
            const T dex = -m * S * Lx + dLw * vabx, dey = -m * S * Ly + dLw * vaby,
                    dez = -m * S * Lz + dLw * vabz;
            const T ede = dex * ex + dey * ey + dez * ez;
            gxr += dLr * ex + (dex - ede * ex) * ir;
            gyr += dLr * ey + (dey - ede * ey) * ir;
            gzr += dLr * ez + (dez - ede * ez) * ir;
            gvx += dLw * ex;
            gvy += dLw * ey;
            gvz += dLw * ez;
            // particle-c scalars
            const T dLAc  = -m * Le * kc * Fc + m * w * muc * kc * Fc;
            const T dLvsu = half * m * au * dmu * du_ * J;
            const T dvsuP = vsu > T(0) ? pdiv(dP > T(0) ? T(1) : T(-1), T(2) * rbar * vsu) : T(0);
            const T dvsur = vsu > T(0) ? pdiv(-vsu, T(4) * rbar) : T(0);
            sP += dLAc + dLvsu * dvsuP;
            if (actc) scs += dLAc * (-half * rhoc * alc * w);
            srho += (actc ? dLAc * pdiv(tc, rhoc) : T(0)) + dLvsu * dvsur;
            sk += -m * Le * Ac * Fc + m * w * muc * Ac * Fc;
            sj += cond * Fc;
            su += half * m * au * dmu * vsu * J;
            shF += (-m * Le * Ac * kc + m * w * muc * Ac * kc + cond * jc) * Fhc;
            const T dqca = actc ? -half * rhoc * csc * w : T(0);
            if (var) {
                // alpha_c of the varying forms: every pair term it enters, the row's own
                // (through q_c in f_cb and g_cb) and the neighbour's (q_c in f_bc), which
                // together give -m (lambda_c - lambda_b).e k_c F_c dq_c + mu_c m w k_c F_c dq_c
                ga += -m * Le * kc * Fc * dqca + muc * m * w * kc * Fc * dqca;
            } else {
                // alpha_AV: this row's own pair term only (lambda_c . f_cb + mu_c g_cb)
                const T dqba = actb ? -half * rhob * csb * w : T(0);
                const T lce  = lxc * ex + lyc * ey + lzc * ez;
                ga += -m * lce * (kc * Fc * dqca + kb * Fb * dqba) + muc * m * w * kc * Fc * dqca;
            }
        }
        const f64 rhoc_ = rhoc, kc_ = kc, jc_ = jc, omc_ = omc, hc_ = hc;
        f64 gu, grho, gpx = 0, gpy = 0, gpz = 0;
        if constexpr (lp07) {
            // P, c_s depend on the position and rho, not on u
            gu   = (f64) su;
            grho = (f64) sP * (f64) csqc + (f64) srho + (f64) sk * (-2 * kc_ / rhoc_)
                   + (f64) sj * (-jc_ / rhoc_);
            // d c_s^2 / d x = -2 q c_s^2 x / R^2
            T ax, ay, az;
            src.apos(rc, ax, ay, az);
            const f64 dcs2 = -2 * p.q * (f64) csqc / (f64) self.rsq;
            const f64 coef = ((f64) sP * rhoc_ + (csc > T(0) ? (f64) scs / (2 * (f64) csc) : 0)) * dcs2;
            gpx = coef * (f64) ax;
            gpy = coef * (f64) ay;
            gpz = coef * (f64) az;
        } else {
            gu = (f64) sP * (p.gamma - 1) * rhoc_
                 + (csc > T(0) ? (f64) scs * p.gamma * (p.gamma - 1) / (2 * (f64) csc) : 0)
                 + (f64) su;
            grho = (f64) sP * (p.gamma - 1) * (f64) uc + (f64) srho
                   + (f64) sk * (-2 * kc_ / rhoc_) + (f64) sj * (-jc_ / rhoc_);
        }
        const f64 gh  = grho * (-3 * rhoc_ / hc_) + (f64) shF;
        const f64 gom = (f64) sk * (-kc_ / omc_) + (f64) sj * (-jc_ / omc_);
        L.lv[0][i] += gvx;
        L.lv[1][i] += gvy;
        L.lv[2][i] += gvz;
        L.lu[i] += gu;
        L.gx[0][i] += (f64) gxr + gpx;
        L.gx[1][i] += (f64) gyr + gpy;
        L.gx[2][i] += (f64) gzr + gpz;
        L.gh[i] += gh;
        L.gom[i] += gom;
        if (var) L.gal[i] += (f64) ga;
        else galpha = ga;
    }
    galpha = block_reduce(galpha, OpAddF64{}, 0.0);
    if (threadIdx.x == 0 && galpha != 0) atomicAdd(g_alpha, galpha);
}

// -------------------------------------------------------------- reverse of Omega and h'
// nu_c = -(gh_c + gom_c dOmega_c/dh_c) h_c / (3 rho_c Omega_c), lom_c = gom_c h_c/(3 rho_c).
template<class Src>
__global__ void __launch_bounds__(256) k_adj_omega_a(RowSpace rs, Src src, const f64 *__restrict__ h_local,
                                                     const f64 *__restrict__ om_local, f64 pmass,
                                                     AdjLocal L) {
    using T = typename Src::T;
    u32 t   = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= rs.n) return;
    const u32 c = rs.row_rank[t], i = rs.row_local[t];
    const T sig = T(kNorm3d);
    typename std::conditional<std::is_same<T, f64>::value, f64, F8>::type pc;
    T px = 0, py = 0, pz = 0, hc;
    if constexpr (std::is_same<T, f64>::value) src.pos(c, px, py, pz, hc);
    else src.pos(c, pc, hc);
    const T ihc = T(1) / hc, ih4 = ihc * ihc * ihc * ihc;
    T S = 0, Sh = 0; // sum dW/dh, sum d2W/dh2 (self pair included)
    const u32 k0 = rs.off[t], k1 = k0 + rs.cnt[t];
    for (u32 k = k0; k < k1; k++) {
        const u32 b = rs.ent[k];
        T dx, dy, dz, hb;
        if constexpr (std::is_same<T, f64>::value) src.dpos(b, px, py, pz, dx, dy, dz, hb);
        else src.dpos(b, pc, dx, dy, dz, hb);
        const T q = psqrt(dx * dx + dy * dy + dz * dz) * ihc;
        if (q >= T(2)) continue;
        const T f0 = m4_f(q), f1 = m4_d1(q), f2 = m4_d2(q);
        S += -sig * (T(3) * f0 + q * f1) * ih4;
        Sh += sig * (T(12) * f0 + T(8) * q * f1 + q * q * f2) * ih4 * ihc;
    }
    // scalar tail in FP64 from the local h and Omega
    const f64 h64 = h_local[i], om64 = om_local[i];
    const f64 rho   = rho_of_h(pmass, h64);
    const f64 coef  = h64 / (3 * rho); // Omega = 1 + coef S, coef = h^4 / (3 m hfact^3)
    const f64 dOmdh = 4 * coef / h64 * pmass * (f64) S + coef * pmass * (f64) Sh;
    const f64 gom   = L.gom[i];
    const f64 ghtot = L.gh[i] + gom * dOmdh;
    L.nu[i]  = -ghtot * h64 / (3 * rho * om64);
    L.lom[i] = gom * coef;
}

// gx_c += sum_b e_cb m [lom_c dG/dr(h_c) + lom_b dG/dr(h_b) + nu_c dW/dr(h_c) + nu_b dW/dr(h_b)]
template<class Src>
__global__ void __launch_bounds__(256) k_adj_omega_b(RowSpace rs, Src src, f64 pmass, AdjLocal L) {
    using T = typename Src::T;
    u32 t   = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= rs.n) return;
    const u32 c = rs.row_rank[t], i = rs.row_local[t];
    const T sig = T(kNorm3d);
    typename std::conditional<std::is_same<T, f64>::value, f64, F8>::type pc;
    T px = 0, py = 0, pz = 0, hc;
    if constexpr (std::is_same<T, f64>::value) src.pos(c, px, py, pz, hc);
    else src.pos(c, pc, hc);
    T nuc, lomc;
    src.mult(c, nuc, lomc);
    const T ihc = T(1) / hc, ihc5 = ihc * ihc * ihc * ihc * ihc;
    T gx = 0, gy = 0, gz = 0;
    const u32 k0 = rs.off[t], k1 = k0 + rs.cnt[t];
    for (u32 k = k0; k < k1; k++) {
        const u32 b = rs.ent[k];
        T dx, dy, dz, hb;
        if constexpr (std::is_same<T, f64>::value) src.dpos(b, px, py, pz, dx, dy, dz, hb);
        else src.dpos(b, pc, dx, dy, dz, hb);
        const T r2 = dx * dx + dy * dy + dz * dz;
        if (r2 == T(0)) continue;
        const T r = psqrt(r2), ir = pdiv(T(1), r);
        const T ihb = pdiv(T(1), hb);
        const T qc = r * ihc, qb = r * ihb;
        if (qc >= T(2) && qb >= T(2)) continue;
        T nub, lomb;
        src.mult(b, nub, lomb);
        const T d1c = m4_d1(qc), d2c = m4_d2(qc), d1b = m4_d1(qb), d2b = m4_d2(qb);
        const T ihb5 = ihb * ihb * ihb * ihb * ihb;
        const T Grc = -sig * (T(4) * d1c + qc * d2c) * ihc5, Grb = -sig * (T(4) * d1b + qb * d2b) * ihb5;
        const T Fc = sig * d1c * ihc5 * hc, Fb = sig * d1b * ihb5 * hb;
        const T s = T(pmass) * (lomc * Grc + lomb * Grb + nuc * Fc + nub * Fb) * ir;
        gx += s * dx;
        gy += s * dy;
        gz += s * dz;
    }
    L.gx[0][i] += gx;
    L.gx[1][i] += gy;
    L.gx[2][i] += gz;
}

// -------------------------------------------------------------- varying viscosity
// Forward of evaluation k (Solver.cpp:2261-2370): per row a, over the pairs inside a's
// support, with g = m dW/dr(r, h_a) r_hat, r = x_a - x_b, v = v_a - v_b, w = A_a - A_b
// (A: the accelerations of the previous evaluation),
//   sd = sum v.g, sc = sum v x g, R_ij = -sum r_i g_j, Dv_ji = -sum v_i g_j, Da_ji = -sum w_i g_j,
//   div v = -k sd, curl v = -k sc (k = 1 / (Omega rho)),
//   d(div v)/dt = tr(Ri Da) - tr((Ri Dv)^2), Ri = R^-1;
// then the switch gives alpha of the evaluation from (div v, curl v, d(div v)/dt) and the
// step's input alpha_AV, sound speed and h (UpdateViscosity.cpp:53-118, 122-215).
// Reverse: pass A recomputes a row's sums, reverses the switch with the row's alpha
// cotangent (from the derivatives' reverse), and folds the cotangents of the sums into 24
// numbers per particle: with Rb, Dvb, Dab, sdb, scb the cotangents of R, Dv, Da, sd, sc,
// a pair's linearised contribution is, for g = m F e,
//   d/dv = Qv g,  d/dw = Qw g,  d/dr = -Rs g + (terms through g(r)),
//   d/dg = Qv^T v - Rs r + Qw^T w,
// with Qv = sdb I - Dvb^T + C(scb) (C(s) g = g x s), Qw = -Dab^T and Rs the symmetric part
// of Rb (R's terms r_i g_j are symmetric, so only Rs enters): Rs (6, xx xy xz yy yz zz),
// Qv (9, row-major), Qw (9).  Pass B gathers, for row c, the derivative with respect to
// c's position, velocity and previous acceleration of every pair term c enters: its own
// row's (with its own cotangents) and each neighbour's (with the neighbour's, staged by
// rank: 96 bytes, three 256-bit loads in FP32).

// velocity-gradient sources: per rank position, v of the evaluation, A of the previous
// one, h and the staged cotangents of the sums
struct VG64 {
    using T = f64;
    const f64 *x, *y, *z, *vx, *vy, *vz, *ax, *ay, *az, *h, *M;
    struct Row {
        f64 x, y, z, vx, vy, vz, ax, ay, az, h;
    };
    __device__ Row row(u32 c) const {
        return Row{x[c], y[c], z[c], vx[c], vy[c], vz[c], ax[c], ay[c], az[c], h[c]};
    }
    __device__ f64 hrow(const Row &r) const { return r.h; }
    __device__ void pair(u32 b, const Row &r, f64 d[3], f64 dv[3], f64 dw[3], f64 &hb) const {
        d[0]  = r.x - x[b];
        d[1]  = r.y - y[b];
        d[2]  = r.z - z[b];
        dv[0] = r.vx - vx[b];
        dv[1] = r.vy - vy[b];
        dv[2] = r.vz - vz[b];
        dw[0] = r.ax - ax[b];
        dw[1] = r.ay - ay[b];
        dw[2] = r.az - az[b];
        hb    = h[b];
    }
    __device__ void mat(u32 b, f64 out[24]) const {
        const f64 *q = M + 32 * (size_t) b;
#pragma unroll
        for (int k = 0; k < 24; k++) out[k] = q[k];
    }
};
// FP32: the position and velocity records of the derivatives' reverse (hi/lo pairs),
// A[r] = {A_x, A_y, A_z, alpha}, M: 6 float4 per rank (24 floats, 32-byte aligned)
struct VG32 {
    using T = float;
    const float4 *P, *V, *A, *M;
    struct Row {
        F8 p, v;
        float4 a;
    };
    __device__ Row row(u32 c) const {
        return Row{ldg256(&P[2 * (size_t) c]), ldg256(&V[2 * (size_t) c]), __ldg(&A[c])};
    }
    __device__ float hrow(const Row &r) const { return r.p.a.w; }
    __device__ void pair(u32 b, const Row &r, float d[3], float dv[3], float dw[3],
                         float &hb) const {
        const F8 p = ldg256(&P[2 * (size_t) b]), v = ldg256(&V[2 * (size_t) b]);
        const float4 a = __ldg(&A[b]);
        d[0]  = (r.p.a.x - p.a.x) + (r.p.b.x - p.b.x);
        d[1]  = (r.p.a.y - p.a.y) + (r.p.b.y - p.b.y);
        d[2]  = (r.p.a.z - p.a.z) + (r.p.b.z - p.b.z);
        dv[0] = (r.v.a.x - v.a.x) + (r.v.b.x - v.b.x);
        dv[1] = (r.v.a.y - v.a.y) + (r.v.b.y - v.b.y);
        dv[2] = (r.v.a.z - v.a.z) + (r.v.b.z - v.b.z);
        dw[0] = r.a.x - a.x;
        dw[1] = r.a.y - a.y;
        dw[2] = r.a.z - a.z;
        hb    = p.a.w;
    }
    __device__ void mat(u32 b, float out[24]) const {
        const float4 *q = M + 6 * (size_t) b;
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const F8 v = ldg256(&q[2 * k]);
            out[8 * k + 0] = v.a.x;
            out[8 * k + 1] = v.a.y;
            out[8 * k + 2] = v.a.z;
            out[8 * k + 3] = v.a.w;
            out[8 * k + 4] = v.b.x;
            out[8 * k + 5] = v.b.y;
            out[8 * k + 6] = v.b.z;
            out[8 * k + 7] = v.b.w;
        }
    }
};

// d/d(r, v, w) of one pair term of a row with folded cotangents M (Rs, Qv, Qw), given
// g = m F e: dr (direct and through g), dv, dw, and ge = (dL/dg).e for the h derivative
template<class T>
__device__ __forceinline__ void vg_pair_grad(const T M[24], T m, T F, T Fr, T rr, const T e[3],
                                             const T r[3], const T v[3], const T w[3], T dr[3],
                                             T dv[3], T dw[3], T &ge) {
    const T g[3] = {m * F * e[0], m * F * e[1], m * F * e[2]};
    const T Rs[3][3] = {{M[0], M[1], M[2]}, {M[1], M[3], M[4]}, {M[2], M[4], M[5]}};
    T gb[3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
        T a = 0, b = 0, c = 0, d = 0;
#pragma unroll
        for (int j = 0; j < 3; j++) {
            a += M[6 + 3 * i + j] * g[j];
            b += M[15 + 3 * i + j] * g[j];
            c -= Rs[i][j] * g[j];
            d += M[6 + 3 * j + i] * v[j] - Rs[i][j] * r[j] + M[15 + 3 * j + i] * w[j];
        }
        dv[i] = a;
        dw[i] = b;
        dr[i] = c;
        gb[i] = d;
    }
    ge = gb[0] * e[0] + gb[1] * e[1] + gb[2] * e[2];
    const T ir = T(1) / rr;
#pragma unroll
    for (int i = 0; i < 3; i++) dr[i] += m * (Fr * ge * e[i] + F * (gb[i] - ge * e[i]) * ir);
}

template<class T>
__device__ __forceinline__ void inv33t(const T m[3][3], T r[3][3]) {
    const T det = m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1])
                - m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0])
                + m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
    const T id = T(1) / det;
    r[0][0] = (m[1][1] * m[2][2] - m[1][2] * m[2][1]) * id;
    r[0][1] = (m[0][2] * m[2][1] - m[0][1] * m[2][2]) * id;
    r[0][2] = (m[0][1] * m[1][2] - m[0][2] * m[1][1]) * id;
    r[1][0] = (m[1][2] * m[2][0] - m[1][0] * m[2][2]) * id;
    r[1][1] = (m[0][0] * m[2][2] - m[0][2] * m[2][0]) * id;
    r[1][2] = (m[0][2] * m[1][0] - m[0][0] * m[1][2]) * id;
    r[2][0] = (m[1][0] * m[2][1] - m[1][1] * m[2][0]) * id;
    r[2][1] = (m[0][1] * m[2][0] - m[0][0] * m[2][1]) * id;
    r[2][2] = (m[0][0] * m[1][1] - m[0][1] * m[1][0]) * id;
}

// Reverse of the switch of one particle: from the cotangent gn of the switched alpha,
// the cotangents of div v, curl v, d(div v)/dt, and accumulations into the input alpha,
// sound speed, h and the switch parameters (alpha_min, alpha_max, sigma_decay).
// Comparisons as in the forward (k_cd10 / k_mm97); a kink takes the branch the forward
// value took.
__device__ __forceinline__ void switch_reverse(const AdjParams &p, f64 gn, f64 div, const f64 curl[3],
                                               f64 dtdiv, f64 cs, f64 h, f64 al, f64 &gdiv,
                                               f64 gcurl[3], f64 &gdt, f64 &gal, f64 &gcs, f64 &gh,
                                               f64 gpar[3]) {
    gdiv = gdt = 0;
    gcurl[0] = gcurl[1] = gcurl[2] = 0;
    gal = gcs = gh = 0;
    const f64 dt = p.dt, sig = p.sigma_decay;
    const f64 inv_tau = cs * sig / h, f = dt * inv_tau, euler = 1 / (1 + f);
    f64 gf = 0;
    if (p.av_kind == 2) {
        // MM97: na = (alpha + max(-div, 0) dt + f alpha_min) euler, alpha' = min(na, alpha_max)
        const f64 md = -div, src = md > 0 ? md : 0;
        const f64 na = (al + src * dt + f * p.alpha_min) * euler;
        if (!(na < p.alpha_max)) {
            gpar[1] += gn;
        } else {
            gal += gn * euler;
            if (md > 0) gdiv = -gn * dt * euler;
            gpar[0] += gn * f * euler;
            gf = gn * euler * (p.alpha_min - na);
        }
    } else {
        const f64 eps = 2.220446049250313e-16;
        const f64 md = -div;
        const f64 fac0 = md > 0 ? md : 0, fac = fac0 * fac0;
        const f64 tr = curl[0] * curl[0] + curl[1] * curl[1] + curl[2] * curl[2];
        const bool bal_on = fac + tr > eps;
        const f64 bal = bal_on ? fac / (fac + tr) : 1;
        const f64 mdt = -dtdiv, mdtp = mdt > 0 ? mdt : 0;
        const f64 A = bal * mdtp, temp = cs * cs;
        f64 loc = cs > 0 ? 10 * h * h * A / temp : p.alpha_min;
        const bool clamped = !(loc < p.alpha_max);
        loc = clamped ? p.alpha_max : loc;
        const bool has_cs = temp > eps;
        loc = has_cs ? loc : p.alpha_min;
        f64 gloc;
        if (loc > al) {
            gloc = gn; // alpha' = alpha_loc
        } else {
            const f64 na = (al + loc * f) * euler;
            gal += gn * euler;
            gloc = gn * f * euler;
            gf   = gn * euler * (loc - na);
        }
        if (!has_cs || !(cs > 0)) {
            gpar[0] += gloc;
        } else if (clamped) {
            gpar[1] += gloc;
        } else {
            gh += gloc * 20 * h * A / temp;
            gcs += gloc * (-20 * h * h * A / (temp * cs));
            const f64 gA = gloc * 10 * h * h / temp;
            if (mdt > 0) {
                gdt = -gA * bal;
                const f64 gbal = gA * mdtp;
                if (bal_on) {
                    const f64 s2 = (fac + tr) * (fac + tr);
                    const f64 gfac = gbal * tr / s2, gtr = -gbal * fac / s2;
                    if (md > 0) gdiv = -gfac * 2 * md;
                    gcurl[0] = gtr * 2 * curl[0];
                    gcurl[1] = gtr * 2 * curl[1];
                    gcurl[2] = gtr * 2 * curl[2];
                }
            }
        }
    }
    // f = dt cs sigma / h
    gcs += gf * dt * sig / h;
    gh += -gf * dt * cs * sig / (h * h);
    gpar[2] += gf * dt * cs / h;
}

template<class VS>
__global__ void __launch_bounds__(128) k_adj_vg_a(RowSpace rs, VS src, AdjParams p, AdjLocal L,
                                                  const f64 *__restrict__ h_local,
                                                  const f64 *__restrict__ om_local,
                                                  f64 *__restrict__ Mloc, f64 *g_av,
                                                  const float *__restrict__ taped) {
    using T = typename VS::T;
    u32 t = blockIdx.x * blockDim.x + threadIdx.x;
    f64 gpar[3] = {0, 0, 0};
    if (t < rs.n) {
        const u32 c = rs.row_rank[t], i = rs.row_local[t];
        const T m = T(p.pmass), sig = T(kNorm3d);
        T R[3][3] = {}, Dv[3][3] = {}, Da[3][3] = {}, sd = 0, sc[3] = {0, 0, 0};
        const u32 k0 = rs.off[t], k1 = taped ? k0 : k0 + rs.cnt[t];
        if (taped) {
            // the forward pass's own sums (bare, times the pair mass here)
            const float *q = taped + 24 * (size_t) i;
            R[0][0] = m * T(q[0]);
            R[0][1] = R[1][0] = m * T(q[1]);
            R[0][2] = R[2][0] = m * T(q[2]);
            R[1][1] = m * T(q[3]);
            R[1][2] = R[2][1] = m * T(q[4]);
            R[2][2] = m * T(q[5]);
#pragma unroll
            for (int a = 0; a < 3; a++)
#pragma unroll
                for (int b = 0; b < 3; b++) {
                    Dv[a][b] = m * T(q[6 + 3 * a + b]);
                    Da[a][b] = m * T(q[15 + 3 * a + b]);
                }
            // sd = sum v.g = -tr Dv, sc = sum v x g: sc_x = Dv[1][2] - Dv[2][1], ...
            sd    = -(Dv[0][0] + Dv[1][1] + Dv[2][2]);
            sc[0] = Dv[1][2] - Dv[2][1];
            sc[1] = Dv[2][0] - Dv[0][2];
            sc[2] = Dv[0][1] - Dv[1][0];
        }
        const auto rc = src.row(c);
        const T hc = src.hrow(rc);
        const T ihc = T(1) / hc, ih4 = ihc * ihc * ihc * ihc;
        for (u32 k = k0; k < k1; k++) {
            T d[3], dv[3], dw[3], hb;
            src.pair(rs.ent[k], rc, d, dv, dw, hb);
            const T r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            const T rr = psqrt(r2);
            if (!(rr >= T(1e-9))) continue;
            const T qc = rr * ihc;
            if (qc >= T(2)) continue;
            const T F = sig * m4_d1(qc) * ih4, ir = pdiv(T(1), rr);
            const T g[3] = {m * F * d[0] * ir, m * F * d[1] * ir, m * F * d[2] * ir};
            sd += dv[0] * g[0] + dv[1] * g[1] + dv[2] * g[2];
            sc[0] += dv[1] * g[2] - dv[2] * g[1];
            sc[1] += dv[2] * g[0] - dv[0] * g[2];
            sc[2] += dv[0] * g[1] - dv[1] * g[0];
#pragma unroll
            for (int a = 0; a < 3; a++)
#pragma unroll
                for (int b = 0; b < 3; b++) {
                    R[a][b] -= d[a] * g[b];
                    Dv[b][a] -= dv[a] * g[b];
                    Da[b][a] -= dw[a] * g[b];
                }
        }
        const f64 h64 = h_local[i], om64 = om_local[i];
        const f64 rho = rho_of_h(p.pmass, h64), kk = 1 / (om64 * rho);
        const f64 div = -kk * (f64) sd;
        const f64 curl[3] = {-kk * (f64) sc[0], -kk * (f64) sc[1], -kk * (f64) sc[2]};
        T Ri[3][3], Gv[3][3];
        inv33t(R, Ri);
        T dtd = 0;
#pragma unroll
        for (int a = 0; a < 3; a++)
#pragma unroll
            for (int b = 0; b < 3; b++) {
                T gv = 0, ga = 0;
#pragma unroll
                for (int q = 0; q < 3; q++) {
                    gv += Ri[a][q] * Dv[q][b];
                    ga += Ri[a][q] * Da[q][b];
                }
                Gv[a][b] = gv;
                if (a == b) dtd += ga;
            }
#pragma unroll
        for (int a = 0; a < 3; a++)
#pragma unroll
            for (int b = 0; b < 3; b++) dtd -= Gv[b][a] * Gv[a][b];
        // the switch
        f64 gdiv, gcurl[3], gdt, gal, gcs, gh;
        switch_reverse(p, L.gal[i], div, curl, (f64) dtd, p.cs_in[i], h64, p.alpha_in[i], gdiv,
                       gcurl, gdt, gal, gcs, gh, gpar);
        L.gain[i] += gal;
        L.gcsin[i] += gcs;
        // k = 1 / (Omega rho(h)): d/dOmega = -k / Omega, d/dh = 3 k / h
        const f64 kb = -((f64) sd * gdiv + (f64) sc[0] * gcurl[0] + (f64) sc[1] * gcurl[1]
                         + (f64) sc[2] * gcurl[2]);
        L.gom[i] += kb * (-kk / om64);
        L.gh[i] += gh + kb * 3 * kk / h64;
        // cotangents of the sums
        const T gt = T(gdt);
        T Gvb[3][3], Ria[3][3];
#pragma unroll
        for (int a = 0; a < 3; a++)
#pragma unroll
            for (int b = 0; b < 3; b++) Gvb[a][b] = T(-2) * gt * Gv[b][a];
        // Dab[q][b] = sum_a Ri[a][q] Gab[a][b] = gt Ri[b][q]; Dvb[q][b] = sum_a Ri[a][q] Gvb[a][b]
        T Dvb[3][3], Dab[3][3];
#pragma unroll
        for (int q = 0; q < 3; q++)
#pragma unroll
            for (int b = 0; b < 3; b++) {
                T dvb = 0;
#pragma unroll
                for (int a = 0; a < 3; a++) dvb += Ri[a][q] * Gvb[a][b];
                Dvb[q][b] = dvb;
                Dab[q][b] = gt * Ri[b][q];
            }
        // Rib[a][q] = sum_b Gab[a][b] Da[q][b] + Gvb[a][b] Dv[q][b]
#pragma unroll
        for (int a = 0; a < 3; a++)
#pragma unroll
            for (int q = 0; q < 3; q++) {
                T v = gt * Da[q][a];
#pragma unroll
                for (int b = 0; b < 3; b++) v += Gvb[a][b] * Dv[q][b];
                Ria[a][q] = v;
            }
        // Rb = -Ri^T Rib Ri^T: Rb[x][y] = -sum_a sum_q Ri[a][x] Rib[a][q] Ri[y][q]
        T Rb[3][3];
#pragma unroll
        for (int x = 0; x < 3; x++)
#pragma unroll
            for (int y = 0; y < 3; y++) {
                T v = 0;
#pragma unroll
                for (int a = 0; a < 3; a++)
#pragma unroll
                    for (int q = 0; q < 3; q++) v += Ri[a][x] * Ria[a][q] * Ri[y][q];
                Rb[x][y] = -v;
            }
        const T sdb = T(-kk * gdiv);
        const T sb[3] = {T(-kk * gcurl[0]), T(-kk * gcurl[1]), T(-kk * gcurl[2])};
        const T C[3][3] = {{0, sb[2], -sb[1]}, {-sb[2], 0, sb[0]}, {sb[1], -sb[0], 0}};
        f64 *out = Mloc + 32 * (size_t) i;
        out[0] = (f64) Rb[0][0];
        out[1] = (f64) (T(0.5) * (Rb[0][1] + Rb[1][0]));
        out[2] = (f64) (T(0.5) * (Rb[0][2] + Rb[2][0]));
        out[3] = (f64) Rb[1][1];
        out[4] = (f64) (T(0.5) * (Rb[1][2] + Rb[2][1]));
        out[5] = (f64) Rb[2][2];
#pragma unroll
        for (int a = 0; a < 3; a++)
#pragma unroll
            for (int b = 0; b < 3; b++) {
                out[6 + 3 * a + b]  = (f64) ((a == b ? sdb : T(0)) - Dvb[b][a] + C[a][b]);
                out[15 + 3 * a + b] = (f64) -Dab[b][a];
            }
        L.gal[i] = 0; // consumed
    }
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const f64 v = block_reduce(gpar[k], OpAddF64{}, 0.0);
        if (threadIdx.x == 0 && v != 0) atomicAdd(&g_av[k], v);
    }
}

template<class VS>
__global__ void __launch_bounds__(128) k_adj_vg_b(RowSpace rs, VS src, AdjParams p, AdjLocal L) {
    using T = typename VS::T;
    u32 t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= rs.n) return;
    const u32 c = rs.row_rank[t], i = rs.row_local[t];
    const auto rc = src.row(c);
    const T hc = src.hrow(rc), m = T(p.pmass), sig = T(kNorm3d);
    const T ihc = T(1) / hc;
    T Mc[24];
    src.mat(c, Mc);
    T gx[3] = {0, 0, 0}, gv[3] = {0, 0, 0}, gw[3] = {0, 0, 0}, gh = 0;
    const u32 k0 = rs.off[t], k1 = k0 + rs.cnt[t];
    for (u32 k = k0; k < k1; k++) {
        const u32 b = rs.ent[k];
        T d[3], dv[3], dw[3], hb;
        src.pair(b, rc, d, dv, dw, hb);
        const T r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        const T rr = psqrt(r2);
        if (!(rr >= T(1e-9))) continue;
        const T ir = pdiv(T(1), rr);
        const T e[3] = {d[0] * ir, d[1] * ir, d[2] * ir};
        const T qc = rr * ihc, ihb = pdiv(T(1), hb), qb = rr * ihb;
        T dr[3], dvv[3], dww[3], ge;
        if (qc < T(2)) {
            // the row's own term (pair (c, b) of c's sums)
            const T ih4 = ihc * ihc * ihc * ihc;
            const T d1 = m4_d1(qc), d2 = m4_d2(qc);
            const T F = sig * d1 * ih4, Fr = sig * d2 * ih4 * ihc;
            vg_pair_grad(Mc, m, F, Fr, rr, e, d, dv, dw, dr, dvv, dww, ge);
#pragma unroll
            for (int a = 0; a < 3; a++) {
                gx[a] += dr[a];
                gv[a] += dvv[a];
                gw[a] += dww[a];
            }
            gh += m * (-sig * (qc * d2 + T(4) * d1) * ih4 * ihc) * ge;
        }
        if (qb < T(2)) {
            // the neighbour's term (pair (b, c) of b's sums): arguments negated, and the
            // derivative with respect to c's inputs is minus that with respect to them
            T Mb[24];
            src.mat(b, Mb);
            const T ih4 = ihb * ihb * ihb * ihb;
            const T d1 = m4_d1(qb), d2 = m4_d2(qb);
            const T F = sig * d1 * ih4, Fr = sig * d2 * ih4 * ihb;
            const T en[3] = {-e[0], -e[1], -e[2]}, dn[3] = {-d[0], -d[1], -d[2]};
            const T vn[3] = {-dv[0], -dv[1], -dv[2]}, wn[3] = {-dw[0], -dw[1], -dw[2]};
            vg_pair_grad(Mb, m, F, Fr, rr, en, dn, vn, wn, dr, dvv, dww, ge);
#pragma unroll
            for (int a = 0; a < 3; a++) {
                gx[a] -= dr[a];
                gv[a] -= dvv[a];
                gw[a] -= dww[a];
            }
        }
    }
#pragma unroll
    for (int a = 0; a < 3; a++) {
        L.gx[a][i] += (f64) gx[a];
        L.lv[a][i] += (f64) gv[a];
        L.lamp[a][i] += (f64) gw[a];
    }
    L.gh[i] += (f64) gh;
}

// per rank: the previous evaluation's accelerations and the evaluation's alpha (ghosts
// copy their source); FP64 arrays or FP32 records {A, alpha}
__global__ void k_adj_av_stage(u32 N, u32 n, const u32 *__restrict__ sort_index,
                               const u32 *__restrict__ ghost_src, const f64 *__restrict__ snap_av,
                               f64 *__restrict__ A64, float4 *__restrict__ A32) {
    u32 r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= N) return;
    u32 id  = sort_index[r];
    u32 src = id < n ? id : ghost_src[id - n];
    size_t n_ = n, N_ = N;
    const f64 ax = snap_av[src], ay = snap_av[n_ + src], az = snap_av[2 * n_ + src];
    const f64 al = snap_av[3 * n_ + src];
    if (A64) {
        A64[r]          = ax;
        A64[N_ + r]     = ay;
        A64[2 * N_ + r] = az;
        A64[3 * N_ + r] = al;
    } else {
        A32[r] = make_float4(hi32(ax), hi32(ay), hi32(az), hi32(al));
    }
}
// the 24 folded cotangents of the sums by rank (FP64, 32 per rank, or FP32, 6 float4)
__global__ void k_adj_vg_stage(u32 N, u32 n, const u32 *__restrict__ sort_index,
                               const u32 *__restrict__ ghost_src, const f64 *__restrict__ Mloc,
                               f64 *__restrict__ M64, float4 *__restrict__ M32) {
    u32 r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= N) return;
    u32 id  = sort_index[r];
    u32 src = id < n ? id : ghost_src[id - n];
    const f64 *q = Mloc + 32 * (size_t) src;
    if (M64) {
        f64 *o = M64 + 32 * (size_t) r;
#pragma unroll
        for (int k = 0; k < 24; k++) o[k] = q[k];
    } else {
#pragma unroll
        for (int k = 0; k < 6; k++)
            M32[6 * (size_t) r + k] = make_float4(hi32(q[4 * k]), hi32(q[4 * k + 1]),
                                                  hi32(q[4 * k + 2]), hi32(q[4 * k + 3]));
    }
}
// the stored sound speed after the step is the last evaluation's: its cotangent goes to
// that evaluation's energy (adiabatic, c_s^2 = gamma (gamma - 1) u) or to the positions
// (LP07, c_s = cs0 (R^2 / r0^2)^(-q/2))
__global__ void k_adj_cs_out(u32 n, const f64 *__restrict__ gcs, const f64 *__restrict__ u_last,
                             const f64 *__restrict__ xl, const f64 *__restrict__ yl,
                             const f64 *__restrict__ zl, AdjParams p, AdjLocal L) {
    u32 i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const f64 g = gcs[i];
    if (g == 0) return;
    if (p.eos_kind == 1) {
        const f64 x = xl[i], y = yl[i], z = zl[i], R2 = x * x + y * y + z * z;
        const f64 cs = p.cs0 * pow(R2 / (p.r0 * p.r0), -p.q / 2);
        const f64 s = g * (-p.q) * cs / R2;
        L.gx[0][i] += s * x;
        L.gx[1][i] += s * y;
        L.gx[2][i] += s * z;
    } else {
        const f64 gg = p.gamma * (p.gamma - 1), u = u_last[i];
        const f64 cs = sqrt(gg * u);
        if (cs > 0) L.lu[i] += g * gg / (2 * cs);
    }
}

// -------------------------------------------------------------- external point mass
// a_ext = mGM r / |r|^3 at the local positions x' of the step: gx += (d a_ext / d x)^T lam
// = mGM (lam / r^3 - 3 r (r . lam) / r^5) for the cotangent lam of the corrector
// evaluation being reversed.
__global__ void k_adj_ext(u32 n, const f64 *__restrict__ xl, const f64 *__restrict__ yl,
                          const f64 *__restrict__ zl, f64 mGM, AdjLocal L) {
    u32 i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const f64 x = xl[i], y = yl[i], z = zl[i];
    const f64 r2 = x * x + y * y + z * z, r = sqrt(r2), ir3 = 1 / (r2 * r), ir5 = ir3 / r2;
    const f64 lx = L.lam[0][i], ly = L.lam[1][i], lz = L.lam[2][i];
    const f64 rl = x * lx + y * ly + z * lz;
    L.gx[0][i] += mGM * (lx * ir3 - 3 * x * rl * ir5);
    L.gx[1][i] += mGM * (ly * ir3 - 3 * y * rl * ir5);
    L.gx[2][i] += mGM * (lz * ir3 - 3 * z * rl * ir5);
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
    if (cs.alpha) {
        // the switched alpha of the last evaluation is the step's output alpha_AV
        L.gal[i]   = cs.alpha[i];
        L.gain[i]  = 0;
        L.gcsin[i] = 0;
    }
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
    if (cs.alpha) {
        cs.alpha[i] = L.gain[i];
        cs.cs[i]    = L.gcsin[i];
    }
}

} // namespace

cudaError_t adjoint_backward(Ctx &c, const RowSpace &rs, u32 n, const f64 *h_local,
                             const f64 *omega_local, const StepTape &tape, const AdjParams &p,
                             const CotState &cot, f64 *g_alpha, f64 *g_av, bool fp32) {
    cudaStream_t s = c.stream;
    cudaError_t e;
    const u32 N   = n + c.n_ghost;
    const u32 K   = tape.iters;
    const f64 hdt = p.dt / 2;
    const bool var = p.av_kind != 0;
    if ((e = c.adj_loc.ensure(sizeof(f64) * 24 * (size_t) n, s)) != cudaSuccess) return e;
    if ((e = c.adj_rank.ensure(sizeof(f64) * 12 * (size_t) N + 256, s)) != cudaSuccess) return e;
    f64 *B = c.adj_loc.as<f64>();
    size_t n_ = n, N_ = N;
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
    L.gal   = B + 21 * n_;
    L.gain  = B + 22 * n_;
    L.gcsin = B + 23 * n_;
    // rank-order staging: FP64 arrays (12 per rank) or FP32 records (88 bytes per rank)
    f64 *R = c.adj_rank.as<f64>();
    // varying viscosity: the previous accelerations and alpha by rank, the cotangents of the
    // velocity-gradient sums by local id (32 each) and by rank
    f64 *Mloc = nullptr, *A64 = nullptr, *VM64 = nullptr;
    float4 *A32 = nullptr, *VM32 = nullptr;
    if (var) {
        // FP32: the A records (N float4) padded to 32 bytes, so that the folded cotangents
        // start on the 32-byte boundary their 256-bit loads need
        const size_t a32 = (2 * N_ + 3) & ~(size_t) 3;
        const size_t need = 32 * n_ + (fp32 ? a32 + 12 * N_ : 4 * N_ + 32 * N_) + 64;
        if ((e = c.adj_vg.ensure(sizeof(f64) * need, s)) != cudaSuccess) return e;
        Mloc = c.adj_vg.as<f64>();
        f64 *rest = Mloc + 32 * n_;
        if (fp32) {
            A32  = (float4 *) rest;
            VM32 = (float4 *) (rest + a32);
        } else {
            A64  = rest;
            VM64 = rest + 4 * N_;
        }
    }
    Src64 s64{rs.x,      rs.y,       rs.z,       R,          R + N_,     R + 2 * N_,
              R + 3 * N_, R + 4 * N_, R + 5 * N_, R + 6 * N_, R + 7 * N_, R + 8 * N_,
              R + 9 * N_, R + 10 * N_, R + 11 * N_, var ? A64 + 3 * N_ : nullptr};
    float4 *P32 = (float4 *) R;
    float4 *V32 = P32 + 2 * N_;
    float4 *L32 = V32 + 2 * N_;
    float2 *M32 = (float2 *) (L32 + N_);
    Src32 s32{P32, V32, L32, M32};
    const u32 *si = c.sort_index.as<u32>(), *gs = c.ghost_src.as<u32>();
    const u32 vs = cot.vs;
    const u32 gb = div_up(n, 256), gN = div_up(N, 256);
    { k_adj_load<<<gb, 256, 0, s>>>(n, cot, vs, L); GBSPH_COUNTED; }
    const f64 *snap = tape.snap->as<f64>();
    const f64 *snap_av = var ? tape.snap_av->as<f64>() : nullptr;
    if (var) {
        // the output sound speed's cotangent, onto the last evaluation's energy / positions
        const f64 *sv = snap + (size_t) (K - 1) * 4 * n_;
        { k_adj_cs_out<<<gb, 256, 0, s>>>(n, cot.cs, sv + 3 * n_, p.xl, p.yl, p.zl, p, L); GBSPH_COUNTED; }
    }
    for (u32 k = K; k >= 1; k--) {
        { k_adj_lin<<<gb, 256, 0, s>>>(n, 0, hdt, L); GBSPH_COUNTED; }
        const f64 *sv = snap + (size_t) (k - 1) * 4 * n_;
        const f64 *sa = var ? snap_av + (size_t) (k - 1) * 4 * n_ : nullptr;
        if (p.ext_x) { k_adj_ext<<<gb, 256, 0, s>>>(n, p.ext_x, p.ext_y, p.ext_z, p.mGM, L); GBSPH_COUNTED; }
        ProfScope ps(c, kProfAdjDerivs, n);
        if (var) { k_adj_av_stage<<<gN, 256, 0, s>>>(N, n, si, gs, sa, A64, A32); GBSPH_COUNTED; }
        if (fp32) {
            { k_adj_stage32<<<gN, 256, 0, s>>>(N, n, si, gs, rs.x, rs.y, rs.z, sv, sv + n_,
                                             sv + 2 * n_, sv + 3 * n_, h_local, omega_local,
                                             L.lam[0], L.lam[1], L.lam[2], L.mu,
                                             var ? sa + 3 * n_ : nullptr, P32, V32, L32); GBSPH_COUNTED; }
            if (p.eos_kind == 1)
                { k_adj_derivs<Src32, true><<<div_up(n, 128), 128, 0, s>>>(rs, s32, p, L, g_alpha); GBSPH_COUNTED; }
            else
                { k_adj_derivs<Src32, false><<<div_up(n, 128), 128, 0, s>>>(rs, s32, p, L, g_alpha); GBSPH_COUNTED; }
        } else {
            { k_adj_gather<<<gN, 256, 0, s>>>(N, n, si, gs, sv, sv + n_, sv + 2 * n_, sv + 3 * n_,
                                            h_local, omega_local, L.lam[0], L.lam[1], L.lam[2],
                                            L.mu, R); GBSPH_COUNTED; }
            if (p.eos_kind == 1)
                { k_adj_derivs<Src64, true><<<div_up(n, 128), 128, 0, s>>>(rs, s64, p, L, g_alpha); GBSPH_COUNTED; }
            else
                { k_adj_derivs<Src64, false><<<div_up(n, 128), 128, 0, s>>>(rs, s64, p, L, g_alpha); GBSPH_COUNTED; }
        }
        if (var) {
            // the switch and the velocity gradients of this evaluation
            ProfScope pv(c, kProfVelGrad, n);
            if (fp32) {
                VG32 vg{P32, V32, A32, VM32};
                const float *taped = tape.vg_recorded
                                         ? tape.snap_vg->as<float>() + (size_t) (k - 1) * 24 * n_
                                         : nullptr;
                { k_adj_vg_a<VG32><<<div_up(n, 128), 128, 0, s>>>(rs, vg, p, L, h_local, omega_local, Mloc, g_av, taped); GBSPH_COUNTED; }
                { k_adj_vg_stage<<<gN, 256, 0, s>>>(N, n, si, gs, Mloc, nullptr, VM32); GBSPH_COUNTED; }
                { k_adj_vg_b<VG32><<<div_up(n, 128), 128, 0, s>>>(rs, vg, p, L); GBSPH_COUNTED; }
            } else {
                VG64 vg{rs.x, rs.y, rs.z, R, R + N_, R + 2 * N_, A64, A64 + N_, A64 + 2 * N_,
                        R + 4 * N_, VM64};
                { k_adj_vg_a<VG64><<<div_up(n, 128), 128, 0, s>>>(rs, vg, p, L, h_local, omega_local, Mloc, g_av, nullptr); GBSPH_COUNTED; }
                { k_adj_vg_stage<<<gN, 256, 0, s>>>(N, n, si, gs, Mloc, VM64, nullptr); GBSPH_COUNTED; }
                { k_adj_vg_b<VG64><<<div_up(n, 128), 128, 0, s>>>(rs, vg, p, L); GBSPH_COUNTED; }
            }
        }
        { k_adj_lin<<<gb, 256, 0, s>>>(n, 1, hdt, L); GBSPH_COUNTED; }
    }
    // Omega and the density constraint (positions, h and Omega are staged by the loop)
    ProfScope ps(c, kProfAdjDensity, n);
    if (fp32) {
        { k_adj_omega_a<Src32><<<gb, 256, 0, s>>>(rs, s32, h_local, omega_local, p.pmass, L); GBSPH_COUNTED; }
        { k_adj_stage32m<<<gN, 256, 0, s>>>(N, n, si, gs, L.nu, L.lom, M32); GBSPH_COUNTED; }
        { k_adj_omega_b<Src32><<<gb, 256, 0, s>>>(rs, s32, p.pmass, L); GBSPH_COUNTED; }
    } else {
        { k_adj_omega_a<Src64><<<gb, 256, 0, s>>>(rs, s64, h_local, omega_local, p.pmass, L); GBSPH_COUNTED; }
        { k_adj_gather2<<<gN, 256, 0, s>>>(N, n, si, gs, L.nu, L.lom, R + 10 * N_, R + 11 * N_); GBSPH_COUNTED; }
        { k_adj_omega_b<Src64><<<gb, 256, 0, s>>>(rs, s64, p.pmass, L); GBSPH_COUNTED; }
    }
    { k_adj_store<<<gb, 256, 0, s>>>(n, p.dt, L, cot, vs); GBSPH_COUNTED; }
    return cudaGetLastError();
}

} // namespace gbsph
