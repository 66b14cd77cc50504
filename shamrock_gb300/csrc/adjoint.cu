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
    struct Row {
        f64 x, y, z, vx, vy, vz, u, h, om, lx, ly, lz, mu;
    };
    struct Nb {
        f64 dx, dy, dz, dvx, dvy, dvz, u, h, om, lx, ly, lz, mu, rsq;
    };
    __device__ Row row(u32 c) const {
        return Row{x[c], y[c], z[c], vx[c], vy[c], vz[c], u[c], h[c], om[c], lx[c], ly[c], lz[c], mu[c]};
    }
    __device__ Nb nb(u32 b, const Row &r) const {
        const f64 xb = x[b], yb = y[b], zb = z[b];
        return Nb{r.x - xb, r.y - yb, r.z - zb, r.vx - vx[b], r.vy - vy[b], r.vz - vz[b],
                  u[b],     h[b],     om[b],    lx[b],        ly[b],        lz[b],
                  mu[b],    xb * xb + yb * yb + zb * zb};
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
//   V[2r..2r+1] = {v_hi, u | v_lo, mu},   Lr[r] = {lambda, 0},   M[r] = {nu, lom}
struct Src32 {
    using T = float;
    const float4 *P, *V, *Lr;
    const float2 *M;
    struct Row {
        F8 p, v;
        float4 l;
    };
    struct Nb {
        float dx, dy, dz, dvx, dvy, dvz, u, h, om, lx, ly, lz, mu, rsq;
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
                  v.a.w, p.a.w, p.b.w, l.x, l.y, l.z, v.b.w, xb * xb + yb * yb + zb * zb};
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
                              float4 *__restrict__ P, float4 *__restrict__ V,
                              float4 *__restrict__ Lr) {
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
    Lr[r]     = make_float4(hi32(lx[src]), hi32(ly[src]), hi32(lz[src]), 0.f);
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
            const T vsc = aAV * csc + bAV * aw, vsb = aAV * csb + bAV * aw;
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
            if (actc) scs += dLAc * (-half * rhoc * aAV * w);
            srho += (actc ? dLAc * pdiv(tc, rhoc) : T(0)) + dLvsu * dvsur;
            sk += -m * Le * Ac * Fc + m * w * muc * Ac * Fc;
            sj += cond * Fc;
            su += half * m * au * dmu * vsu * J;
            shF += (-m * Le * Ac * kc + m * w * muc * Ac * kc + cond * jc) * Fhc;
            // alpha_AV: this row's own pair term only (lambda_c . f_cb + mu_c g_cb)
            const T dqca = actc ? -half * rhoc * csc * w : T(0);
            const T dqba = actb ? -half * rhob * csb * w : T(0);
            const T lce  = lxc * ex + lyc * ey + lzc * ez;
            ga += -m * lce * (kc * Fc * dqca + kb * Fb * dqba) + muc * m * w * kc * Fc * dqca;
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
        galpha = ga;
    }
    galpha = block_reduce(galpha, OpAddF64{}, 0.0);
    if (threadIdx.x == 0) atomicAdd(g_alpha, galpha);
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
                             const CotState &cot, f64 *g_alpha, bool fp32) {
    cudaStream_t s = c.stream;
    cudaError_t e;
    const u32 N   = n + c.n_ghost;
    const u32 K   = tape.iters;
    const f64 hdt = p.dt / 2;
    if ((e = c.adj_loc.ensure(sizeof(f64) * 21 * (size_t) n, s)) != cudaSuccess) return e;
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
    // rank-order staging: FP64 arrays (12 per rank) or FP32 records (88 bytes per rank)
    f64 *R = c.adj_rank.as<f64>();
    Src64 s64{rs.x,      rs.y,       rs.z,       R,          R + N_,     R + 2 * N_,
              R + 3 * N_, R + 4 * N_, R + 5 * N_, R + 6 * N_, R + 7 * N_, R + 8 * N_,
              R + 9 * N_, R + 10 * N_, R + 11 * N_};
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
    for (u32 k = K; k >= 1; k--) {
        { k_adj_lin<<<gb, 256, 0, s>>>(n, 0, hdt, L); GBSPH_COUNTED; }
        const f64 *sv = snap + (size_t) (k - 1) * 4 * n_;
        if (p.ext_x) { k_adj_ext<<<gb, 256, 0, s>>>(n, p.ext_x, p.ext_y, p.ext_z, p.mGM, L); GBSPH_COUNTED; }
        ProfScope ps(c, kProfAdjDerivs, n);
        if (fp32) {
            { k_adj_stage32<<<gN, 256, 0, s>>>(N, n, si, gs, rs.x, rs.y, rs.z, sv, sv + n_,
                                             sv + 2 * n_, sv + 3 * n_, h_local, omega_local,
                                             L.lam[0], L.lam[1], L.lam[2], L.mu, P32, V32, L32); GBSPH_COUNTED; }
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
