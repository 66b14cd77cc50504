// Argument bundles of the SPH pair kernels and the host wrappers that launch them.
#pragma once

#include "gbsph_ctx.cuh"

namespace gbsph {

// A set of CSR rows and the index space their entries live in.
//  - module form (reference layout): row t is local particle t, entries are merged
//    ids, positions are indexed by merged id; row_rank == row_local == nullptr.
//  - pipeline form: row t is the t-th local particle in Morton order,
//    row_rank[t] its rank, row_local[t] its local id; entries are ranks and
//    positions are the rank-ordered copies.  Rows come from the library's own cache:
//    each starts on a 4-entry boundary and its slot is padded to a multiple of 4, so
//    entries may be read four at a time.
struct RowSpace {
    u32 n;
    const u32 *row_rank;
    const u32 *row_local;
    const u32 *cnt;
    const u32 *off;
    const u32 *ent;
    const f64 *x, *y, *z;
};

// Hydro fields in the same index space as the CSR entries.  alpha (optional): the
// per-particle viscosity of the varying-AV form, else the constant alpha_AV.
struct HydroSpace {
    const f64 *h, *u, *vx, *vy, *vz, *omega, *P, *cs;
    const f64 *alpha;
    // optional per-particle factors of the FP64 pair loop, computed once by the staging
    // pass with the pair loop's own expressions (so the same bits): rho_h(m, h),
    // inv_sat_zero(rho^2 Omega) and rho Omega
    const f64 *rho, *inv_sub, *rho_om;
};

// Equation of state of the step: adiabatic (P = (gamma - 1) rho u) or locally
// isothermal LP07 (c_s^2 = cs0^2 (R^2 / r0^2)^(-q) at the position R, P = c_s^2 rho;
// shammodels/sph/src/modules/ComputeEos.cpp:725-798).
struct EosParams {
    u32 kind; // 0 adiabatic, 1 locally isothermal LP07
    f64 gamma, cs0, r0, q;
};

// Velocity-independent external acceleration (local ids, SoA), added to the hydro
// acceleration of every corrector evaluation; all null when there is none.
struct ExtAccel {
    const f64 *x, *y, *z;
};

// The caller's per-particle arrays (local ids).  Vector components are separate
// pointers sharing the element stride vs (1 for SoA, 3 or 4 for AoS f64_3).
struct LocalFields {
    f64 *x, *y, *z;
    f64 *vx, *vy, *vz;
    f64 *ax, *ay, *az;
    u32 vs;
    f64 *h, *u, *du;
};

// sph64.cu
// eps_p: per-particle Newton threshold (a particle is updated while its eps > eps_p;
// 1e-6 in the reference, IterateSmoothingLengthDensity.cpp)
cudaError_t h_iterate64(Ctx &c, const RowSpace &rs, const f64 *h_old, f64 *h_new, f64 *eps,
                        f64 pmass, f64 h_evol_max, f64 h_evol_iter_max, u32 iters,
                        f64 eps_p = 1e-6);
cudaError_t omega64(Ctx &c, const RowSpace &rs, const f64 *h_row, f64 pmass, f64 *out,
                    const u32 *out_index);
cudaError_t eos64(Ctx &c, u32 n, const f64 *h, const f64 *u, f64 pmass, f64 gamma, f64 *P, f64 *cs);
cudaError_t gather_eos64(Ctx &c, u32 N, u32 n_local, const LocalFields &lf, const f64 *omega_local,
                         f64 pmass, const EosParams &eos);
cudaError_t eos_lp07(Ctx &c, u32 n, const f64 *x, const f64 *y, const f64 *z, u32 vs, const f64 *h,
                     f64 pmass, f64 cs0, f64 r0, f64 q, f64 *P, f64 *cs);
cudaError_t derivs64(Ctx &c, const RowSpace &rs, const HydroSpace &hs, f64 pmass, f64 alpha_u,
                     f64 alpha_AV, f64 beta_AV, f64 *ax, f64 *ay, f64 *az, f64 *du, f64 *vsig);
cudaError_t derivs_step64(Ctx &c, const RowSpace &rs, const HydroSpace &hs, f64 pmass, f64 alpha_u,
                          f64 alpha_AV, f64 beta_AV, f64 hdt, f64 C_cour, f64 C_force,
                          const LocalFields &lf, const ExtAccel &ext);
// mGM != 0: the central point-mass acceleration (-M G) r / |r|^3 at the drifted
// positions, before the wrap, into ext_out (AddForceCentralGravPotential.cpp:37-48)
cudaError_t predict64(Ctx &c, const LocalFields &lf, u32 n, f64 dt, int periodic, const f64 *bmin,
                      const f64 *bmax, f64 mGM = 0, f64 *ext_x = nullptr, f64 *ext_y = nullptr,
                      f64 *ext_z = nullptr);
cudaError_t kdk_correct64(Ctx &c, const LocalFields &lf, u32 n, const f64 *aox, const f64 *aoy,
                          const f64 *aoz, u32 avs, const f64 *du_old, f64 dt);
cudaError_t cfl64(Ctx &c, u32 n, const f64 *h, const f64 *vsig, const f64 *ax, const f64 *ay,
                  const f64 *az, u32 avs, f64 C_cour, f64 C_force, f64 *dt_part);
// varying (Cullen & Dehnen 2010) viscosity, sph64.cu:
// div v, curl v, d(div v)/dt per pipeline row from rank-ordered fields (hs: h, v, omega;
// ax..az: the accelerations of the last evaluation), outputs by local id
cudaError_t velgrad64(Ctx &c, const RowSpace &rs, const HydroSpace &hs, const f64 *ax,
                      const f64 *ay, const f64 *az, f64 pmass, f64 *divv, f64 *cx, f64 *cy,
                      f64 *cz, u32 cvs, f64 *dtdivv);
// the switch update of n local particles (UpdateViscosity.cpp:170-215)
cudaError_t cd10_update(Ctx &c, u32 n, const f64 *divv, const f64 *cx, const f64 *cy,
                        const f64 *cz, u32 cvs, const f64 *dtdivv, const f64 *cs, const f64 *h,
                        const f64 *alpha, f64 dt, f64 sigma_decay, f64 alpha_min, f64 alpha_max,
                        f64 *alpha_new, bool fp32 = false);
// conservation totals {sum m v (3), sum m a (3), sum m (u + v.v/2), sum m (v.a + du)} of
// n local particles into out_dev[8] (scratch: 8 x 1024 doubles), deterministic order
cudaError_t conservation64(Ctx &c, const LocalFields &lf, u32 n, f64 pmass, f64 *out_dev,
                           f64 *scratch);
// the Morris & Monaghan (1997) switch update (UpdateViscosity.cpp:53-118)
cudaError_t mm97_update(Ctx &c, u32 n, const f64 *divv, const f64 *cs, const f64 *h,
                        const f64 *alpha, f64 dt, f64 sigma_decay, f64 alpha_min, f64 alpha_max,
                        f64 *alpha_new, bool fp32 = false);
// dst[r] = src[(merged id of rank r) -> local source] * stride, r < N (ghosts copy their source)
cudaError_t gather_merged64(Ctx &c, u32 N, u32 n_local, const f64 *src, u32 stride, f64 *dst);
// dst[row_local[t]] = src[row_rank[t]] for the n pipeline rows
cudaError_t rank_to_local64(Ctx &c, u32 n, const f64 *src_rank, f64 *dst);
cudaError_t scatter_rows(Ctx &c, u32 n, const f64 *src, f64 *dst);
cudaError_t gather_rows(Ctx &c, u32 n, const f64 *src_rank, f64 *dst, f64 *dst2);
cudaError_t fill64(Ctx &c, u32 n, f64 *dst, f64 v);

} // namespace gbsph
