// Mixed-precision (FP32 pair arithmetic) variants of the SPH pair kernels.
#pragma once

#include "sph_kernels.cuh"

namespace gbsph {

// Rank-ordered FP32 staging of merged fields for the mixed pair kernels, two 32-byte
// records per particle, each read with one 256-bit load:
//   position record P[2r], P[2r+1]:
//     {x_hi, y_hi, z_hi, 1/h}  {x_lo, y_lo, z_lo, c_s}
//   hydro record H[2r], H[2r+1]:
//     {vx_hi, vy_hi, vz_hi, u}  {P_hi, 1/(rho^2 Omega), bf16x2(vx_lo, vy_lo), bf16x2(vz_lo, P_lo)}
// A position is carried as an unevaluated sum hi + lo of two floats (hi = fl32(x),
// lo = fl32(x - hi)), so a pair separation (hi_a - hi_b) + (lo_a - lo_b) is accurate
// to FP32 rounding of the separation itself, wherever the particles sit in the box.
// Velocities and pressure keep their residuals as bfloat16 (about 2^-33 relative in
// total); rho = m (hfact/h)^3 and 1/(rho Omega) are rebuilt from 1/h in the kernel.
struct MixedSpace {
    const float4 *P; // 2 per particle
    const float4 *H; // 2 per particle
};

cudaError_t stage_positions_mixed(Ctx &c, u32 N, f64 h_tol);
// the position records staged by stage_positions_mixed (B.w = fl32 cache threshold)
const float4 *mixed_positions(Ctx &c);
cudaError_t h_iterate_mixed(Ctx &c, const RowSpace &rs, const f64 *h_old, f64 *h_new, f64 *eps,
                            f64 pmass, f64 h_evol_max, f64 h_evol_iter_max, u32 iters,
                            f64 eps_p = 1e-6);
// the pipeline's Omega: restages the records' 1/h from the converged h (local ids), then
// Omega per row and, in the same pass, each cache row compacted in place to the pairs
// inside either support (the entries the corrector kernels visit); the cache is no
// longer exportable afterwards (cache_valid = false)
cudaError_t omega_compact_mixed(Ctx &c, const RowSpace &rs, u32 N, u32 n_local, const f64 *h_local,
                                const f64 *h_row, f64 *omega_local);
// the corrector's EOS + record staging for merged ranks 0..N-1 (replaces gather_eos64
// + the FP64 rank-ordered copies in the mixed path; only h is kept in FP64, in c.sh2),
// then the fused derivatives step, which reads the records, c.sh2 and the caller's
// local fields
// varying_av: also stage FP32 acceleration records and the plain c_s per rank
// compensated: also the compensated tier's records (c.f_comp, 2 float4 per rank:
// {X_hi, X_lo, (1/h)_lo, P_lo} {u_lo, (1/h^4)_hi, (1/h^4)_lo, 0} with
// X = P / (rho^2 Omega)), and the LP07 power in FP64
cudaError_t gather_stage_mixed(Ctx &c, u32 N, u32 n_local, const LocalFields &lf,
                               const f64 *omega_local, f64 pmass, const EosParams &eos,
                               bool varying_av = false, bool compensated = false);
// varying_av: per-particle alpha folded into the records' c_s lane (stage_alpha_mixed)
// cond: also accumulate the condition sums of the error estimate (Scalars::cond_*)
cudaError_t derivs_step_mixed(Ctx &c, const RowSpace &rs, f64 pmass, f64 alpha_u, f64 alpha_AV,
                              f64 beta_AV, f64 hdt, f64 C_cour, f64 C_force,
                              const LocalFields &lf, const ExtAccel &ext, bool varying_av = false,
                              bool cond = false);
// varying viscosity: div v, curl v, d(div v)/dt per row (outputs by local id), after
// gather_stage_mixed(..., true); alpha of the local particles into the records; the
// staged plain c_s back to local order
// sums (optional, 24 floats per row by local id): the row's bare R, Dv and Da, recorded
// for the adjoint's reverse pass
cudaError_t velgrad_mixed(Ctx &c, const RowSpace &rs, const f64 *omega_local, f64 pmass,
                          f64 *divv, f64 *cx, f64 *cy, f64 *cz, u32 cvs, f64 *dtdivv,
                          float *sums = nullptr);
cudaError_t stage_alpha_mixed(Ctx &c, u32 N, u32 n_local, const f64 *alpha_local);
cudaError_t cs_to_local_mixed(Ctx &c, u32 n, f64 *dst);
// sph_comp.cu, the compensated tier: one double-float Newton step of h per row (rows
// whose iteration did not converge keep their h) and Omega at the result (by local id),
// from the position records of stage_positions_mixed
cudaError_t dens_polish_df(Ctx &c, const RowSpace &rs, const f64 *h_old, f64 *h_row, const f64 *eps,
                           f64 h_evol_max, f64 h_evol_iter_max, f64 *omega_local);
// compensated derivatives step (after gather_stage_mixed(..., compensated = true))
cudaError_t derivs_step_comp(Ctx &c, const RowSpace &rs, f64 pmass, f64 alpha_u, f64 alpha_AV,
                             f64 beta_AV, f64 hdt, f64 C_cour, f64 C_force, const LocalFields &lf,
                             const ExtAccel &ext, bool varying_av = false, bool cond = false);
cudaError_t derivs_mixed_module(Ctx &c, const RowSpace &rs, const HydroSpace &hs, f64 pmass,
                                f64 alpha_u, f64 alpha_AV, f64 beta_AV, f64 *ax, f64 *ay, f64 *az,
                                f64 *du, f64 *vsig);

} // namespace gbsph
