// Reverse-mode (adjoint) of one SPH step: declarations shared by adjoint.cu and the
// step driver.
#pragma once

#include "sph_kernels.cuh"

namespace gbsph {

// Recorded by a forward step run for the adjoint: velocity and internal energy (SoA,
// n each) before each corrector evaluation of the derivatives.
struct StepTape {
    u32 forced_iters = 0;   // run exactly this many corrector evaluations
    u32 iters        = 0;   // evaluations recorded
    DevBuf *snap     = nullptr;
    // varying viscosity: before each evaluation the accelerations of the last one (the
    // velocity gradients' input, 3 n) and the evaluation's switched alpha (n), local ids
    DevBuf *snap_av  = nullptr;
    // mixed-precision varying viscosity: the velocity gradients' bare sums of each
    // evaluation (R, Dv, Da: 24 floats per particle), so the reverse need not redo them
    DevBuf *snap_vg  = nullptr;
    bool vg_recorded = false; // the forward recorded them (mixed tiers)
};
constexpr u32 kTapeMaxIters = 16;

struct AdjParams {
    f64 pmass, gamma, alpha_u, alpha_AV, beta_AV, dt;
    // equation of state: 0 adiabatic, 1 locally isothermal LP07 (c_s^2 = cs0^2 (R^2/r0^2)^-q)
    u32 eos_kind;
    f64 cs0, r0, q;
    // central point mass (mGM = -G M; ext_x null when absent) and the local positions
    // after the step it was evaluated at
    f64 mGM;
    const f64 *ext_x, *ext_y, *ext_z;
    // viscosity: 0 constant alpha_AV, 1 Cullen & Dehnen (2010), 2 Morris & Monaghan (1997)
    // switch with its parameters; alpha_in and cs_in are the state the step started from
    // (per-particle alpha_AV and stored sound speed, local ids)
    u32 av_kind;
    f64 alpha_min, alpha_max, sigma_decay;
    const f64 *alpha_in, *cs_in;
    // local positions after the step (the LP07 sound speed's position dependence)
    const f64 *xl, *yl, *zl;
};

// Cotangents of one particle state (SoA), updated in place by adjoint_backward: on
// entry with respect to the state after the step, on return with respect to the state
// before it.
struct CotState {
    f64 *x[3], *v[3], *a[3];
    f64 *u, *du;
    u32 vs; // element stride of the vectors
    // varying viscosity: per-particle alpha_AV and stored sound speed (null otherwise)
    f64 *alpha, *cs;
};

// Runs the reverse pass of the step just recomputed in c (tree, cache, ghosts, the
// converged h and Omega in h_local / omega_local, and the tape).  g_alpha accumulates
// dL/d alpha_AV on the device (constant viscosity), g_av dL/d (alpha_min, alpha_max,
// sigma_decay) (varying viscosity).  fp32: FP32 pair arithmetic (else FP64).
cudaError_t adjoint_backward(Ctx &c, const RowSpace &rs, u32 n, const f64 *h_local,
                             const f64 *omega_local, const StepTape &tape, const AdjParams &p,
                             const CotState &cot, f64 *g_alpha, f64 *g_av, bool fp32);

} // namespace gbsph
