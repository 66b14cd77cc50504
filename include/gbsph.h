/*
 * gbsph.h — C ABI of the GB300-native SPH timestep hot path.
 *
 * A drop-in for the single-GPU path of Shamrock's shammodels::sph solver:
 * Morton keys -> bitonic sort -> leaf reduction -> Karras tree / LBVH, the
 * two-stage neighbour cache, the h-rho Newton iteration, Omega, the adiabatic
 * EOS, constant-AV derivatives, v_sig / CFL and the leapfrog KDK step.
 *
 * Conventions
 *  - Every entry point returns GBSPH_OK (0) or a GBSPH_ERR_* code; the message
 *    of the last failure is gbsph_last_error(ctx).  No exception crosses the ABI.
 *  - Array arguments are DEVICE pointers unless the parameter name ends in _host.
 *    Scalars and small fixed arrays (box corners) are host values.
 *  - `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).
 *  - Positions/velocities/accelerations of the caller are three component
 *    pointers sharing an element stride in doubles (gbsph_vec3): stride 1 for
 *    structure-of-arrays, 4 for the reference's padded f64_3 with x = base,
 *    y = base + 1, z = base + 2.
 *  - Index spaces: "local" = the caller's particles [0, n_local); "merged" =
 *    locals followed by periodic ghosts, as the reference's merged_xyzh.
 *  - A context owns its scratch arena (tree, caches, ghost tables) and is used by
 *    one host thread and one stream at a time.
 *
 * Citations are paths inside the Shamrock source tree.
 */
#ifndef GBSPH_H
#define GBSPH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBSPH_OK 0
#define GBSPH_ERR_ARG 1           /* bad argument (maps to std::invalid_argument) */
#define GBSPH_ERR_CUDA 2          /* CUDA runtime error */
#define GBSPH_ERR_CAPACITY 3      /* caller buffer too small / 32-bit CSR overflow */
#define GBSPH_ERR_NOT_CONVERGED 4 /* h iteration or corrector did not converge */
#define GBSPH_ERR_STATE 5         /* call order violated (e.g. cache before tree) */

#define GBSPH_FP64 0  /* every pair sum in FP64, bit-identical to the FP64 oracle */
#define GBSPH_MIXED 1 /* FP32 pair arithmetic, FP64 positions/drift/h test/totals */
/* FP32 pair arithmetic with the sums that cancel in double-float (two floats per value,
 * error-free transformations on the FP32 pipes): h finished by one double-float Newton
 * step, Omega, and the background-pressure part of the force.  For use where GBSPH_MIXED
 * loses accuracy to cancellation (a large uniform pressure, e.g. a sound wave: 1e-6 of
 * the FP64 path where GBSPH_MIXED errs by 4e-3). */
#define GBSPH_MIXED_COMPENSATED 2
/* Error-controlled mixed precision (gbsph_evolve_once): each step estimates the error of
 * the FP32 tier from condition sums the derivatives pass accumulates (the summed pair
 * force and du/dt magnitudes against the largest result); a step whose estimate exceeds
 * gbsph_config.mixed_tol is recomputed from its start state in the compensated tier, and
 * later steps stay there until the estimate falls below a quarter of the tolerance.  The
 * estimate is refreshed on every fourth step where it cannot reach the tolerance in the
 * steps between (below an eighth of it, or below 0.8 of it and growing slowly enough),
 * else on every step.  gbsph_step_log reports the tier, reruns and estimates. */
#define GBSPH_MIXED_GUARDED 3

typedef struct gbsph_ctx gbsph_ctx;

typedef struct {
    double *x, *y, *z;
    uint32_t stride; /* element stride in doubles */
    uint32_t pad;
} gbsph_vec3;

/* The caller-owned particle fields of one patch (PatchDataLayer fields
 * xyz, vxyz, axyz, hpart, uint, duint of the reference's SPH layout). */
typedef struct {
    uint32_t n;
    uint32_t pad;
    gbsph_vec3 xyz, vxyz, axyz;
    double *hpart, *uint, *duint;
    double *omega; /* optional output, may be NULL */
    /* Varying viscosity (av_kind GBSPH_AV_VARYING_CD10) only, NULL otherwise.  State
     * carried between steps, read and updated in place: alpha_AV and soundspeed (the
     * sound speed of the last EOS evaluation, the reference's "soundspeed" field;
     * zero-initialised like the reference's fields).  Optional outputs of the last
     * corrector evaluation: divv, curlv, dtdivv (the reference's fields of those names). */
    double *alpha_AV, *soundspeed;
    double *divv;
    gbsph_vec3 curlv;
    double *dtdivv;
} gbsph_particles;

/* Solver configuration (the hot-path subset of shammodels::sph::SolverConfig,
 * shammodels/sph/include/shammodels/sph/SolverConfig.hpp). */
typedef struct {
    double gamma;                   /* adiabatic EOS */
    double pmass;                   /* gpart_mass */
    double alpha_u, alpha_AV, beta_AV; /* constant AV (config/AVConfig.hpp:52-54) */
    double cfl_cour, cfl_force, cfl_mult_stiffness;
    double htol_up_coarse, htol_up_fine; /* 1.1, 1.1 */
    double epsilon_h;               /* 1e-6 */
    uint32_t h_iter_per_subcycles;  /* 50 */
    uint32_t h_max_subcycles;       /* 100 */
    uint32_t tree_reduction_level;  /* 3 */
    uint32_t periodic;              /* 1 periodic box, 0 free boundaries */
    double box_min[3], box_max[3];
    uint32_t precision;             /* GBSPH_FP64, GBSPH_MIXED, _COMPENSATED or _GUARDED */
    uint32_t pad;
    /* Per-particle Newton threshold: a particle's h is updated while its eps_h exceeds
     * it (1e-6 in the reference's IterateSmoothingLengthDensity kernel; 0 selects
     * that).  Smaller values converge h further, e.g. for finite-difference checks of
     * the adjoint, which differentiates h as the exact root of the density constraint. */
    double epsilon_h_particle;
    /* Equation of state: GBSPH_EOS_ADIABATIC (gamma) or GBSPH_EOS_LOCALLY_ISOTHERMAL_LP07,
     * c_s^2 = cs0^2 (R^2 / r0^2)^(-q) at the particle's position R, P = c_s^2 rho
     * (SolverConfig EOSConfig::LocallyIsothermalLP07, ComputeEos.cpp:725-798). */
    uint32_t eos_kind;
    /* External force: GBSPH_EXT_NONE or GBSPH_EXT_POINT_MASS, a central mass at the origin,
     * a = -G M r / |r|^3, evaluated after the drift and added to the hydro acceleration
     * (ExtForceConfig::PointMass, AddForceCentralGravPotential.cpp:37-48), without
     * accretion. */
    uint32_t ext_kind;
    double cs0, eos_r0, eos_q;
    double central_mass, constant_G;
    /* Artificial viscosity: GBSPH_AV_CONSTANT (alpha_AV), GBSPH_AV_VARYING_CD10,
     * Cullen & Dehnen (2010): per-particle alpha relaxed towards a shock indicator built
     * from div v, curl v and d(div v)/dt, in [alpha_min, alpha_max] with decay rate
     * sigma_decay (AVConfig::VaryingCD10, UpdateViscosity.cpp:122-215), or
     * GBSPH_AV_VARYING_MM97, Morris & Monaghan (1997): alpha driven by max(-div v, 0) and
     * decaying to alpha_min (AVConfig::VaryingMM97, UpdateViscosity.cpp:53-118); alpha_u
     * and beta_AV as for the constant form.  Both varying forms use the particle fields
     * alpha_AV and soundspeed. */
    uint32_t av_kind;
    uint32_t pad2;
    double alpha_min, alpha_max, sigma_decay;
    /* GBSPH_MIXED_GUARDED: the largest estimated error of a step's accelerations and du/dt
     * (relative to the largest magnitude of each field) the FP32 tier may leave; 0 selects
     * 1e-5. */
    double mixed_tol;
    /* Corrector evaluations after which a step that still fails the eps_v test gives up
     * with GBSPH_ERR_NOT_CONVERGED (the reference stops at 50, Solver.cpp:2252-2256);
     * 0 selects 50. */
    uint32_t corrector_max_iters;
    uint32_t pad3;
} gbsph_config;

#define GBSPH_EOS_ADIABATIC 0
#define GBSPH_EOS_LOCALLY_ISOTHERMAL_LP07 1
#define GBSPH_EXT_NONE 0
#define GBSPH_EXT_POINT_MASS 1
#define GBSPH_AV_CONSTANT 0
#define GBSPH_AV_VARYING_CD10 1
#define GBSPH_AV_VARYING_MM97 2

/* Synchronised solver state (the scheduler edges "time", "dt", "cfl_multiplier",
 * shammodels/sph/include/shammodels/sph/Solver.hpp:99-145). */
typedef struct {
    double t, dt, cfl_mult;
} gbsph_time_state;

typedef struct {
    double t, dt, next_dt, cfl_mult;
    uint32_t n_local, n_ghost, leaf_count, h_subcycles, h_iterations, corrector_iters;
    uint64_t cache_size;
    double eps_v, max_eps_h;
    double elapsed_s; /* wall time of the step (host clock, after the final sync) */
    double rate;      /* n_local / elapsed_s, as Solver.cpp:3200 */
    /* mixed precision: the tier that produced the step (GBSPH_FP64, GBSPH_MIXED or
     * GBSPH_MIXED_COMPENSATED), whether a GBSPH_MIXED_GUARDED step was recomputed in the
     * compensated tier (1) or not (0), and the estimated error of the FP32 tier's
     * accelerations and du/dt on the last corrector evaluation (relative to the largest
     * magnitude of each field; 0 in FP64) */
    uint32_t tier, tier_reruns;
    double err_est_a, err_est_du;
    /* neighbour-cache entries the corrector evaluations visit: the pairs inside either
     * particle's support, which the FP32 tier compacts the rows to (cache_size otherwise) */
    uint64_t cache_kept;
    /* GBSPH_MIXED_GUARDED: 1 when this step refreshed the error estimate (its first
     * corrector evaluation accumulated the condition sums), 0 when it reports the last
     * refreshed one; 1 in the other precisions */
    uint32_t est_refreshed, pad4;
} gbsph_step_log;

/* ------------------------------------------------------------------ lifetime */
int gbsph_create(gbsph_ctx **out, int device);
void gbsph_destroy(gbsph_ctx *ctx);
const char *gbsph_last_error(const gbsph_ctx *ctx);
const char *gbsph_version(void);

/* ------------------------------------------------------------------ tree (shamtree) */

/* Morton codes of n positions (SoA) clamped to [bmin, bmax], padded to
 * morton_count with the all-ones code.  key_bits 32 (the SPH path) or 64.
 * Replaces shamtree::morton_code_set_from_positions, shamtree/src/MortonCodeSet.cpp:63-118. */
int gbsph_morton_codes(gbsph_ctx *ctx, const double *x, const double *y, const double *z,
                       uint32_t n, uint32_t morton_count, const double bmin_host[3],
                       const double bmax_host[3], int key_bits, void *keys_out, void *stream);

/* In-place key/value bitonic sort, len a power of two; identical network (and so
 * identical order of equal keys) to shamalgs::algorithm::sort_by_key,
 * shamalgs/src/primitives/sort_by_keys.cpp:36-43 ->
 * shamalgs/src/details/algorithm/bitonicSort_updated_usm.cpp:285-396. */
int gbsph_sort_by_key(gbsph_ctx *ctx, void *keys, uint32_t *vals, uint32_t len, int key_bits,
                      void *stream);

/* Full compressed-leaf BVH over n positions (SoA): Morton set over morton_count
 * slots (0 = next power of two), sort, reduction (level), Karras topology, node
 * AABBs and, when h != NULL, the interaction radius field max(h) * htol.
 * Replaces CompressedLeafBVH::rebuild_from_positions, shamtree/src/CompressedLeafBVH.cpp:79-95,
 * plus Solver::compute_presteps_rint, shammodels/sph/src/Solver.cpp:1322-1356. */
int gbsph_build_tree(gbsph_ctx *ctx, const double *x, const double *y, const double *z,
                     const double *h, uint32_t n, const double bmin_host[3],
                     const double bmax_host[3], uint32_t reduction_level, double htol,
                     int key_bits, uint32_t morton_count, void *stream);

int gbsph_tree_counts(gbsph_ctx *ctx, uint32_t *morton_count_host, uint32_t *leaf_count_host);

/* Copy the last tree out (each pointer may be NULL).  Node arrays follow the
 * reference numbering: internal cells [0, L-1), leaves at offset L-1.  aabb_* are
 * (2L-1) x 3 doubles, keys are u32 or u64 per the build's key_bits. */
int gbsph_tree_export(gbsph_ctx *ctx, void *sorted_keys, uint32_t *sort_index, uint32_t *reduc,
                      void *reduced_keys, uint32_t *lchild, uint32_t *rchild, uint8_t *lflag,
                      uint8_t *rflag, uint32_t *endrange, double *aabb_min, double *aabb_max,
                      double *rint, void *stream);

/* Object query over the last tree, in DFS order (CLBVHObjectIterator::rtree_for,
 * shamtree/include/shamtree/CLBVHObjectIterator.hpp:127-169).  mode 0: every
 * object; mode 1: objects inside [q - s, q + s], visiting nodes whose AABB
 * intersects that box.  Writes per-query counts; when out != NULL and capacity is
 * large enough also the object ids.  *total_host receives the entry count. */
int gbsph_tree_query(gbsph_ctx *ctx, const double *qx, const double *qy, const double *qz,
                     uint32_t nq, int mode, double s, uint32_t *counts, uint32_t *out,
                     uint64_t capacity, uint64_t *total_host, void *stream);

/* ------------------------------------------------------------------ neighbour cache */

/* Two-stage neighbour cache of the first n_local particles against the n_merged
 * positions of the last gbsph_build_tree call (built with h).  Pair test
 * !(r^2 > (h_a htol)^2 R^2 && r^2 > (h_b htol)^2 R^2), R = 2.
 * Replaces NeighbourCache::start_neighbors_cache_2stages,
 * shammodels/sph/src/modules/NeighbourCache.cpp:223-596.  With GBSPH_MIXED the pair
 * test is first estimated in FP32 and only pairs within 1e-5 of the threshold are
 * decided in FP64: the cache is identical, the work mostly FP32. */
int gbsph_neighbour_cache(gbsph_ctx *ctx, uint32_t n_local, double htol, uint32_t precision,
                          void *stream);

/* total_host: stage-2 entries of the last cache.  leaf_total_host: stage-1 rank ranges
 * when the last build ran the two-pass stage 1 (slots past the budget), else 0. */
int gbsph_cache_size(gbsph_ctx *ctx, uint64_t *total_host, uint64_t *leaf_total_host);

/* The cache in the reference's ObjectCache layout (TreeTraversal.hpp:375-485):
 * per local id a count and exclusive offset, entries are merged ids. */
int gbsph_cache_export(gbsph_ctx *ctx, uint32_t *cnt, uint32_t *scanned, uint32_t *entries,
                       void *stream);

/* ------------------------------------------------------------------ SPH modules
 * CSR arguments (cnt, scanned, entries) are in the reference ObjectCache layout.
 * Positions and fields are merged-id SoA arrays; outputs are per local id. */

/* `iters` Newton iterations of IterateSmoothingLengthDensity
 * (shammodels/sph/src/modules/IterateSmoothingLengthDensity.cpp:28-120); iters = 1
 * is exactly one module evaluation.  max/min eps and the largest iteration count
 * any particle used are returned through the *_host pointers (may be NULL). */
int gbsph_h_iterate(gbsph_ctx *ctx, const uint32_t *cnt, const uint32_t *scanned,
                    const uint32_t *entries, const double *x, const double *y, const double *z,
                    const double *h_old, double *h_new, double *eps, uint32_t n_local,
                    double pmass, double h_evol_max, double h_evol_iter_max, uint32_t iters,
                    double *max_eps_host, double *min_eps_host, uint32_t *iters_used_host,
                    void *stream);

/* NodeComputeOmega, shammodels/sph/src/modules/ComputeOmega.cpp:25-74. */
int gbsph_omega(gbsph_ctx *ctx, const uint32_t *cnt, const uint32_t *scanned,
                const uint32_t *entries, const double *x, const double *y, const double *z,
                const double *h, uint32_t n_local, double pmass, double *omega, void *stream);

/* Locally isothermal EOS, LP07 (ComputeEos.cpp:725-798, shamphys/eos.hpp:87-98):
 * c_s^2 = cs0^2 (R^2 / r0^2)^(-q) at the position R, P = c_s^2 rho_h(m, h). */
int gbsph_eos_locally_isothermal(gbsph_ctx *ctx, gbsph_vec3 xyz, const double *h, uint32_t n,
                                 double pmass, double cs0, double r0, double q, double *P,
                                 double *cs, void *stream);

/* ComputeEOSAdiabatic from h, shammodels/sph/src/modules/ComputeEos.cpp:153-245. */
int gbsph_eos_adiabatic(gbsph_ctx *ctx, const double *h, const double *u, uint32_t n, double pmass,
                        double gamma, double *P, double *cs, void *stream);

/* UpdateDerivs::update_derivs_constantAV, shammodels/sph/src/modules/UpdateDerivs.cpp:88-288;
 * with vsig != NULL also the v_sig maximum of Solver.cpp:2716-2788.
 * precision GBSPH_FP64 or GBSPH_MIXED. */
int gbsph_derivs_constAV(gbsph_ctx *ctx, const uint32_t *cnt, const uint32_t *scanned,
                         const uint32_t *entries, const double *x, const double *y,
                         const double *z, const double *vx, const double *vy, const double *vz,
                         const double *h, const double *omega, const double *u, const double *P,
                         const double *cs, uint32_t n_local, uint32_t n_merged, double pmass,
                         double alpha_u, double alpha_AV, double beta_AV, uint32_t precision,
                         double *ax, double *ay, double *az, double *du, double *vsig,
                         void *stream);

/* Allocation-free variant of gbsph_derivs_constAV(..., GBSPH_MIXED, ...) for callers
 * that may not allocate device memory (a framework whose pool owns all device memory,
 * a loop that must not allocate once running) and so cannot hold a gbsph_ctx.  It has
 * no counterpart in the reference.  Needs no context: it runs on the current device
 * and takes the same inputs, outputs and results as the context entry point.
 *  - The FP32 staging lives in a fixed device array inside the library, sized for at
 *    most 65,536 merged particles (4 MiB, reserved on every GPU that loads the library
 *    until the process exits); larger n_merged returns GBSPH_ERR_CAPACITY.
 *  - Every call looks the array's device address up in the current context (a cached
 *    address would be wrong after cudaDeviceReset or under another context on the same
 *    device).  The first call in a context also loads the library's device code: make
 *    that first call before any stream capture.
 *  - All calls share the one array: calls that overlap on the GPU (other streams, other
 *    threads) race; serialise them.  Nothing needs clearing between calls.
 *  - Asynchronous on `stream`; returns GBSPH_OK, GBSPH_ERR_CAPACITY, GBSPH_ERR_ARG or
 *    GBSPH_ERR_CUDA (there is no context to hold a message). */
int gbsph_derivs_constAV_mixed_noalloc(const uint32_t *cnt, const uint32_t *scanned,
                                       const uint32_t *entries, const double *x, const double *y,
                                       const double *z, const double *vx, const double *vy,
                                       const double *vz, const double *h, const double *omega,
                                       const double *u, const double *P, const double *cs,
                                       uint32_t n_local, uint32_t n_merged, double pmass,
                                       double alpha_u, double alpha_AV, double beta_AV,
                                       double *ax, double *ay, double *az, double *du,
                                       double *vsig, void *stream);

/* Periodic ghost layer of one patch covering [bmin, bmax]
 * (BasicSPHGhostHandler::find_interfaces + gen_id_table_interfaces +
 * build_comm_merge_positions, shammodels/sph/src/BasicSPHGhosts.cpp:260-360,512-530).
 * Returns the ghost count; gbsph_ghost_export then gives, per ghost, the source
 * local id, the offset index (0..25, x-outer/z-inner order without the zero
 * offset) and the merged positions/h (n_local + n_ghost entries). */
int gbsph_periodic_ghosts(gbsph_ctx *ctx, gbsph_vec3 xyz, const double *h, uint32_t n_local,
                          const double bmin_host[3], const double bmax_host[3], double htol,
                          uint32_t *n_ghost_host, void *stream);
int gbsph_ghost_export(gbsph_ctx *ctx, uint32_t *src, uint8_t *offset_id, double *mx, double *my,
                       double *mz, double *mh, void *stream);

/* Leapfrog predictor of Solver::evolve_once (Solver.cpp:390-524 with
 * shamrock/src/math/integrators.cpp:27-86): v += dt/2 a, u += dt/2 du, x += dt v, then
 * the second half kick; with periodic != 0 the positions are wrapped into the box
 * (integrators.cpp:207-237).  In place on p's xyz, vxyz, uint (reads axyz, duint). */
int gbsph_kdk_predict(gbsph_ctx *ctx, const gbsph_particles *p, double dt, uint32_t periodic,
                      const double bmin_host[3], const double bmax_host[3], void *stream);

/* Leapfrog corrector (integrators.cpp:88-120, Solver.cpp:2506-2616): with p's axyz / duint
 * holding the new derivatives, v += dt/2 (a_new - a_old), u += dt/2 (du_new - du_old);
 * *eps_v_host = max |dv| / sqrt(sum v^2 / n), the corrector's rerun test (0 when the
 * mean vanishes). */
int gbsph_kdk_correct(gbsph_ctx *ctx, const gbsph_particles *p, gbsph_vec3 a_old,
                      const double *du_old, double dt, double *eps_v_host, void *stream);

/* CFL time step (ComputeCFLCourant.hpp:45-60, ComputeCFLForce.hpp:50-62) per particle,
 * dt_a = min(C_cour h / v_sig, C_force sqrt(h / |a|)), into dt_part (optional), and its
 * minimum over the particles (Solver.cpp:3046-3119) into *dt_min_host. */
int gbsph_cfl(gbsph_ctx *ctx, const double *h, const double *vsig, gbsph_vec3 a, uint32_t n,
              double C_cour, double C_force, double *dt_part, double *dt_min_host, void *stream);

/* Conservation totals of ConservativeCheck::check_conservation
 * (shammodels/sph/src/modules/ConservativeCheck.cpp:56-180), in FP64 with a fixed
 * summation order: out_host = {sum m v (3), sum m a (3), sum m (u + v.v / 2),
 * sum m (v.a + du)}, with a the caller's total acceleration (hydro + external). */
int gbsph_conservation(gbsph_ctx *ctx, const gbsph_particles *p, double pmass, double out_host[8],
                       void *stream);

/* ------------------------------------------------------------------ full step */

/* One Solver::evolve_once on one patch (shammodels/sph/src/Solver.cpp:1942-3272):
 * leapfrog predictor + periodic wrap, sph_prestep (ghosts, tree, neighbour cache,
 * h iteration with restarts, Omega), corrector loop (ghost fields, EOS,
 * derivatives, corrector, eps_v rerun test), v_sig/CFL, time/dt/multiplier update.
 * Particle fields are updated in place; ts is read and updated. */
int gbsph_evolve_once(gbsph_ctx *ctx, const gbsph_particles *p, const gbsph_config *cfg,
                      gbsph_time_state *ts, gbsph_step_log *log, void *stream);

/* ------------------------------------------------------------------ adjoint */

/* Cotangents (dL/d field) of one particle state, device arrays of n entries. */
typedef struct {
    uint32_t n;
    uint32_t pad;
    gbsph_vec3 gx, gv, ga; /* positions, velocities, accelerations */
    double *gu, *gdu;      /* internal energy and its rate */
    /* Varying viscosity (GBSPH_AV_VARYING_CD10 / _MM97) only, NULL otherwise: the
     * per-particle alpha_AV and stored sound speed (device arrays, n each, in/out like
     * the others), and host accumulators incremented by dL/d alpha_min, alpha_max and
     * sigma_decay of the step's switch. */
    double *galpha, *gsoundspeed;
    double g_alpha_min, g_alpha_max, g_sigma_decay;
} gbsph_cotangents;

/* Reverse mode of one evolve_once (no reference counterpart: the differentiable step
 * of the hot path).  `start` is the state the forward step began from (x, v, a, h, u,
 * du; read only), t / dt / corrector_iters the forward step's time, dt and
 * gbsph_step_log.corrector_iters.  The step is recomputed from `start` with the same
 * dt and number of corrector evaluations (same tree, neighbour cache and ghosts), then
 * reversed: on entry `cot` holds dL/d(state after the step), on return dL/d(state
 * before it).  h after the step is treated as the exact solution of the density
 * constraint; dt and the neighbour set are held fixed.  *g_alpha_av (host) is
 * incremented by dL/d alpha_AV of this step (constant viscosity).  With a varying
 * viscosity `start` also gives alpha_AV and soundspeed, the velocity gradients and the
 * switch are reversed too, and cot->galpha / gsoundspeed / g_alpha_min / g_alpha_max /
 * g_sigma_decay carry their cotangents.  The recompute runs in cfg->precision (a
 * concrete tier: GBSPH_FP64, GBSPH_MIXED or GBSPH_MIXED_COMPENSATED, the tier the
 * forward step ran in); the reverse pass is FP64 after an FP64 recompute and FP32 pair
 * arithmetic with FP64 accumulators after a mixed one. */
int gbsph_adjoint_step(gbsph_ctx *ctx, const gbsph_particles *start, const gbsph_config *cfg,
                       double t, double dt, uint32_t corrector_iters, gbsph_cotangents *cot,
                       double *g_alpha_av, void *stream);

/* gbsph_adjoint_step in two halves, for a rollout that keeps several steps recorded at
 * once (one context per step): gbsph_adjoint_record recomputes the step from `start`
 * with its tape, keeps what the reverse pass needs in the context (tree, neighbour cache,
 * h, Omega, the tape, and the recomputed state after the step, which stays valid until
 * the context records again) and, when `after` is given, points it at that state; the
 * state after one step is the start state of the next, so a segment of steps is
 * recomputed once.  gbsph_adjoint_reverse then reverses the recorded step (same `start`,
 * cfg->precision and dt; GBSPH_ERR_STATE without a recording).  Record followed by
 * reverse on one context is gbsph_adjoint_step. */
int gbsph_adjoint_record(gbsph_ctx *ctx, const gbsph_particles *start, const gbsph_config *cfg,
                         double t, double dt, uint32_t corrector_iters, gbsph_particles *after,
                         void *stream);
int gbsph_adjoint_reverse(gbsph_ctx *ctx, const gbsph_particles *start, const gbsph_config *cfg,
                          double dt, gbsph_cotangents *cot, double *g_alpha_av, void *stream);

/* ------------------------------------------------------------------ instrumentation
 * Per-stage device time measured with CUDA events on the launching stream (the role
 * of the reference's per-step timers, SolverStorage.hpp:111-118).  Enabling resets the
 * totals; reading folds the recorded events in (it synchronises the context stream). */
uint32_t gbsph_profile_kinds(void);
/* Number of kernels this library has launched in the process so far. */
uint64_t gbsph_kernel_launches(void);

/* Memory budget of the neighbour cache's one-pass slots (bytes; 0 = the library
 * default, 24 GiB).  Both cache stages are first built in one pass into fixed slots per
 * leaf / per particle; a build that overflows is rerun with slots sized to its largest
 * row, and when those would exceed the budget the exact two-pass build (count, scan,
 * fill) runs instead.  The resulting cache is identical either way. */
int gbsph_set_cache_budget(gbsph_ctx *ctx, uint64_t bytes);
const char *gbsph_profile_name(uint32_t kind);
int gbsph_profile_enable(gbsph_ctx *ctx, int on);
int gbsph_profile_read(gbsph_ctx *ctx, double *ms_host, uint64_t *launches_host,
                       uint64_t *units_host, uint32_t n);

#ifdef __cplusplus
}
#endif

#endif /* GBSPH_H */
