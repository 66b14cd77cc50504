// Library context: the scratch arena behind the C ABI.  One context serves one
// host thread and one stream at a time (the same contract as the reference's
// per-rank compute queue).  All buffers grow on demand and are reused across steps.
#pragma once

#include "gbsph_internal.cuh"

#include <string>
#include <vector>

namespace gbsph {

// Widened bounding box of the merged positions and the Morton grid step
// (BuildTrees.cpp:26-59, CoordRangeTransform.cpp:169-184).
struct BBox {
    f64 lo[3];
    f64 hi[3];
    f64 fact[3];
};

// Small device-side reduction results, read back through pinned memory.
struct Scalars {
    u64 bbox_min[3];   // ordered-u64 min of merged positions
    u64 bbox_max[3];   // ordered-u64 max
    u64 hmax;          // ordered-u64 max of local h
    u64 eps_max;       // ordered-u64 max of eps_h (h iteration)
    u64 eps_min;       // ordered-u64 min of eps_h
    u64 epsv2_max;     // ordered-u64 max of |dv corrector|^2
    u64 dt_min;        // ordered-u64 min of per-particle CFL dt
    u64 n_unconverged; // particles whose per-thread iteration cap was hit
    u64 csr_entries;   // stage-2 entries of the one-pass cache build
    u64 csr_kept;      // entries kept by the mixed path's row compaction
    u64 cond_fa;       // ordered-u64 max over rows of the force condition sum (mixed)
    u64 cond_fu;       // ordered-u64 max of the du/dt condition sum
    u64 cond_a;        // ordered-u64 max |bare hydro force sum|
    u64 cond_du;       // ordered-u64 max |bare du/dt sum|
    f64 sum_v2;        // sum of |v|^2 after the corrector
    f64 g_alpha;       // adjoint: dL / d alpha_AV of one step
    f64 g_av[3];       // adjoint: dL / d (alpha_min, alpha_max, sigma_decay) of one step
    f64 cons[8];       // conservation totals (momentum, energies)
    u32 total;         // scan totals
    u32 total2;
    u32 ghost_total;
    u32 iters_max;     // max Newton iterations used by any particle
    u32 flags;         // error flags raised by kernels
    u32 leaf_cnt_max;  // largest stage-1 list among leaves that overflowed their slots
    u32 row_cnt_max;   // largest stage-2 row among rows that overflowed their slots
    u32 dup_keys;      // radix-sorted Morton keys had equal neighbours
};

enum KernelFlags : u32 {
    kFlagStackOverflow = 1u,
    kFlagOwnerMissing  = 2u,
    kFlagCsrOverflow   = 4u,
    kFlagLeafCap       = 8u,  // a leaf had more stage-1 candidates than the one-pass slots
    kFlagCsrCap        = 16u, // a row had more stage-2 entries than the one-pass slots
};

// FP32 copy of a node box for pre-tests: lo.w = interaction radius x Rkern.
// 32 bytes, read with one 256-bit load.
struct __align__(32) NodeBoxF {
    float4 lo;
    float4 hi;
};

// The two children of an internal node with their FP32 boxes (64 bytes, two 256-bit
// loads), so a traversal tests both children of a node together; hi.w of each box
// carries the child's node index (internal n, or leaf L - 1 + l) as raw bits.
struct __align__(32) NodePairF {
    NodeBoxF l, r;
};

// Live per-stage timing with CUDA events on the launching stream (off by default).
enum ProfKind : int {
    kProfPredict = 0,
    kProfGhosts,
    kProfMerge,
    kProfSort,
    kProfTree,
    kProfStage1,
    kProfOwner,
    kProfCacheCount,
    kProfCacheFill,
    kProfHIter,
    kProfOmega,
    kProfGatherEos,
    kProfDerivs,
    kProfAdjDerivs, // adjoint: reverse of the derivatives (staging + pair kernel)
    kProfAdjDensity, // adjoint: reverse of Omega and the density constraint
    kProfVelGrad,    // varying AV: div v, curl v, d(div v)/dt and the switch
    kProfCount
};

struct Prof {
    bool on = false;
    std::vector<cudaEvent_t> pool; // start/stop pairs
    std::vector<int> kinds;
    size_t used = 0;
    double ms[kProfCount]       = {};
    u64 launches[kProfCount]    = {};
    u64 units[kProfCount]       = {};
};

struct Ctx {
    Prof prof;
    int device          = 0;
    cudaStream_t stream = 0;
    std::string err;
    int last_status = 0;

    DevBuf scan_scratch;
    DevBuf d_scalars; // Scalars
    Scalars *h_scalars = nullptr; // pinned mirror
    DevBuf d_bbox;    // BBox

    // ---- tree (CompressedLeafBVH) over the merged set
    int key_bits = 32;
    u32 n_obj = 0, morton_count = 0, leaf_count = 0;
    DevBuf keys, sort_index, flags_a, flags_b, offsets, reduc, reduced;
    DevBuf radix_k, radix_v, radix_hist, radix_off; // radix sort ping-pong and digit tables
    DevBuf lchild, rchild, lflag, rflag, endrange, parent, boxes, visit, fboxes, fpairs;
    bool has_rint = false;

    // ---- rank-ordered copies of merged fields
    DevBuf rank_of;            // merged id -> rank
    DevBuf sx, sy, sz, sh;     // positions, h (tree build time)
    DevBuf row_rank, row_local; // local rows in rank order
    DevBuf row_flags, row_offsets;

    // ---- neighbour cache
    u64 leaf_csr_total = 0, csr_total = 0;
    u32 leaf_cap = 0, row_cap = 0; // one-pass slots per leaf / row (grown on overflow)
    u32 row_seen = 0;              // largest stage-2 row of the last build
    u64 slot_budget = 0;            // bytes of one-pass slots allowed (0: library default)
    DevBuf leaf_cnt, leaf_off, leaf_ent; // stage 1 (leaf ids)
    DevBuf owner;                        // per row: leaf index
    DevBuf leaf_thr;                     // per leaf: FP32 bits of max thr over its owned rows
    DevBuf csr_cnt, csr_off, csr_ent;    // stage 2, per row, entries are ranks
    u32 n_local = 0;
    bool cache_valid = false;

    // ---- ghosts
    u32 n_ghost = 0;
    DevBuf ghost_src, ghost_oid;  // source local id, offset index (0..25)
    DevBuf ghost_block_counts;    // per block x 26
    DevBuf mx, my, mz, mh;        // merged positions / h (merged id order)
    f64 ghost_offsets[26][3];
    DevBuf d_ghost_offsets;       // f64[26][3]

    // ---- per-step fields in rank order (corrector phase)
    DevBuf su, svx, svy, svz, som, sP, scs, sh2;
    DevBuf srho, sinv, srom; // FP64 pair-loop factors per merged particle (HydroSpace)
    // mixed precision staging (rank order); f_comp: the compensated tier's extra records
    DevBuf f_pos, f_anchor, f_aux0, f_aux1, f_aux2, f_comp;
    // error-controlled mixed precision: the tier the next step starts in (1 FP32 pair
    // arithmetic, 2 compensated) and the start state a step is recomputed from
    u32 guard_tier = 1;
    // steps left before the FP32 tier's error estimate is refreshed (0: this step), the
    // last estimate (a, du/dt), and the refresh before it with the steps between the two
    // (its growth rate; guard_prev_est < 0: none); see evolve_impl
    u32 guard_skip = 0;
    f64 guard_est_a = 0, guard_est_du = 0;
    f64 guard_prev_est = -1;
    u32 guard_since = 0;
    const f64 *guard_of = nullptr; // the position array and count the state is for
    u32 guard_n = 0;
    bool cond_this_step = true;
    DevBuf guard_state;

    // ---- per-row / per-local work arrays
    DevBuf h_old_row, eps_row, omega_local, a_old, du_old, hnew_row, omega_row;
    DevBuf aext; // external acceleration of the step (3 n, SoA)
    // varying AV: rank-ordered accelerations (3 N) and alpha (N), the updated alpha (n),
    // div v / curl v / d(div v)/dt when the caller does not take them (5 n)
    DevBuf av_arank, av_alpha_rank, av_alpha_upd, av_diag;
    DevBuf dt_part;

    // ---- adjoint: working state, tape, accumulators (local and rank order)
    DevBuf adj_state, adj_snap, adj_loc, adj_rank, adj_snap_av, adj_snap_vg, adj_vg;

    ~Ctx();
};

// ------------------------------------------------------------------ profiling
int prof_begin(Ctx &c, int kind, u64 units);
void prof_end(Ctx &c, int idx);
void prof_collect(Ctx &c); // after a stream sync: fold recorded pairs into the totals

struct ProfScope {
    Ctx &c;
    int idx;
    ProfScope(Ctx &c_, int kind, u64 units) : c(c_), idx(c_.prof.on ? prof_begin(c_, kind, units) : -1) {}
    ~ProfScope() {
        if (idx >= 0) prof_end(c, idx);
    }
};

// ------------------------------------------------------------------ stage functions
// All return cudaError_t and enqueue work on ctx.stream.

// tree.cu
// fast_sort: sort the n real keys with the radix sort (the permutation equals the bitonic
// network's whenever the keys are distinct, which it checks; the padding's order is not
// kept, so only builds whose sorted padding is never exported may ask for it)
cudaError_t tree_build(Ctx &c, const f64 *x, const f64 *y, const f64 *z, const f64 *h, u32 n,
                       u32 level, f64 htol, int key_bits, u32 morton_count, bool fast_sort = false);
cudaError_t set_bbox_host(Ctx &c, const f64 *bmin, const f64 *bmax);
cudaError_t bbox_from_merged(Ctx &c, u32 n); // reduce mx/my/mz -> widened d_bbox
cudaError_t sync_scalars(Ctx &c);            // copy Scalars to pinned host, wait

// neigh.cu
cudaError_t build_rows(Ctx &c, u32 n_local);
// P: optional FP32 position records (2 float4 per rank: hi + 1/h, lo + fl32(thr));
// when given, candidate pairs are pre-tested in FP32 (same resulting cache).
cudaError_t neigh_cache_build(Ctx &c, f64 h_tolerance, const float4 *P = nullptr);
cudaError_t tree_query(Ctx &c, const f64 *qx, const f64 *qy, const f64 *qz, u32 nq, int mode,
                       f64 s, u32 *counts, u32 *offsets, u32 *out, bool fill);

// ghosts.cu
cudaError_t periodic_ghosts(Ctx &c, const f64 *x, const f64 *y, const f64 *z, u32 vs,
                            const f64 *h, u32 n, const f64 *bmin, const f64 *bmax, f64 htol);
cudaError_t merge_positions(Ctx &c, const f64 *x, const f64 *y, const f64 *z, u32 vs,
                            const f64 *h, u32 n);

} // namespace gbsph
