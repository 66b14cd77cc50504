// C ABI of the GB300 SPH hot path (include/gbsph.h) and the one-patch
// Solver::evolve_once orchestration (shammodels/sph/src/Solver.cpp:1942-3272).

#include "../../include/gbsph.h"
#include "gbsph_ctx.cuh"
#include "adjoint.cuh"
#include "guard_rule.h"
#include "sph_kernels.cuh"
#include "sph_mixed.cuh"

#include <chrono>
#include <cmath>
#include <cstring>
#include <limits>
#include <string>

struct gbsph_ctx {
    gbsph::Ctx c;
    // the step recorded by gbsph_adjoint_record for gbsph_adjoint_reverse: its tape, the
    // recomputed state after the step (in c.adj_state), and what the reverse must match
    gbsph::StepTape adj_tape;
    gbsph_particles adj_after{};
    bool adj_ready   = false;
    bool adj_var     = false;
    uint32_t adj_n   = 0, adj_prec = 0;
    double adj_dt    = 0;
};

namespace gbsph {

template<class K>
cudaError_t sort_keys_dev(K *keys, u32 *vals, u32 len, cudaStream_t s);
cudaError_t morton_codes_dev(Ctx &c, const f64 *x, const f64 *y, const f64 *z, u32 n, u32 P,
                             int key_bits, void *out);
cudaError_t export_boxes(Ctx &c, f64 *mn, f64 *mx, f64 *rint);

std::atomic<unsigned long long> g_kernel_launches{0};

int prof_begin(Ctx &c, int kind, u64 units) {
    size_t need = 2 * (c.prof.used + 1);
    while (c.prof.pool.size() < need) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) return -1;
        c.prof.pool.push_back(e);
    }
    int idx = (int) c.prof.used++;
    if (c.prof.kinds.size() < c.prof.used) c.prof.kinds.resize(c.prof.used);
    c.prof.kinds[idx] = kind;
    c.prof.units[kind] += units;
    c.prof.launches[kind] += 1;
    cudaEventRecord(c.prof.pool[2 * idx], c.stream);
    return idx;
}

void prof_end(Ctx &c, int idx) { cudaEventRecord(c.prof.pool[2 * idx + 1], c.stream); }

void prof_collect(Ctx &c) {
    for (size_t i = 0; i < c.prof.used; i++) {
        float ms = 0;
        if (cudaEventElapsedTime(&ms, c.prof.pool[2 * i], c.prof.pool[2 * i + 1]) == cudaSuccess)
            c.prof.ms[c.prof.kinds[i]] += ms;
    }
    c.prof.used = 0;
}

Ctx::~Ctx() {
    for (cudaEvent_t e : prof.pool) cudaEventDestroy(e);
    DevBuf *bufs[] = {&scan_scratch, &d_scalars, &d_bbox, &keys, &sort_index, &flags_a, &flags_b,
                      &offsets, &reduc, &reduced, &radix_k, &radix_v, &radix_hist, &radix_off, &lchild, &rchild, &lflag, &rflag, &endrange,
                      &parent, &boxes, &visit, &fboxes, &fpairs, &rank_of, &sx, &sy, &sz, &sh, &row_rank,
                      &row_local, &row_flags, &row_offsets, &leaf_cnt, &leaf_off, &leaf_ent,
                      &owner, &leaf_thr, &csr_cnt, &csr_off, &csr_ent, &ghost_src, &ghost_oid,
                      &ghost_block_counts, &mx, &my, &mz, &mh, &d_ghost_offsets, &su, &svx, &svy,
                      &svz, &som, &sP, &scs, &srho, &sinv, &srom, &sh2, &f_pos, &f_anchor, &f_aux0, &f_aux1, &f_aux2, &f_comp, &guard_state,
                      &h_old_row, &eps_row, &omega_local, &a_old, &du_old, &hnew_row, &omega_row,
                      &dt_part, &adj_state, &adj_snap, &adj_loc, &adj_rank, &adj_snap_av, &adj_snap_vg, &adj_vg, &aext, &av_arank,
                      &av_alpha_rank, &av_alpha_upd, &av_diag};
    cudaSetDevice(device);
    for (DevBuf *b : bufs) b->release(stream);
    cudaStreamSynchronize(stream);
    if (h_scalars) cudaFreeHost(h_scalars);
}

namespace {

__global__ void k_cache_export_counts(u32 n, const u32 *__restrict__ row_local,
                                      const u32 *__restrict__ cnt, u32 *__restrict__ out_cnt) {
    u32 t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) out_cnt[row_local[t]] = cnt[t];
}
__global__ void k_cache_export_entries(u32 n, const u32 *__restrict__ row_local,
                                       const u32 *__restrict__ cnt, const u32 *__restrict__ off,
                                       const u32 *__restrict__ ent,
                                       const u32 *__restrict__ sort_index,
                                       const u32 *__restrict__ out_scanned,
                                       u32 *__restrict__ out_ent) {
    u32 t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    u32 w = out_scanned[row_local[t]];
    for (u32 k = off[t]; k < off[t] + cnt[t]; k++) out_ent[w++] = sort_index[ent[k]];
}

struct ScalarsReset {
    static void eps(Scalars &s) {
        s.eps_max   = 0;
        s.eps_min   = ~0ull;
        s.iters_max = 0;
    }
};

__global__ void k_reset_eps(Scalars *sc) {
    sc->eps_max   = 0;
    sc->eps_min   = ~0ull;
    sc->iters_max = 0;
}
__global__ void k_reset_corrector(Scalars *sc) {
    sc->epsv2_max = 0;
    sc->dt_min    = ~0ull;
    sc->sum_v2    = 0;
}

// tape: velocity and energy (SoA) before a corrector evaluation
__global__ void k_snap_vu(u32 n, const f64 *__restrict__ vx, const f64 *__restrict__ vy,
                          const f64 *__restrict__ vz, u32 vs, const f64 *__restrict__ u,
                          f64 *__restrict__ out) {
    u32 i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    size_t iv = (size_t) i * vs, n_ = n;
    out[i]          = vx[iv];
    out[n_ + i]     = vy[iv];
    out[2 * n_ + i] = vz[iv];
    out[3 * n_ + i] = u[i];
}

// working copy of a particle state (strided vectors -> SoA) for the adjoint recompute
__global__ void k_copy_state(u32 n, gbsph_vec3 x, gbsph_vec3 v, gbsph_vec3 a, const f64 *h,
                             const f64 *u, const f64 *du, f64 *__restrict__ out) {
    u32 i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    size_t n_ = n;
    out[0 * n_ + i]  = x.x[(size_t) i * x.stride];
    out[1 * n_ + i]  = x.y[(size_t) i * x.stride];
    out[2 * n_ + i]  = x.z[(size_t) i * x.stride];
    out[3 * n_ + i]  = v.x[(size_t) i * v.stride];
    out[4 * n_ + i]  = v.y[(size_t) i * v.stride];
    out[5 * n_ + i]  = v.z[(size_t) i * v.stride];
    out[6 * n_ + i]  = a.x[(size_t) i * a.stride];
    out[7 * n_ + i]  = a.y[(size_t) i * a.stride];
    out[8 * n_ + i]  = a.z[(size_t) i * a.stride];
    out[9 * n_ + i]  = h[i];
    out[10 * n_ + i] = u[i];
    out[11 * n_ + i] = du[i];
}

// inverse of k_copy_state: SoA working copy -> the caller's (strided) fields
__global__ void k_restore_state(u32 n, gbsph_vec3 x, gbsph_vec3 v, gbsph_vec3 a, f64 *h, f64 *u,
                                f64 *du, const f64 *__restrict__ in) {
    u32 i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    size_t n_ = n;
    x.x[(size_t) i * x.stride] = in[0 * n_ + i];
    x.y[(size_t) i * x.stride] = in[1 * n_ + i];
    x.z[(size_t) i * x.stride] = in[2 * n_ + i];
    v.x[(size_t) i * v.stride] = in[3 * n_ + i];
    v.y[(size_t) i * v.stride] = in[4 * n_ + i];
    v.z[(size_t) i * v.stride] = in[5 * n_ + i];
    a.x[(size_t) i * a.stride] = in[6 * n_ + i];
    a.y[(size_t) i * a.stride] = in[7 * n_ + i];
    a.z[(size_t) i * a.stride] = in[8 * n_ + i];
    h[i]  = in[9 * n_ + i];
    u[i]  = in[10 * n_ + i];
    du[i] = in[11 * n_ + i];
}

} // namespace
} // namespace gbsph

using namespace gbsph;

static int fail(gbsph_ctx *ctx, int code, const std::string &msg) {
    ctx->c.err         = msg;
    ctx->c.last_status = code;
    return code;
}

#define CU(expr)                                                                                  \
    do {                                                                                          \
        cudaError_t _e = (expr);                                                                  \
        if (_e != cudaSuccess) {                                                                  \
            std::string _m = std::string(#expr) + ": " + cudaGetErrorString(_e);                  \
            if (!ctx->c.err.empty()) _m += " (" + ctx->c.err + ")";                               \
            return fail(ctx, GBSPH_ERR_CUDA, _m);                                                 \
        }                                                                                         \
    } while (0)

#define REQUIRE_ARG(cond, msg)                                                                    \
    do {                                                                                          \
        if (!(cond)) return fail(ctx, GBSPH_ERR_ARG, msg);                                        \
    } while (0)

// Select the device and stream for this call; a stream switch drains the old one so
// the stream-ordered scratch allocations are safe to reuse.
static int enter(gbsph_ctx *ctx, void *stream) {
    if (!ctx) return GBSPH_ERR_ARG;
    ctx->c.err.clear();
    cudaError_t e = cudaSetDevice(ctx->c.device);
    if (e != cudaSuccess) return fail(ctx, GBSPH_ERR_CUDA, cudaGetErrorString(e));
    cudaStream_t s = (cudaStream_t) stream;
    if (s != ctx->c.stream) {
        cudaStreamSynchronize(ctx->c.stream);
        ctx->c.stream = s;
    }
    return GBSPH_OK;
}
#define ENTER(ctx, stream)                                                                        \
    do {                                                                                          \
        int _r = enter((ctx), (stream));                                                          \
        if (_r) return _r;                                                                        \
    } while (0)

extern "C" {

const char *gbsph_version(void) { return "gbsph 0.1 (sm_103a)"; }

static const char *kProfNames[kProfCount] = {
    "predict", "ghosts", "merge_bbox", "morton_sort", "tree", "leaf_lists", "owner",
    "cache_count", "cache_fill", "h_iterate", "omega", "gather_eos", "derivs", "adj_derivs",
    "adj_density", "velgrad"};

uint32_t gbsph_profile_kinds(void) { return kProfCount; }

uint64_t gbsph_kernel_launches(void) { return g_kernel_launches.load(std::memory_order_relaxed); }

int gbsph_set_cache_budget(gbsph_ctx *ctx, uint64_t bytes) {
    if (!ctx) return GBSPH_ERR_ARG;
    ctx->c.slot_budget = bytes;
    ctx->c.leaf_cap    = 0;
    ctx->c.row_cap     = 0;
    return GBSPH_OK;
}

const char *gbsph_profile_name(uint32_t kind) {
    return kind < kProfCount ? kProfNames[kind] : "";
}

int gbsph_profile_enable(gbsph_ctx *ctx, int on) {
    if (!ctx) return GBSPH_ERR_ARG;
    Prof &p = ctx->c.prof;
    cudaStreamSynchronize(ctx->c.stream);
    p.on   = on != 0;
    p.used = 0;
    for (int k = 0; k < kProfCount; k++) {
        p.ms[k]       = 0;
        p.launches[k] = 0;
        p.units[k]    = 0;
    }
    return GBSPH_OK;
}

int gbsph_profile_read(gbsph_ctx *ctx, double *ms_host, uint64_t *launches_host,
                       uint64_t *units_host, uint32_t n) {
    if (!ctx) return GBSPH_ERR_ARG;
    cudaStreamSynchronize(ctx->c.stream);
    prof_collect(ctx->c);
    for (uint32_t k = 0; k < n && k < (uint32_t) kProfCount; k++) {
        if (ms_host) ms_host[k] = ctx->c.prof.ms[k];
        if (launches_host) launches_host[k] = ctx->c.prof.launches[k];
        if (units_host) units_host[k] = ctx->c.prof.units[k];
    }
    return GBSPH_OK;
}

int gbsph_create(gbsph_ctx **out, int device) {
    if (!out) return GBSPH_ERR_ARG;
    *out = nullptr;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return GBSPH_ERR_CUDA;
    gbsph_ctx *ctx = new gbsph_ctx();
    ctx->c.device  = device;
    ctx->c.stream  = 0;
    if (cudaMallocHost(&ctx->c.h_scalars, sizeof(Scalars)) != cudaSuccess ||
        ctx->c.d_scalars.ensure(sizeof(Scalars), 0) != cudaSuccess ||
        ctx->c.d_bbox.ensure(sizeof(BBox), 0) != cudaSuccess) {
        delete ctx;
        return GBSPH_ERR_CUDA;
    }
    cudaMemsetAsync(ctx->c.d_scalars.p, 0, sizeof(Scalars), 0);
    cudaStreamSynchronize(0);
    *out = ctx;
    return GBSPH_OK;
}

void gbsph_destroy(gbsph_ctx *ctx) {
    if (ctx) delete ctx;
}

const char *gbsph_last_error(const gbsph_ctx *ctx) { return ctx ? ctx->c.err.c_str() : "null context"; }

int gbsph_morton_codes(gbsph_ctx *ctx, const double *x, const double *y, const double *z,
                       uint32_t n, uint32_t morton_count, const double bmin_host[3],
                       const double bmax_host[3], int key_bits, void *keys_out, void *stream) {
    ENTER(ctx, stream);
    REQUIRE_ARG(morton_count >= n, "MortonCodeSet: morton_count < cnt_obj");
    REQUIRE_ARG(key_bits == 32 || key_bits == 64, "key_bits must be 32 or 64");
    CU(set_bbox_host(ctx->c, bmin_host, bmax_host));
    CU(morton_codes_dev(ctx->c, x, y, z, n, morton_count, key_bits, keys_out));
    return GBSPH_OK;
}

int gbsph_sort_by_key(gbsph_ctx *ctx, void *keys, uint32_t *vals, uint32_t len, int key_bits,
                      void *stream) {
    ENTER(ctx, stream);
    REQUIRE_ARG(len == 0 || (len & (len - 1)) == 0,
                "this algorithm can only be used with length that are powers of two");
    if (key_bits == 64) CU(sort_keys_dev<u64>((u64 *) keys, vals, len, ctx->c.stream));
    else CU(sort_keys_dev<u32>((u32 *) keys, vals, len, ctx->c.stream));
    return GBSPH_OK;
}

int gbsph_build_tree(gbsph_ctx *ctx, const double *x, const double *y, const double *z,
                     const double *h, uint32_t n, const double bmin_host[3],
                     const double bmax_host[3], uint32_t reduction_level, double htol,
                     int key_bits, uint32_t morton_count, void *stream) {
    ENTER(ctx, stream);
    REQUIRE_ARG(n > 0, "obj_cnt is 0, cannot build a CompressedLeafBVH");
    REQUIRE_ARG(key_bits == 32 || key_bits == 64, "key_bits must be 32 or 64");
    REQUIRE_ARG(morton_count == 0 || (morton_count >= n && (morton_count & (morton_count - 1)) == 0),
                "morton_count must be 0 or a power of two >= n");
    CU(cudaMemsetAsync(ctx->c.d_scalars.p, 0, sizeof(Scalars), ctx->c.stream));
    CU(set_bbox_host(ctx->c, bmin_host, bmax_host));
    CU(tree_build(ctx->c, x, y, z, h, n, reduction_level, htol, key_bits, morton_count));
    ctx->c.cache_valid = false;
    CU(cudaStreamSynchronize(ctx->c.stream));
    return GBSPH_OK;
}

int gbsph_tree_counts(gbsph_ctx *ctx, uint32_t *mc, uint32_t *lc) {
    if (!ctx) return GBSPH_ERR_ARG;
    if (mc) *mc = ctx->c.morton_count;
    if (lc) *lc = ctx->c.leaf_count;
    return GBSPH_OK;
}

int gbsph_tree_export(gbsph_ctx *ctx, void *sorted_keys, uint32_t *sort_index, uint32_t *reduc,
                      void *reduced_keys, uint32_t *lchild, uint32_t *rchild, uint8_t *lflag,
                      uint8_t *rflag, uint32_t *endrange, double *aabb_min, double *aabb_max,
                      double *rint, void *stream) {
    ENTER(ctx, stream);
    Ctx &c = ctx->c;
    REQUIRE_ARG(c.leaf_count > 0, "no tree built");
    size_t ks = c.key_bits / 8;
    u32 P = c.morton_count, L = c.leaf_count, I = L - 1;
    cudaStream_t s = c.stream;
    auto cp = [&](void *dst, const void *src, size_t bytes) {
        return (dst && bytes) ? cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, s)
                              : cudaSuccess;
    };
    CU(cp(sorted_keys, c.keys.p, ks * P));
    CU(cp(sort_index, c.sort_index.p, 4 * (size_t) P));
    CU(cp(reduc, c.reduc.p, 4 * ((size_t) L + 2)));
    CU(cp(reduced_keys, c.reduced.p, ks * L));
    CU(cp(lchild, c.lchild.p, 4 * (size_t) I));
    CU(cp(rchild, c.rchild.p, 4 * (size_t) I));
    CU(cp(lflag, c.lflag.p, I));
    CU(cp(rflag, c.rflag.p, I));
    CU(cp(endrange, c.endrange.p, 4 * (size_t) I));
    if (aabb_min || aabb_max || rint) CU(export_boxes(c, aabb_min, aabb_max, rint));
    CU(cudaStreamSynchronize(s));
    return GBSPH_OK;
}

int gbsph_tree_query(gbsph_ctx *ctx, const double *qx, const double *qy, const double *qz,
                     uint32_t nq, int mode, double s, uint32_t *counts, uint32_t *out,
                     uint64_t capacity, uint64_t *total_host, void *stream) {
    ENTER(ctx, stream);
    Ctx &c = ctx->c;
    REQUIRE_ARG(c.leaf_count > 0, "no tree built");
    REQUIRE_ARG(counts != nullptr, "counts required");
    CU(cudaMemsetAsync(c.d_scalars.p, 0, sizeof(Scalars), c.stream));
    CU(tree_query(c, qx, qy, qz, nq, mode, s, counts, nullptr, nullptr, false));
    CU(c.offsets.ensure(sizeof(u32) * ((size_t) nq + 1), c.stream));
    CU(scan_exclusive_u32(counts, c.offsets.as<u32>(), nq, &c.d_scalars.as<Scalars>()->total,
                          c.scan_scratch, c.stream));
    CU(sync_scalars(c));
    u64 total = c.h_scalars->total;
    if (total_host) *total_host = total;
    if (out && capacity >= total) {
        CU(tree_query(c, qx, qy, qz, nq, mode, s, nullptr, c.offsets.as<u32>(), out, true));
        CU(cudaStreamSynchronize(c.stream));
    } else if (out) {
        return fail(ctx, GBSPH_ERR_CAPACITY, "tree_query: output capacity too small");
    }
    return GBSPH_OK;
}

int gbsph_neighbour_cache(gbsph_ctx *ctx, uint32_t n_local, double htol, uint32_t precision,
                          void *stream) {
    ENTER(ctx, stream);
    Ctx &c = ctx->c;
    if (c.leaf_count == 0 || !c.has_rint || c.key_bits != 32)
        return fail(ctx, GBSPH_ERR_STATE, "neighbour cache needs a 32-bit tree built with h");
    REQUIRE_ARG(n_local <= c.n_obj, "n_local > merged count");
    REQUIRE_ARG(precision == GBSPH_FP64 || precision == GBSPH_MIXED, "unknown precision");
    CU(cudaMemsetAsync(c.d_scalars.p, 0, sizeof(Scalars), c.stream));
    CU(build_rows(c, n_local));
    if (precision == GBSPH_MIXED) {
        CU(stage_positions_mixed(c, c.n_obj, htol));
        CU(neigh_cache_build(c, htol, mixed_positions(c)));
    } else {
        CU(neigh_cache_build(c, htol));
    }
    CU(cudaStreamSynchronize(c.stream));
    return GBSPH_OK;
}

int gbsph_cache_size(gbsph_ctx *ctx, uint64_t *total, uint64_t *leaf_total) {
    if (!ctx) return GBSPH_ERR_ARG;
    if (total) *total = ctx->c.csr_total;
    if (leaf_total) *leaf_total = ctx->c.leaf_csr_total;
    return GBSPH_OK;
}

int gbsph_cache_export(gbsph_ctx *ctx, uint32_t *cnt, uint32_t *scanned, uint32_t *entries,
                       void *stream) {
    ENTER(ctx, stream);
    Ctx &c = ctx->c;
    if (!c.cache_valid) return fail(ctx, GBSPH_ERR_STATE, "no neighbour cache built");
    REQUIRE_ARG(cnt && scanned, "cnt and scanned required");
    u32 n = c.n_local;
    { k_cache_export_counts<<<div_up(n, 256), 256, 0, c.stream>>>(n, c.row_local.as<u32>(),
                                                                c.csr_cnt.as<u32>(), cnt); GBSPH_COUNTED; }
    CU(cudaGetLastError());
    CU(scan_exclusive_u32(cnt, scanned, n, &c.d_scalars.as<Scalars>()->total2, c.scan_scratch,
                          c.stream));
    if (entries)
        { k_cache_export_entries<<<div_up(n, 256), 256, 0, c.stream>>>(
            n, c.row_local.as<u32>(), c.csr_cnt.as<u32>(), c.csr_off.as<u32>(), c.csr_ent.as<u32>(),
            c.sort_index.as<u32>(), scanned, entries); GBSPH_COUNTED; }
    CU(cudaGetLastError());
    CU(cudaStreamSynchronize(c.stream));
    return GBSPH_OK;
}

int gbsph_h_iterate(gbsph_ctx *ctx, const uint32_t *cnt, const uint32_t *scanned,
                    const uint32_t *entries, const double *x, const double *y, const double *z,
                    const double *h_old, double *h_new, double *eps, uint32_t n_local,
                    double pmass, double h_evol_max, double h_evol_iter_max, uint32_t iters,
                    double *max_eps_host, double *min_eps_host, uint32_t *iters_used_host,
                    void *stream) {
    ENTER(ctx, stream);
    Ctx &c = ctx->c;
    REQUIRE_ARG(iters >= 1, "iters >= 1");
    RowSpace rs{n_local, nullptr, nullptr, cnt, scanned, entries, x, y, z};
    { k_reset_eps<<<1, 1, 0, c.stream>>>(c.d_scalars.as<Scalars>()); GBSPH_COUNTED; }
    CU(h_iterate64(c, rs, h_old, h_new, eps, pmass, h_evol_max, h_evol_iter_max, iters));
    CU(sync_scalars(c));
    if (max_eps_host) *max_eps_host = ordered_to_f64(c.h_scalars->eps_max);
    if (min_eps_host) *min_eps_host = ordered_to_f64(c.h_scalars->eps_min);
    if (iters_used_host) *iters_used_host = c.h_scalars->iters_max;
    return GBSPH_OK;
}

int gbsph_omega(gbsph_ctx *ctx, const uint32_t *cnt, const uint32_t *scanned,
                const uint32_t *entries, const double *x, const double *y, const double *z,
                const double *h, uint32_t n_local, double pmass, double *omega, void *stream) {
    ENTER(ctx, stream);
    RowSpace rs{n_local, nullptr, nullptr, cnt, scanned, entries, x, y, z};
    CU(omega64(ctx->c, rs, h, pmass, omega, nullptr));
    CU(cudaStreamSynchronize(ctx->c.stream));
    return GBSPH_OK;
}

int gbsph_eos_adiabatic(gbsph_ctx *ctx, const double *h, const double *u, uint32_t n, double pmass,
                        double gamma, double *P, double *cs, void *stream) {
    ENTER(ctx, stream);
    CU(eos64(ctx->c, n, h, u, pmass, gamma, P, cs));
    CU(cudaStreamSynchronize(ctx->c.stream));
    return GBSPH_OK;
}

int gbsph_kdk_predict(gbsph_ctx *ctx, const gbsph_particles *p, double dt, uint32_t periodic,
                      const double *bmin_host, const double *bmax_host, void *stream) {
    ENTER(ctx, stream);
    Ctx &c = ctx->c;
    REQUIRE_ARG(p && p->n > 0, "empty patch");
    REQUIRE_ARG(!periodic || (bmin_host && bmax_host), "the periodic wrap needs the box");
    REQUIRE_ARG(p->xyz.stride == p->vxyz.stride && p->xyz.stride == p->axyz.stride,
                "xyz, vxyz and axyz must share one element stride");
    LocalFields lf{p->xyz.x,  p->xyz.y,  p->xyz.z,  p->vxyz.x, p->vxyz.y,  p->vxyz.z,
                   p->axyz.x, p->axyz.y, p->axyz.z, p->xyz.stride, p->hpart, p->uint, p->duint};
    const f64 zero[3] = {0, 0, 0};
    CU(predict64(c, lf, p->n, dt, periodic ? 1 : 0, periodic ? bmin_host : zero,
                 periodic ? bmax_host : zero));
    CU(cudaStreamSynchronize(c.stream));
    return GBSPH_OK;
}

int gbsph_kdk_correct(gbsph_ctx *ctx, const gbsph_particles *p, gbsph_vec3 a_old,
                      const double *du_old, double dt, double *eps_v_host, void *stream) {
    ENTER(ctx, stream);
    Ctx &c = ctx->c;
    REQUIRE_ARG(p && p->n > 0, "empty patch");
    REQUIRE_ARG(a_old.x && a_old.y && a_old.z && du_old, "a_old and du_old required");
    REQUIRE_ARG(p->vxyz.stride == p->axyz.stride, "vxyz and axyz must share one element stride");
    LocalFields lf{p->xyz.x,  p->xyz.y,  p->xyz.z,  p->vxyz.x, p->vxyz.y,  p->vxyz.z,
                   p->axyz.x, p->axyz.y, p->axyz.z, p->vxyz.stride, p->hpart, p->uint, p->duint};
    Scalars *dsc = c.d_scalars.as<Scalars>();
    { k_reset_corrector<<<1, 1, 0, c.stream>>>(dsc); GBSPH_COUNTED; }
    CU(kdk_correct64(c, lf, p->n, a_old.x, a_old.y, a_old.z, a_old.stride, du_old, dt));
    CU(sync_scalars(c));
    f64 veps  = std::sqrt(ordered_to_f64(c.h_scalars->epsv2_max));
    f64 vmean = std::sqrt(c.h_scalars->sum_v2 / f64(p->n));
    f64 eps_v = veps / vmean;
    if (vmean <= 0) eps_v = 0;
    if (eps_v_host) *eps_v_host = eps_v;
    return GBSPH_OK;
}

int gbsph_cfl(gbsph_ctx *ctx, const double *h, const double *vsig, gbsph_vec3 a, uint32_t n,
              double C_cour, double C_force, double *dt_part, double *dt_min_host, void *stream) {
    ENTER(ctx, stream);
    Ctx &c = ctx->c;
    REQUIRE_ARG(h && vsig && a.x && a.y && a.z, "h, vsig and a required");
    REQUIRE_ARG(n > 0, "empty patch");
    Scalars *dsc = c.d_scalars.as<Scalars>();
    { k_reset_corrector<<<1, 1, 0, c.stream>>>(dsc); GBSPH_COUNTED; }
    CU(cfl64(c, n, h, vsig, a.x, a.y, a.z, a.stride, C_cour, C_force, dt_part));
    CU(sync_scalars(c));
    if (dt_min_host) *dt_min_host = ordered_to_f64(c.h_scalars->dt_min);
    return GBSPH_OK;
}

int gbsph_conservation(gbsph_ctx *ctx, const gbsph_particles *p, double pmass, double out_host[8],
                       void *stream) {
    ENTER(ctx, stream);
    Ctx &c = ctx->c;
    REQUIRE_ARG(p && out_host, "null argument");
    REQUIRE_ARG(p->n > 0, "empty patch");
    REQUIRE_ARG(p->vxyz.stride == p->axyz.stride, "vxyz and axyz must share one element stride");
    LocalFields lf{p->xyz.x,  p->xyz.y,  p->xyz.z,  p->vxyz.x, p->vxyz.y,  p->vxyz.z,
                   p->axyz.x, p->axyz.y, p->axyz.z, p->vxyz.stride, p->hpart, p->uint, p->duint};
    CU(c.av_diag.ensure(sizeof(f64) * (8 * 1024 + 8), c.stream));
    f64 *scratch = c.av_diag.as<f64>();
    CU(conservation64(c, lf, p->n, pmass, scratch + 8 * 1024, scratch));
    CU(cudaMemcpyAsync(out_host, scratch + 8 * 1024, 8 * sizeof(f64), cudaMemcpyDeviceToHost, c.stream));
    CU(cudaStreamSynchronize(c.stream));
    return GBSPH_OK;
}

int gbsph_eos_locally_isothermal(gbsph_ctx *ctx, gbsph_vec3 xyz, const double *h, uint32_t n,
                                 double pmass, double cs0, double r0, double q, double *P,
                                 double *cs, void *stream) {
    ENTER(ctx, stream);
    REQUIRE_ARG(xyz.x && xyz.y && xyz.z && h && P && cs, "null argument");
    REQUIRE_ARG(r0 > 0, "r0 must be positive");
    if (n == 0) return GBSPH_OK;
    CU(eos_lp07(ctx->c, n, xyz.x, xyz.y, xyz.z, xyz.stride, h, pmass, cs0, r0, q, P, cs));
    CU(cudaStreamSynchronize(ctx->c.stream));
    return GBSPH_OK;
}

int gbsph_derivs_constAV(gbsph_ctx *ctx, const uint32_t *cnt, const uint32_t *scanned,
                         const uint32_t *entries, const double *x, const double *y,
                         const double *z, const double *vx, const double *vy, const double *vz,
                         const double *h, const double *omega, const double *u, const double *P,
                         const double *cs, uint32_t n_local, uint32_t n_merged, double pmass,
                         double alpha_u, double alpha_AV, double beta_AV, uint32_t precision,
                         double *ax, double *ay, double *az, double *du, double *vsig,
                         void *stream) {
    ENTER(ctx, stream);
    REQUIRE_ARG(n_merged >= n_local, "n_merged < n_local");
    ctx->c.n_obj = n_merged;
    RowSpace rs{n_local, nullptr, nullptr, cnt, scanned, entries, x, y, z};
    HydroSpace hs{h, u, vx, vy, vz, omega, P, cs};
    if (precision == GBSPH_MIXED) {
        CU(derivs_mixed_module(ctx->c, rs, hs, pmass, alpha_u, alpha_AV, beta_AV, ax, ay, az, du,
                               vsig));
    } else {
        REQUIRE_ARG(precision == GBSPH_FP64, "unknown precision");
        CU(derivs64(ctx->c, rs, hs, pmass, alpha_u, alpha_AV, beta_AV, ax, ay, az, du, vsig));
    }
    CU(cudaStreamSynchronize(ctx->c.stream));
    return GBSPH_OK;
}

int gbsph_periodic_ghosts(gbsph_ctx *ctx, gbsph_vec3 xyz, const double *h, uint32_t n_local,
                          const double bmin_host[3], const double bmax_host[3], double htol,
                          uint32_t *n_ghost_host, void *stream) {
    ENTER(ctx, stream);
    Ctx &c = ctx->c;
    REQUIRE_ARG(n_local > 0, "empty patch");
    CU(periodic_ghosts(c, xyz.x, xyz.y, xyz.z, xyz.stride, h, n_local, bmin_host, bmax_host, htol));
    CU(merge_positions(c, xyz.x, xyz.y, xyz.z, xyz.stride, h, n_local));
    CU(cudaStreamSynchronize(c.stream));
    c.n_local = n_local;
    if (n_ghost_host) *n_ghost_host = c.n_ghost;
    return GBSPH_OK;
}

int gbsph_ghost_export(gbsph_ctx *ctx, uint32_t *src, uint8_t *offset_id, double *mx, double *my,
                       double *mz, double *mh, void *stream) {
    ENTER(ctx, stream);
    Ctx &c = ctx->c;
    u32 G = c.n_ghost, N = c.n_local + c.n_ghost;
    cudaStream_t s = c.stream;
    if (src && G) CU(cudaMemcpyAsync(src, c.ghost_src.p, 4 * (size_t) G, cudaMemcpyDeviceToDevice, s));
    if (offset_id && G) CU(cudaMemcpyAsync(offset_id, c.ghost_oid.p, G, cudaMemcpyDeviceToDevice, s));
    if (mx) CU(cudaMemcpyAsync(mx, c.mx.p, 8 * (size_t) N, cudaMemcpyDeviceToDevice, s));
    if (my) CU(cudaMemcpyAsync(my, c.my.p, 8 * (size_t) N, cudaMemcpyDeviceToDevice, s));
    if (mz) CU(cudaMemcpyAsync(mz, c.mz.p, 8 * (size_t) N, cudaMemcpyDeviceToDevice, s));
    if (mh) CU(cudaMemcpyAsync(mh, c.mh.p, 8 * (size_t) N, cudaMemcpyDeviceToDevice, s));
    CU(cudaStreamSynchronize(s));
    return GBSPH_OK;
}

} // extern "C"

// Estimated relative error of the FP32 tier's accelerations and du/dt on the first
// corrector evaluation of a step: the FP32 rounding of the pair terms, and of the h, rho,
// P, Omega and u they are built from, errs in proportion to the summed term magnitudes,
// which the derivatives pass accumulates per row.  With the condition C = largest sum /
// largest result of a field, the estimate is 3e-7 + 1.5e-7 C: measured errors per unit
// of condition (one step, FP32 tier against FP64) span 1.5e-8 to 1.4e-7 on the Sedov,
// clustered, sound-wave, disc and homogeneous workloads (C from 1 to 3.2e4), and
// 2.4e-7 at C = 1 (the rounding of well-conditioned sums); the estimate is above every
// measured error.  A field that vanishes while its terms do not is taken as unbounded
// error.
static constexpr f64 kErrBase = 3e-7;
static constexpr f64 kErrCond = 1.5e-7;
static f64 err_estimate(u64 sum_bits, u64 max_bits) {
    const f64 s = ordered_to_f64(sum_bits), m = ordered_to_f64(max_bits);
    if (!(s > 0)) return 0;
    if (!(m > 0)) return std::numeric_limits<f64>::infinity();
    return kErrBase + kErrCond * s / m;
}

// One step (Solver::evolve_once) in one precision tier (GBSPH_FP64, GBSPH_MIXED or
// GBSPH_MIXED_COMPENSATED).  With a tape, exactly tape->forced_iters corrector
// evaluations run and the velocity / energy before each is recorded.
static int evolve_tier(gbsph_ctx *ctx, const gbsph_particles *p, const gbsph_config *cfg,
                       gbsph_time_state *ts, gbsph_step_log *log, StepTape *tape, u32 tier) {
    Ctx &c = ctx->c;
    REQUIRE_ARG(p && cfg && ts, "null argument");
    REQUIRE_ARG(p->n > 0, "empty patch");
    REQUIRE_ARG(cfg->pmass > 0,
                "invalid gpart_mass, this configuration can not converge (Solver.cpp:1096-1102)");
    REQUIRE_ARG(tier == GBSPH_FP64 || tier == GBSPH_MIXED || tier == GBSPH_MIXED_COMPENSATED,
                "unknown precision");
    REQUIRE_ARG(p->xyz.stride == p->vxyz.stride && p->xyz.stride == p->axyz.stride,
                "xyz, vxyz and axyz must share one element stride");
    REQUIRE_ARG(cfg->eos_kind == GBSPH_EOS_ADIABATIC || cfg->eos_kind == GBSPH_EOS_LOCALLY_ISOTHERMAL_LP07,
                "unknown equation of state");
    REQUIRE_ARG(cfg->ext_kind == GBSPH_EXT_NONE || cfg->ext_kind == GBSPH_EXT_POINT_MASS,
                "unknown external force");
    REQUIRE_ARG(cfg->eos_kind != GBSPH_EOS_LOCALLY_ISOTHERMAL_LP07 || cfg->eos_r0 > 0,
                "locally isothermal EOS needs r0 > 0");
    REQUIRE_ARG(cfg->av_kind == GBSPH_AV_CONSTANT || cfg->av_kind == GBSPH_AV_VARYING_CD10 ||
                    cfg->av_kind == GBSPH_AV_VARYING_MM97,
                "unknown artificial viscosity");
    // varying viscosity (CD10 or MM97): per-particle alpha from the velocity gradients
    const bool cd10 = cfg->av_kind != GBSPH_AV_CONSTANT;
    REQUIRE_ARG(!cd10 || (p->alpha_AV && p->soundspeed),
                "the varying viscosity needs the alpha_AV and soundspeed fields");
    REQUIRE_ARG(!cd10 || !p->curlv.x || (p->curlv.y && p->curlv.z && p->curlv.stride > 0),
                "curlv needs its three components and a stride");
    auto t_start = std::chrono::steady_clock::now();
    cudaStream_t s = c.stream;
    const u32 n    = p->n;
    const f64 dt   = ts->dt;
    const bool mixed = tier != GBSPH_FP64;
    const bool comp  = tier == GBSPH_MIXED_COMPENSATED;
    LocalFields lf{p->xyz.x,  p->xyz.y,  p->xyz.z,  p->vxyz.x, p->vxyz.y,  p->vxyz.z,
                   p->axyz.x, p->axyz.y, p->axyz.z, p->xyz.stride, p->hpart, p->uint, p->duint};
    gbsph_step_log lg;
    std::memset(&lg, 0, sizeof(lg));
    lg.t       = ts->t;
    lg.dt      = dt;
    lg.n_local = n;
    Scalars *dsc = c.d_scalars.as<Scalars>();
    CU(cudaMemsetAsync(dsc, 0, sizeof(Scalars), s));

    // ---- leapfrog predictor + position boundary (+ velocity-independent external force)
    ExtAccel ext{nullptr, nullptr, nullptr};
    if (cfg->ext_kind == GBSPH_EXT_POINT_MASS) {
        CU(c.aext.ensure(sizeof(f64) * 3 * (size_t) n, s));
        f64 *A = c.aext.as<f64>();
        ext    = ExtAccel{A, A + n, A + 2 * (size_t) n};
        CU(predict64(c, lf, n, dt, (int) cfg->periodic, cfg->box_min, cfg->box_max,
                     -cfg->central_mass * cfg->constant_G, A, A + n, A + 2 * (size_t) n));
    } else {
        CU(predict64(c, lf, n, dt, (int) cfg->periodic, cfg->box_min, cfg->box_max));
    }
    const EosParams eos{cfg->eos_kind, cfg->gamma, cfg->cs0, cfg->eos_r0, cfg->eos_q};

    // ---- sph_prestep (Solver.cpp:1060-1304)
    CU(c.h_old_row.ensure(8 * (size_t) n, s));
    CU(c.hnew_row.ensure(8 * (size_t) n, s));
    CU(c.eps_row.ensure(8 * (size_t) n, s));
    CU(c.omega_local.ensure(8 * (size_t) n, s));
    // per-particle Newton threshold (0 selects the reference's 1e-6)
    const f64 eps_p    = cfg->epsilon_h_particle > 0 ? cfg->epsilon_h_particle : 1e-6;
    const bool fused_h = cfg->epsilon_h <= eps_p;
    u32 hstep = 0;
    f64 max_eps = 0, min_eps = 0;
    bool converged = false;
    RowSpace rs{};
    for (; hstep < cfg->h_max_subcycles; hstep++) {
        if (cfg->periodic) {
            CU(periodic_ghosts(c, lf.x, lf.y, lf.z, lf.vs, lf.h, n, cfg->box_min, cfg->box_max,
                               cfg->htol_up_coarse));
        } else {
            c.n_ghost = 0;
        }
        CU(merge_positions(c, lf.x, lf.y, lf.z, lf.vs, lf.h, n));
        u32 N = n + c.n_ghost;
        CU(bbox_from_merged(c, N));
        CU(tree_build(c, c.mx.as<f64>(), c.my.as<f64>(), c.mz.as<f64>(), c.mh.as<f64>(), N,
                      cfg->tree_reduction_level, cfg->htol_up_coarse, 32, 0, true));
        CU(build_rows(c, n));
        // both precisions pre-test the pairs in FP32 (exact FP64 test inside the rounding
        // band): the cache is the FP64 one either way
        CU(stage_positions_mixed(c, N, cfg->htol_up_coarse));
        CU(neigh_cache_build(c, cfg->htol_up_coarse, mixed_positions(c)));
        rs = RowSpace{n,                  c.row_rank.as<u32>(), c.row_local.as<u32>(),
                      c.csr_cnt.as<u32>(), c.csr_off.as<u32>(), c.csr_ent.as<u32>(),
                      c.sx.as<f64>(),      c.sy.as<f64>(),      c.sz.as<f64>()};
        CU(gather_rows(c, n, c.sh.as<f64>(), c.h_old_row.as<f64>(), c.hnew_row.as<f64>()));
        CU(fill64(c, n, c.eps_row.as<f64>(), 100.0));
        u32 iters_total = 0;
        if (fused_h) {
            { k_reset_eps<<<1, 1, 0, s>>>(dsc); GBSPH_COUNTED; }
            if (mixed)
                CU(h_iterate_mixed(c, rs, c.h_old_row.as<f64>(), c.hnew_row.as<f64>(),
                                   c.eps_row.as<f64>(), cfg->pmass, cfg->htol_up_coarse,
                                   cfg->htol_up_fine, cfg->h_iter_per_subcycles, eps_p));
            else
                CU(h_iterate64(c, rs, c.h_old_row.as<f64>(), c.hnew_row.as<f64>(),
                               c.eps_row.as<f64>(), cfg->pmass, cfg->htol_up_coarse,
                               cfg->htol_up_fine, cfg->h_iter_per_subcycles, eps_p));
            CU(sync_scalars(c));
            max_eps     = ordered_to_f64(c.h_scalars->eps_max);
            min_eps     = ordered_to_f64(c.h_scalars->eps_min);
            iters_total = c.h_scalars->iters_max;
        } else {
            for (u32 it = 0; it < cfg->h_iter_per_subcycles; it++) {
                { k_reset_eps<<<1, 1, 0, s>>>(dsc); GBSPH_COUNTED; }
                if (mixed)
                    CU(h_iterate_mixed(c, rs, c.h_old_row.as<f64>(), c.hnew_row.as<f64>(),
                                       c.eps_row.as<f64>(), cfg->pmass, cfg->htol_up_coarse,
                                       cfg->htol_up_fine, 1, eps_p));
                else
                    CU(h_iterate64(c, rs, c.h_old_row.as<f64>(), c.hnew_row.as<f64>(),
                                   c.eps_row.as<f64>(), cfg->pmass, cfg->htol_up_coarse,
                                   cfg->htol_up_fine, 1, eps_p));
                CU(sync_scalars(c));
                max_eps = ordered_to_f64(c.h_scalars->eps_max);
                min_eps = ordered_to_f64(c.h_scalars->eps_min);
                iters_total++;
                if (max_eps < cfg->epsilon_h) break;
            }
        }
        lg.h_iterations += iters_total;
        // the iterated h is written back whether or not the sub-cycle converged
        CU(scatter_rows(c, n, c.hnew_row.as<f64>(), lf.h));
        converged = (max_eps < cfg->epsilon_h) && !(min_eps < 0);
        if (converged) break;
    }
    // hstep + 1 sub-cycles ran; h_max_subcycles + 1 flags "never converged", after which
    // the reference logs an error and carries on with the step (Solver.cpp:1271-1273)
    lg.h_subcycles = hstep + 1;
    lg.max_eps_h   = max_eps;
    lg.n_ghost     = c.n_ghost;
    lg.leaf_count  = c.leaf_count;
    lg.cache_size  = c.csr_total;
    u32 N          = n + c.n_ghost;
    if (comp) {
        // compensated tier: h finished by one double-float Newton step, Omega at it
        CU(dens_polish_df(c, rs, c.h_old_row.as<f64>(), c.hnew_row.as<f64>(), c.eps_row.as<f64>(),
                          cfg->htol_up_coarse, cfg->htol_up_fine, c.omega_local.as<f64>()));
        CU(scatter_rows(c, n, c.hnew_row.as<f64>(), lf.h));
    } else if (mixed) {
        CU(omega_compact_mixed(c, rs, N, n, lf.h, c.hnew_row.as<f64>(), c.omega_local.as<f64>()));
    } else {
        CU(omega64(c, rs, c.hnew_row.as<f64>(), cfg->pmass, c.omega_local.as<f64>(),
                   c.row_local.as<u32>()));
    }
    if (p->omega)
        CU(cudaMemcpyAsync(p->omega, c.omega_local.p, 8 * (size_t) n, cudaMemcpyDeviceToDevice, s));

    // ---- corrector loop (Solver.cpp:2247-3171)
    // FP64 rank-ordered hydro copies (the mixed path stages 32-byte records and keeps
    // only h in FP64)
    DevBuf *rank_bufs[] = {&c.sh2, &c.su,  &c.svx,  &c.svy, &c.svz, &c.som,
                           &c.sP,  &c.scs, &c.srho, &c.sinv, &c.srom};
    for (DevBuf *b : rank_bufs) {
        CU(b->ensure(8 * (size_t) N, s));
        if (mixed) break;
    }
    if (tape) {
        CU(tape->snap->ensure(sizeof(f64) * 4 * (size_t) n * tape->forced_iters, s));
        if (cd10) CU(tape->snap_av->ensure(sizeof(f64) * 4 * (size_t) n * tape->forced_iters, s));
        if (cd10 && mixed && tape->snap_vg)
            CU(tape->snap_vg->ensure(sizeof(float) * 24 * (size_t) n * tape->forced_iters, s));
        tape->iters = 0;
    }
    HydroSpace hs{c.sh2.as<f64>(), c.su.as<f64>(),  c.svx.as<f64>(), c.svy.as<f64>(),
                  c.svz.as<f64>(), c.som.as<f64>(), c.sP.as<f64>(),  c.scs.as<f64>()};
    if (!mixed) {
        hs.rho    = c.srho.as<f64>();
        hs.inv_sub = c.sinv.as<f64>();
        hs.rho_om = c.srom.as<f64>();
    }
    f64 next_cfl   = 0;
    bool rerun     = false;
    u32 corr_iters = 0;
    const u32 corr_cap = cfg->corrector_max_iters ? cfg->corrector_max_iters : 50;
    do {
        if (corr_iters == corr_cap)
            return fail(ctx, GBSPH_ERR_NOT_CONVERGED,
                        "the corrector has made over " + std::to_string(corr_cap) +
                            " loops, either their is a bug, either you are using a dt that is "
                            "too large");
        if (mixed)
            CU(gather_stage_mixed(c, N, n, lf, c.omega_local.as<f64>(), cfg->pmass, eos, cd10, comp));
        else CU(gather_eos64(c, N, n, lf, c.omega_local.as<f64>(), cfg->pmass, eos));
        hs.alpha = nullptr;
        if (cd10) {
            // varying viscosity (Solver.cpp:2261-2370): div v, curl v and d(div v)/dt from
            // the current velocities and the accelerations of the last evaluation, the
            // switch update from alpha_AV and the stored sound speed, alpha on the ghosts.
            // (EOS values do not enter these, so staging them first changes nothing.)
            CU(c.av_diag.ensure(sizeof(f64) * 5 * (size_t) n, s));
            CU(c.av_alpha_upd.ensure(sizeof(f64) * (size_t) n, s));
            f64 *diag = c.av_diag.as<f64>();
            f64 *divv = p->divv ? p->divv : diag;
            f64 *dtdv = p->dtdivv ? p->dtdivv : diag + n;
            f64 *cx = p->curlv.x, *cy = p->curlv.y, *cz = p->curlv.z;
            u32 cvs = p->curlv.stride;
            if (!cx) {
                cx  = diag + 2 * (size_t) n;
                cy  = diag + 3 * (size_t) n;
                cz  = diag + 4 * (size_t) n;
                cvs = 1;
            }
            f64 *alpha_upd = c.av_alpha_upd.as<f64>();
            if (mixed) {
                float *vg_sums = (tape && tape->snap_vg)
                                     ? tape->snap_vg->as<float>() + (size_t) corr_iters * 24 * n
                                     : nullptr;
                CU(velgrad_mixed(c, rs, c.omega_local.as<f64>(), cfg->pmass, divv, cx, cy, cz, cvs,
                                 dtdv, vg_sums));
                if (vg_sums) tape->vg_recorded = true;
            } else {
                CU(c.av_arank.ensure(sizeof(f64) * 3 * (size_t) N, s));
                f64 *ar = c.av_arank.as<f64>();
                CU(gather_merged64(c, N, n, lf.ax, lf.vs, ar));
                CU(gather_merged64(c, N, n, lf.ay, lf.vs, ar + N));
                CU(gather_merged64(c, N, n, lf.az, lf.vs, ar + 2 * (size_t) N));
                CU(velgrad64(c, rs, hs, ar, ar + N, ar + 2 * (size_t) N, cfg->pmass, divv, cx, cy,
                             cz, cvs, dtdv));
            }
            if (cfg->av_kind == GBSPH_AV_VARYING_CD10)
                CU(cd10_update(c, n, divv, cx, cy, cz, cvs, dtdv, p->soundspeed, lf.h, p->alpha_AV,
                               dt, cfg->sigma_decay, cfg->alpha_min, cfg->alpha_max, alpha_upd,
                               mixed));
            else
                CU(mm97_update(c, n, divv, p->soundspeed, lf.h, p->alpha_AV, dt, cfg->sigma_decay,
                               cfg->alpha_min, cfg->alpha_max, alpha_upd, mixed));
            if (mixed) {
                CU(stage_alpha_mixed(c, N, n, alpha_upd));
            } else {
                CU(c.av_alpha_rank.ensure(sizeof(f64) * (size_t) N, s));
                CU(gather_merged64(c, N, n, alpha_upd, 1, c.av_alpha_rank.as<f64>()));
                hs.alpha = c.av_alpha_rank.as<f64>();
            }
        }
        if (tape) {
            { k_snap_vu<<<div_up(n, 256), 256, 0, s>>>(
                n, lf.vx, lf.vy, lf.vz, lf.vs, lf.u,
                tape->snap->as<f64>() + (size_t) corr_iters * 4 * n); GBSPH_COUNTED; }
            if (cd10) {
                // the velocity gradients' accelerations (the previous evaluation's) and this
                // evaluation's switched alpha
                { k_snap_vu<<<div_up(n, 256), 256, 0, s>>>(
                    n, lf.ax, lf.ay, lf.az, lf.vs, c.av_alpha_upd.as<f64>(),
                    tape->snap_av->as<f64>() + (size_t) corr_iters * 4 * n); GBSPH_COUNTED; }
            }
            tape->iters = corr_iters + 1;
        }
        { k_reset_corrector<<<1, 1, 0, s>>>(dsc); GBSPH_COUNTED; }
        f64 C_cour  = cfg->cfl_cour * ts->cfl_mult;
        f64 C_force = cfg->cfl_force * ts->cfl_mult;
        // the error estimate of the mixed tiers comes from the step's first evaluation
        // the condition sums feed the error estimate; the adjoint's recomputation of a
        // recorded step (tape) has no use for them
        const bool cond = corr_iters == 0 && c.cond_this_step && !tape;
        if (comp)
            CU(derivs_step_comp(c, rs, cfg->pmass, cfg->alpha_u, cfg->alpha_AV, cfg->beta_AV,
                                dt / 2, C_cour, C_force, lf, ext, cd10, cond));
        else if (mixed)
            CU(derivs_step_mixed(c, rs, cfg->pmass, cfg->alpha_u, cfg->alpha_AV, cfg->beta_AV,
                                 dt / 2, C_cour, C_force, lf, ext, cd10, cond));
        else
            CU(derivs_step64(c, rs, hs, cfg->pmass, cfg->alpha_u, cfg->alpha_AV, cfg->beta_AV,
                             dt / 2, C_cour, C_force, lf, ext));
        CU(sync_scalars(c));
        f64 rank_veps_v = std::sqrt(ordered_to_f64(c.h_scalars->epsv2_max));
        f64 vmean       = std::sqrt(c.h_scalars->sum_v2 / f64(n));
        f64 eps_v       = rank_veps_v / vmean;
        if (vmean <= 0) eps_v = 0;
        lg.eps_v = eps_v;
        if (tape) {
            rerun    = corr_iters + 1 < tape->forced_iters;
            next_cfl = ordered_to_f64(c.h_scalars->dt_min);
        } else if (eps_v > 1e-2) {
            rerun        = true;
            ts->cfl_mult = ts->cfl_mult / 2;
        } else {
            rerun    = false;
            next_cfl = ordered_to_f64(c.h_scalars->dt_min);
        }
        if (cd10 && !rerun) {
            // write back alpha_AV and the sound speed of this evaluation
            // (Solver.cpp:2620-2650, 3125-3160)
            CU(cudaMemcpyAsync(p->alpha_AV, c.av_alpha_upd.p, sizeof(f64) * (size_t) n,
                               cudaMemcpyDeviceToDevice, s));
            if (mixed) CU(cs_to_local_mixed(c, n, p->soundspeed));
            else CU(rank_to_local64(c, n, c.scs.as<f64>(), p->soundspeed));
        }
        corr_iters++;
    } while (rerun);
    if (c.h_scalars->flags & (kFlagStackOverflow | kFlagOwnerMissing | kFlagCsrOverflow))
        return fail(ctx, GBSPH_ERR_CUDA, "kernel error flags raised during the step");

    auto t_end    = std::chrono::steady_clock::now();
    f64 elapsed   = std::chrono::duration<f64>(t_end - t_start).count();
    lg.corrector_iters = corr_iters;
    ts->dt             = next_cfl;
    ts->t              = ts->t + dt;
    f64 stiff          = cfg->cfl_mult_stiffness;
    ts->cfl_mult       = (ts->cfl_mult * stiff + 1.) / (stiff + 1.);
    lg.next_dt         = ts->dt;
    lg.cfl_mult        = ts->cfl_mult;
    lg.elapsed_s       = elapsed;
    lg.rate            = elapsed > 0 ? f64(n) / elapsed : 0;
    lg.tier            = tier;
    lg.cache_kept      = (mixed && !comp) ? c.h_scalars->csr_kept : lg.cache_size;
    lg.est_refreshed   = (c.cond_this_step && !tape) ? 1 : 0;
    if (mixed && c.cond_this_step && !tape) {
        lg.err_est_a  = err_estimate(c.h_scalars->cond_fa, c.h_scalars->cond_a);
        lg.err_est_du = err_estimate(c.h_scalars->cond_fu, c.h_scalars->cond_du);
    } else if (mixed) {
        lg.err_est_a  = c.guard_est_a; // the last refreshed estimate
        lg.err_est_du = c.guard_est_du;
    }
    if (log) *log = lg;
    if (!converged) ctx->c.err = "the h iterator is not converged after the maximum number of "
                                 "sub-cycles (step continued, as the reference does)";
    return GBSPH_OK;
}

// Start state of a step that may be recomputed: the caller's x, v, a, h, u, du (and the
// varying viscosity's alpha_AV and sound speed), SoA in c.guard_state.
static int save_state(gbsph_ctx *ctx, const gbsph_particles *p, bool av) {
    Ctx &c = ctx->c;
    const u32 n = p->n;
    const size_t n_ = n;
    CU(c.guard_state.ensure(sizeof(f64) * 14 * n_, c.stream));
    f64 *S = c.guard_state.as<f64>();
    { k_copy_state<<<div_up(n, 256), 256, 0, c.stream>>>(n, p->xyz, p->vxyz, p->axyz, p->hpart,
                                                       p->uint, p->duint, S); GBSPH_COUNTED; }
    CU(cudaGetLastError());
    if (av) {
        CU(cudaMemcpyAsync(S + 12 * n_, p->alpha_AV, 8 * n_, cudaMemcpyDeviceToDevice, c.stream));
        CU(cudaMemcpyAsync(S + 13 * n_, p->soundspeed, 8 * n_, cudaMemcpyDeviceToDevice, c.stream));
    }
    return GBSPH_OK;
}

static int restore_state(gbsph_ctx *ctx, const gbsph_particles *p, bool av) {
    Ctx &c = ctx->c;
    const u32 n = p->n;
    const size_t n_ = n;
    const f64 *S = c.guard_state.as<f64>();
    { k_restore_state<<<div_up(n, 256), 256, 0, c.stream>>>(n, p->xyz, p->vxyz, p->axyz, p->hpart,
                                                          p->uint, p->duint, S); GBSPH_COUNTED; }
    CU(cudaGetLastError());
    if (av) {
        CU(cudaMemcpyAsync(p->alpha_AV, S + 12 * n_, 8 * n_, cudaMemcpyDeviceToDevice, c.stream));
        CU(cudaMemcpyAsync(p->soundspeed, S + 13 * n_, 8 * n_, cudaMemcpyDeviceToDevice, c.stream));
    }
    return GBSPH_OK;
}

// One step in the configured precision; GBSPH_MIXED_GUARDED picks the tier (see gbsph.h).
static int evolve_impl(gbsph_ctx *ctx, const gbsph_particles *p, const gbsph_config *cfg,
                       gbsph_time_state *ts, gbsph_step_log *log, StepTape *tape) {
    REQUIRE_ARG(p && cfg && ts, "null argument");
    if (cfg->precision != GBSPH_MIXED_GUARDED)
        return evolve_tier(ctx, p, cfg, ts, log, tape, cfg->precision);
    REQUIRE_ARG(!tape, "the adjoint step recomputes the forward step in the tier it ran in "
                       "(gbsph_step_log.tier), not in GBSPH_MIXED_GUARDED");
    REQUIRE_ARG(p->n > 0, "empty patch");
    Ctx &c = ctx->c;
    if (p->xyz.x != c.guard_of || p->n != c.guard_n) {
        // other particle arrays: their estimate starts afresh, in the FP32 tier
        c.guard_of = p->xyz.x, c.guard_n = p->n;
        c.guard_tier = GBSPH_MIXED, c.guard_skip = 0, c.guard_prev_est = -1, c.guard_since = 0;
    }
    auto t0        = std::chrono::steady_clock::now();
    const f64 tol  = cfg->mixed_tol > 0 ? cfg->mixed_tol : 1e-5;
    const bool av  = cfg->av_kind != GBSPH_AV_CONSTANT && p->alpha_AV && p->soundspeed;
    u32 tier       = c.guard_tier == GBSPH_MIXED_COMPENSATED ? GBSPH_MIXED_COMPENSATED : GBSPH_MIXED;
    const gbsph_time_state ts0 = *ts;
    // The estimate is refreshed on every fourth step when it cannot reach the tolerance in
    // the three steps between: when it is below an eighth of the tolerance, or below 0.8 of
    // it and, grown at twice its rate between the last two refreshes, stays there for four
    // steps (the condition sums follow the pressure and velocity fields, which a CFL step
    // changes by a fraction; and the sums cost their evaluation about a third more time).
    // Otherwise, and after any step that ran compensated, on every step.
    const bool refresh = c.guard_skip == 0;
    c.cond_this_step   = refresh;
    if (tier == GBSPH_MIXED && refresh) {
        int st = save_state(ctx, p, av);
        if (st != GBSPH_OK) return st;
    }
    gbsph_step_log lg;
    std::memset(&lg, 0, sizeof(lg));
    int st = evolve_tier(ctx, p, cfg, ts, &lg, nullptr, tier);
    c.cond_this_step = true;
    if (st != GBSPH_OK) return st;
    f64 est = std::max(lg.err_est_a, lg.err_est_du);
    u32 reruns = 0;
    if (tier == GBSPH_MIXED && refresh && !(est <= tol)) {
        // the FP32 tier cannot be trusted with this state: redo the step compensated
        st = restore_state(ctx, p, av);
        if (st != GBSPH_OK) return st;
        *ts = ts0;
        st = evolve_tier(ctx, p, cfg, ts, &lg, nullptr, GBSPH_MIXED_COMPENSATED);
        if (st != GBSPH_OK) return st;
        reruns = 1;
        tier   = GBSPH_MIXED_COMPENSATED;
        est    = std::max(lg.err_est_a, lg.err_est_du);
    }
    // the next step starts in the tier this one needed, and returns to FP32 once the
    // estimate is well inside the tolerance
    c.guard_tier    = (tier == GBSPH_MIXED_COMPENSATED && !(est <= tol / 4)) ? GBSPH_MIXED_COMPENSATED
                                                                            : GBSPH_MIXED;
    c.guard_since++;
    if (refresh) {
        c.guard_est_a  = lg.err_est_a;
        c.guard_est_du = lg.err_est_du;
        c.guard_skip     = guard_refresh_skip(est, c.guard_prev_est, c.guard_since, tol,
                                              tier == GBSPH_MIXED);
        c.guard_prev_est = tier == GBSPH_MIXED ? est : -1;
        c.guard_since    = 0;
    } else {
        c.guard_skip--;
    }
    lg.est_refreshed = refresh ? 1 : 0;
    lg.tier_reruns  = reruns;
    lg.elapsed_s    = std::chrono::duration<f64>(std::chrono::steady_clock::now() - t0).count();
    lg.rate         = lg.elapsed_s > 0 ? f64(p->n) / lg.elapsed_s : 0;
    if (log) *log = lg;
    return GBSPH_OK;
}

extern "C" {

int gbsph_evolve_once(gbsph_ctx *ctx, const gbsph_particles *p, const gbsph_config *cfg,
                      gbsph_time_state *ts, gbsph_step_log *log, void *stream) {
    ENTER(ctx, stream);
    return evolve_impl(ctx, p, cfg, ts, log, nullptr);
}

int gbsph_adjoint_record(gbsph_ctx *ctx, const gbsph_particles *start, const gbsph_config *cfg,
                         double t, double dt, uint32_t corrector_iters, gbsph_particles *after,
                         void *stream) {
    ENTER(ctx, stream);
    Ctx &c = ctx->c;
    ctx->adj_ready = false;
    REQUIRE_ARG(start && cfg, "null argument");
    REQUIRE_ARG(start->n > 0, "empty patch");
    REQUIRE_ARG(corrector_iters >= 1 && corrector_iters <= kTapeMaxIters,
                "corrector_iters must be the forward step's count (1..16)");
    REQUIRE_ARG(dt >= 0, "dt must be the forward step's dt");
    REQUIRE_ARG(cfg->eos_kind == GBSPH_EOS_ADIABATIC || cfg->eos_kind == GBSPH_EOS_LOCALLY_ISOTHERMAL_LP07,
                "unknown equation of state");
    REQUIRE_ARG((cfg->eos_kind == GBSPH_EOS_ADIABATIC && cfg->ext_kind == GBSPH_EXT_NONE) ||
                    !cfg->periodic,
                "the adjoint of the locally isothermal EOS or the point mass needs free "
                "boundaries (a periodic image's pressure depends on its shifted position)");
    const bool var = cfg->av_kind != GBSPH_AV_CONSTANT;
    REQUIRE_ARG(!var || (start->alpha_AV && start->soundspeed),
                "the varying viscosity's adjoint needs alpha_AV and soundspeed in the start state");
    REQUIRE_ARG(cfg->precision != GBSPH_MIXED_GUARDED,
                "give the adjoint step the tier the forward step ran in (gbsph_step_log.tier)");
    cudaStream_t s = c.stream;
    const u32 n    = start->n;
    // recompute the step on a working copy of the start state
    CU(c.adj_state.ensure(sizeof(f64) * 14 * (size_t) n, s));
    f64 *W = c.adj_state.as<f64>();
    size_t n_ = n;
    { k_copy_state<<<div_up(n, 256), 256, 0, s>>>(n, start->xyz, start->vxyz, start->axyz,
                                                start->hpart, start->uint, start->duint, W); GBSPH_COUNTED; }
    CU(cudaGetLastError());
    if (var) {
        CU(cudaMemcpyAsync(W + 12 * n_, start->alpha_AV, 8 * n_, cudaMemcpyDeviceToDevice, s));
        CU(cudaMemcpyAsync(W + 13 * n_, start->soundspeed, 8 * n_, cudaMemcpyDeviceToDevice, s));
    }
    gbsph_particles w;
    std::memset(&w, 0, sizeof(w));
    w.n     = n;
    w.xyz   = gbsph_vec3{W, W + n_, W + 2 * n_, 1, 0};
    w.vxyz  = gbsph_vec3{W + 3 * n_, W + 4 * n_, W + 5 * n_, 1, 0};
    w.axyz  = gbsph_vec3{W + 6 * n_, W + 7 * n_, W + 8 * n_, 1, 0};
    w.hpart = W + 9 * n_;
    w.uint  = W + 10 * n_;
    w.duint = W + 11 * n_;
    if (var) {
        w.alpha_AV   = W + 12 * n_;
        w.soundspeed = W + 13 * n_;
    }
    gbsph_time_state ts{t, dt, 1.0};
    StepTape &tape = ctx->adj_tape;
    tape           = StepTape{};
    tape.forced_iters = corrector_iters;
    tape.snap         = &c.adj_snap;
    tape.snap_av      = &c.adj_snap_av;
    tape.snap_vg      = &c.adj_snap_vg;
    int st = evolve_impl(ctx, &w, cfg, &ts, nullptr, &tape);
    if (st != GBSPH_OK) return st;
    ctx->adj_after = w;
    ctx->adj_ready = true;
    ctx->adj_var   = var;
    ctx->adj_n     = n;
    ctx->adj_prec  = cfg->precision;
    ctx->adj_dt    = dt;
    if (after) *after = w;
    return GBSPH_OK;
}

int gbsph_adjoint_reverse(gbsph_ctx *ctx, const gbsph_particles *start, const gbsph_config *cfg,
                          double dt, gbsph_cotangents *cot, double *g_alpha_av, void *stream) {
    ENTER(ctx, stream);
    Ctx &c = ctx->c;
    REQUIRE_ARG(start && cfg && cot, "null argument");
    if (!ctx->adj_ready)
        return fail(ctx, GBSPH_ERR_STATE, "gbsph_adjoint_reverse needs the step recorded by "
                                          "gbsph_adjoint_record on this context");
    REQUIRE_ARG(start->n == ctx->adj_n && cot->n == start->n, "cotangents and state differ in size");
    REQUIRE_ARG(cfg->precision == ctx->adj_prec && dt == ctx->adj_dt,
                "the reverse must use the recorded step's precision and dt");
    REQUIRE_ARG(cot->gx.stride == cot->gv.stride && cot->gx.stride == cot->ga.stride,
                "gx, gv and ga must share one element stride");
    const bool var = ctx->adj_var;
    REQUIRE_ARG(!var || (start->alpha_AV && start->soundspeed && cot->galpha && cot->gsoundspeed),
                "the varying viscosity's adjoint needs alpha_AV and soundspeed in the start state "
                "and galpha and gsoundspeed in the cotangents");
    cudaStream_t s = c.stream;
    const u32 n    = start->n;
    const gbsph_particles &w = ctx->adj_after;
    RowSpace rs{n,                  c.row_rank.as<u32>(), c.row_local.as<u32>(),
                c.csr_cnt.as<u32>(), c.csr_off.as<u32>(), c.csr_ent.as<u32>(),
                c.sx.as<f64>(),      c.sy.as<f64>(),      c.sz.as<f64>()};
    AdjParams ap{cfg->pmass, cfg->gamma, cfg->alpha_u, cfg->alpha_AV, cfg->beta_AV, dt,
                 cfg->eos_kind, cfg->cs0, cfg->eos_r0 > 0 ? cfg->eos_r0 : 1.0, cfg->eos_q,
                 -cfg->central_mass * cfg->constant_G, nullptr, nullptr, nullptr,
                 cfg->av_kind, cfg->alpha_min, cfg->alpha_max, cfg->sigma_decay,
                 var ? start->alpha_AV : nullptr, var ? start->soundspeed : nullptr,
                 w.xyz.x, w.xyz.y, w.xyz.z};
    if (cfg->ext_kind == GBSPH_EXT_POINT_MASS) {
        ap.ext_x = w.xyz.x;
        ap.ext_y = w.xyz.y;
        ap.ext_z = w.xyz.z;
    }
    CotState cs;
    cs.x[0] = cot->gx.x; cs.x[1] = cot->gx.y; cs.x[2] = cot->gx.z;
    cs.v[0] = cot->gv.x; cs.v[1] = cot->gv.y; cs.v[2] = cot->gv.z;
    cs.a[0] = cot->ga.x; cs.a[1] = cot->ga.y; cs.a[2] = cot->ga.z;
    cs.u    = cot->gu;
    cs.du   = cot->gdu;
    cs.vs   = cot->gx.stride;
    cs.alpha = var ? cot->galpha : nullptr;
    cs.cs    = var ? cot->gsoundspeed : nullptr;
    Scalars *dsc = c.d_scalars.as<Scalars>();
    CU(cudaMemsetAsync(&dsc->g_alpha, 0, sizeof(f64), s));
    CU(cudaMemsetAsync(dsc->g_av, 0, 3 * sizeof(f64), s));
    // FP32 reverse pass after either mixed tier's recompute, FP64 after the FP64 one
    CU(adjoint_backward(c, rs, n, w.hpart, c.omega_local.as<f64>(), ctx->adj_tape, ap, cs,
                        &dsc->g_alpha, dsc->g_av, cfg->precision != GBSPH_FP64));
    CU(sync_scalars(c));
    ctx->adj_ready = false;
    if (g_alpha_av) *g_alpha_av += c.h_scalars->g_alpha;
    if (var) {
        cot->g_alpha_min += c.h_scalars->g_av[0];
        cot->g_alpha_max += c.h_scalars->g_av[1];
        cot->g_sigma_decay += c.h_scalars->g_av[2];
    }
    return GBSPH_OK;
}

int gbsph_adjoint_step(gbsph_ctx *ctx, const gbsph_particles *start, const gbsph_config *cfg,
                       double t, double dt, uint32_t corrector_iters, gbsph_cotangents *cot,
                       double *g_alpha_av, void *stream) {
    if (ctx && cot && start && cot->n != start->n)
        return fail(ctx, GBSPH_ERR_ARG, "cotangents and state differ in size");
    int st = gbsph_adjoint_record(ctx, start, cfg, t, dt, corrector_iters, nullptr, stream);
    if (st != GBSPH_OK) return st;
    return gbsph_adjoint_reverse(ctx, start, cfg, dt, cot, g_alpha_av, stream);
}

} // extern "C"
