// Periodic ghost layer for one patch covering the simulation box —
//   interface search shammodels/sph/src/BasicSPHGhosts.cpp:260-360 (offsets in x-outer,
//   z-inner order, the zero offset skipped), interaction range
//   shammodels/sph/include/shammodels/sph/SPHUtilities.hpp:79-95 (max h * htol * Rkern),
//   selection by half-open box shamrock/include/shamrock/patch/Patch.hpp:210-215 in
//   particle order (BasicSPHGhosts.cpp:512-530), ghosts appended after the locals in
//   interface order (shammodels/sph/include/shammodels/sph/BasicSPHGhosts.hpp:452-517).
//
// Per axis the interface interval depends only on that axis' offset, so each
// particle classifies itself once per axis (3 x 3 tests) and the 26 memberships are
// products of those.  Ghost slots are assigned by an order-preserving multi-list
// compaction: per-block counts per interface, a scan per interface, then a scatter
// that uses warp ballots for the in-block order.

#include "gbsph_ctx.cuh"

namespace gbsph {

namespace {

constexpr int kGhostThreads = 256;
constexpr int kNoff         = 26;

struct GhostTable {
    f64 lo[3][3]; // [axis][offset+1]
    f64 hi[3][3];
    f64 off[kNoff][3];
    i32 o[kNoff][3];
};

__global__ void k_hmax(const f64 *__restrict__ h, u32 n, Scalars *sc) {
    u64 m = 0;
    for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        u64 o = f64_to_ordered(h[i]);
        m     = o > m ? o : m;
    }
    m = block_reduce(m, OpMaxU64{}, 0ull);
    if (threadIdx.x == 0) atomicMax((unsigned long long *) &sc->hmax, (unsigned long long) m);
}

__global__ void k_ghost_table(const Scalars *sc, f64 htol, f64 b0, f64 b1, f64 b2, f64 e0, f64 e1,
                              f64 e2, GhostTable *tab) {
    if (threadIdx.x != 0) return;
    f64 bmin[3] = {b0, b1, b2}, bmax[3] = {e0, e1, e2};
    f64 hmax = ordered_to_f64(sc->hmax);
    f64 R    = __dmul_rn(__dmul_rn(hmax, htol), kRkern);
    f64 bsize[3];
    for (int c = 0; c < 3; c++) bsize[c] = __dsub_rn(bmax[c], bmin[c]);
    for (int c = 0; c < 3; c++)
        for (int o = -1; o <= 1; o++) {
            f64 off  = __dmul_rn((f64) o, bsize[c]);
            f64 rlo  = __dadd_rn(__dsub_rn(bmin[c], R), -off);
            f64 rhi  = __dadd_rn(__dadd_rn(bmax[c], R), -off);
            tab->lo[c][o + 1] = fmax(bmin[c], rlo);
            tab->hi[c][o + 1] = fmin(bmax[c], rhi);
        }
    int k = 0;
    for (int xo = -1; xo <= 1; xo++)
        for (int yo = -1; yo <= 1; yo++)
            for (int zo = -1; zo <= 1; zo++) {
                if (xo == 0 && yo == 0 && zo == 0) continue;
                int oo[3] = {xo, yo, zo};
                for (int c = 0; c < 3; c++) {
                    tab->off[k][c] = __dmul_rn((f64) oo[c], bsize[c]);
                    tab->o[k][c]   = oo[c];
                }
                k++;
            }
}

// bit k set iff the particle lies in interface k
__device__ __forceinline__ u32 ghost_mask(const GhostTable &t, const f64 p[3]) {
    u32 ax[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
        u32 m = 0;
#pragma unroll
        for (int o = 0; o < 3; o++)
            m |= ((t.lo[c][o] <= p[c]) && (p[c] < t.hi[c][o])) ? (1u << o) : 0u;
        ax[c] = m;
    }
    u32 mask = 0;
    int k    = 0;
#pragma unroll
    for (int xo = 0; xo < 3; xo++)
#pragma unroll
        for (int yo = 0; yo < 3; yo++)
#pragma unroll
            for (int zo = 0; zo < 3; zo++) {
                if (xo == 1 && yo == 1 && zo == 1) continue;
                bool in = ((ax[0] >> xo) & 1) && ((ax[1] >> yo) & 1) && ((ax[2] >> zo) & 1);
                mask |= in ? (1u << k) : 0u;
                k++;
            }
    return mask;
}

__global__ void __launch_bounds__(kGhostThreads) k_ghost_count(
    const f64 *__restrict__ x, const f64 *__restrict__ y, const f64 *__restrict__ z, u32 vs, u32 n,
    const GhostTable *__restrict__ tab, u32 nblocks, u32 *__restrict__ block_counts) {
    __shared__ GhostTable t;
    __shared__ u32 cnt[kNoff];
    if (threadIdx.x == 0) t = *tab;
    if (threadIdx.x < kNoff) cnt[threadIdx.x] = 0;
    __syncthreads();
    u32 i    = blockIdx.x * blockDim.x + threadIdx.x;
    u32 mask = 0;
    if (i < n) {
        f64 p[3] = {x[(size_t) i * vs], y[(size_t) i * vs], z[(size_t) i * vs]};
        mask     = ghost_mask(t, p);
    }
    int lane = threadIdx.x & 31;
    for (int k = 0; k < kNoff; k++) {
        u32 b = __ballot_sync(0xffffffffu, (mask >> k) & 1u);
        if (lane == 0 && b) atomicAdd(&cnt[k], (u32) __popc(b));
    }
    __syncthreads();
    if (threadIdx.x < kNoff) block_counts[threadIdx.x * nblocks + blockIdx.x] = cnt[threadIdx.x];
}

// one block per interface: exclusive scan of its block counts in place; totals out
__global__ void k_ghost_scan(u32 *__restrict__ block_counts, u32 nblocks, u32 *__restrict__ totals) {
    u32 *bc = block_counts + blockIdx.x * nblocks;
    __shared__ u32 carry_s;
    __shared__ u32 warp_tot[32];
    if (threadIdx.x == 0) carry_s = 0;
    __syncthreads();
    for (u32 base = 0; base < nblocks; base += blockDim.x) {
        u32 i = base + threadIdx.x;
        u32 v = (i < nblocks) ? bc[i] : 0;
        // block exclusive scan
        int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        u32 inc = v;
        for (int o = 1; o < 32; o <<= 1) {
            u32 t = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += t;
        }
        if (lane == 31) warp_tot[wid] = inc;
        __syncthreads();
        u32 wpre = 0, tot = 0;
        for (int w = 0; w < (int) (blockDim.x >> 5); w++) {
            if (w < wid) wpre += warp_tot[w];
            tot += warp_tot[w];
        }
        if (i < nblocks) bc[i] = carry_s + wpre + inc - v;
        __syncthreads();
        if (threadIdx.x == 0) carry_s += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) totals[blockIdx.x] = carry_s;
}

__global__ void k_ghost_bases(u32 *__restrict__ totals, Scalars *sc) {
    if (threadIdx.x != 0) return;
    u32 acc = 0;
    for (int k = 0; k < kNoff; k++) {
        u32 t     = totals[k];
        totals[k] = acc; // becomes the base of interface k
        acc += t;
    }
    sc->ghost_total = acc;
}

__global__ void __launch_bounds__(kGhostThreads) k_ghost_scatter(
    const f64 *__restrict__ x, const f64 *__restrict__ y, const f64 *__restrict__ z, u32 vs, u32 n,
    const GhostTable *__restrict__ tab, u32 nblocks, const u32 *__restrict__ block_offsets,
    const u32 *__restrict__ bases, u32 *__restrict__ ghost_src, u8 *__restrict__ ghost_oid) {
    __shared__ GhostTable t;
    __shared__ u32 wcnt[kNoff][kGhostThreads / 32];
    if (threadIdx.x == 0) t = *tab;
    __syncthreads();
    u32 i    = blockIdx.x * blockDim.x + threadIdx.x;
    u32 mask = 0;
    if (i < n) {
        f64 p[3] = {x[(size_t) i * vs], y[(size_t) i * vs], z[(size_t) i * vs]};
        mask     = ghost_mask(t, p);
    }
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    u32 lt   = (1u << lane) - 1u;
    u32 ballots[kNoff];
#pragma unroll
    for (int k = 0; k < kNoff; k++) {
        ballots[k] = __ballot_sync(0xffffffffu, (mask >> k) & 1u);
        if (lane == 0) wcnt[k][wid] = __popc(ballots[k]);
    }
    __syncthreads();
    if (!mask) return;
#pragma unroll
    for (int k = 0; k < kNoff; k++) {
        if ((mask >> k) & 1u) {
            u32 pre = 0;
            for (int w = 0; w < wid; w++) pre += wcnt[k][w];
            u32 pos = bases[k] + block_offsets[k * nblocks + blockIdx.x] + pre
                      + (u32) __popc(ballots[k] & lt);
            ghost_src[pos] = i;
            ghost_oid[pos] = (u8) k;
        }
    }
}

__global__ void k_merge(const f64 *__restrict__ x, const f64 *__restrict__ y,
                        const f64 *__restrict__ z, u32 vs, const f64 *__restrict__ h, u32 n, u32 G,
                        const u32 *__restrict__ ghost_src, const u8 *__restrict__ ghost_oid,
                        const GhostTable *__restrict__ tab, f64 *__restrict__ mx,
                        f64 *__restrict__ my, f64 *__restrict__ mz, f64 *__restrict__ mh) {
    u32 i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n + G) return;
    if (i < n) {
        mx[i] = x[(size_t) i * vs];
        my[i] = y[(size_t) i * vs];
        mz[i] = z[(size_t) i * vs];
        mh[i] = h[i];
    } else {
        u32 k   = i - n;
        u32 src = ghost_src[k];
        u32 o   = ghost_oid[k];
        mx[i]   = __dadd_rn(x[(size_t) src * vs], tab->off[o][0]);
        my[i]   = __dadd_rn(y[(size_t) src * vs], tab->off[o][1]);
        mz[i]   = __dadd_rn(z[(size_t) src * vs], tab->off[o][2]);
        mh[i]   = h[src];
    }
}

} // namespace

cudaError_t periodic_ghosts(Ctx &c, const f64 *x, const f64 *y, const f64 *z, u32 vs,
                            const f64 *h, u32 n, const f64 *bmin, const f64 *bmax, f64 htol) {
    cudaStream_t s = c.stream;
    cudaError_t e;
    Scalars *dsc = c.d_scalars.as<Scalars>();
    u32 nblocks  = div_up(n, kGhostThreads);
    if (nblocks == 0) nblocks = 1;
    if ((e = c.d_ghost_offsets.ensure(sizeof(GhostTable), s)) != cudaSuccess) return e;
    if ((e = c.ghost_block_counts.ensure(sizeof(u32) * ((size_t) kNoff * nblocks + kNoff), s)) !=
        cudaSuccess)
        return e;
    GhostTable *tab = c.d_ghost_offsets.as<GhostTable>();
    u32 *bc         = c.ghost_block_counts.as<u32>();
    u32 *totals     = bc + (size_t) kNoff * nblocks;
    if ((e = cudaMemsetAsync(&dsc->hmax, 0, sizeof(u64), s)) != cudaSuccess) return e;
    int pg = c.prof.on ? prof_begin(c, kProfGhosts, n) : -1;
    { k_hmax<<<nblocks < 1216 ? nblocks : 1216, 256, 0, s>>>(h, n, dsc); GBSPH_COUNTED; }
    { k_ghost_table<<<1, 32, 0, s>>>(dsc, htol, bmin[0], bmin[1], bmin[2], bmax[0], bmax[1], bmax[2],
                                   tab); GBSPH_COUNTED; }
    { k_ghost_count<<<nblocks, kGhostThreads, 0, s>>>(x, y, z, vs, n, tab, nblocks, bc); GBSPH_COUNTED; }
    { k_ghost_scan<<<kNoff, 1024, 0, s>>>(bc, nblocks, totals); GBSPH_COUNTED; }
    { k_ghost_bases<<<1, 32, 0, s>>>(totals, dsc); GBSPH_COUNTED; }
    if (pg >= 0) prof_end(c, pg);
    if ((e = sync_scalars(c)) != cudaSuccess) return e;
    ProfScope ps(c, kProfGhosts, 0);
    u32 G     = c.h_scalars->ghost_total;
    c.n_ghost = G;
    if ((e = c.ghost_src.ensure(sizeof(u32) * ((size_t) G + 1), s)) != cudaSuccess) return e;
    if ((e = c.ghost_oid.ensure((size_t) G + 1, s)) != cudaSuccess) return e;
    if (G)
        { k_ghost_scatter<<<nblocks, kGhostThreads, 0, s>>>(x, y, z, vs, n, tab, nblocks, bc, totals,
                                                          c.ghost_src.as<u32>(),
                                                          c.ghost_oid.as<u8>()); GBSPH_COUNTED; }
    return cudaGetLastError();
}

cudaError_t merge_positions(Ctx &c, const f64 *x, const f64 *y, const f64 *z, u32 vs,
                            const f64 *h, u32 n) {
    cudaStream_t s = c.stream;
    cudaError_t e;
    u32 N = n + c.n_ghost;
    if ((e = c.mx.ensure(sizeof(f64) * (size_t) N, s)) != cudaSuccess) return e;
    if ((e = c.my.ensure(sizeof(f64) * (size_t) N, s)) != cudaSuccess) return e;
    if ((e = c.mz.ensure(sizeof(f64) * (size_t) N, s)) != cudaSuccess) return e;
    if ((e = c.mh.ensure(sizeof(f64) * (size_t) N, s)) != cudaSuccess) return e;
    if ((e = c.d_ghost_offsets.ensure(sizeof(GhostTable), s)) != cudaSuccess) return e;
    ProfScope ps(c, kProfMerge, N);
    { k_merge<<<div_up(N, 256), 256, 0, s>>>(x, y, z, vs, h, n, c.n_ghost, c.ghost_src.as<u32>(),
                                           c.ghost_oid.as<u8>(), c.d_ghost_offsets.as<GhostTable>(),
                                           c.mx.as<f64>(), c.my.as<f64>(), c.mz.as<f64>(),
                                           c.mh.as<f64>()); GBSPH_COUNTED; }
    return cudaGetLastError();
}

} // namespace gbsph
