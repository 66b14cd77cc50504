// Compressed-leaf BVH build on the GPU: Morton keys, bitonic key/value sort, leaf
// reduction, Karras radix tree, leaf AABB / interaction radius and bottom-up union.
// Bit-exact with the reference semantics (see the oracle restatement):
//   Morton     shamtree/src/MortonCodeSet.cpp:63-118, shammath/sfc/morton.hpp:46-230
//   sort       shamalgs/src/details/algorithm/bitonicSort_updated_usm.cpp:26-396
//   reduction  shamtree/src/kernels/reduction_alg.cpp:62-85,196-244,274-295,413-456
//   Karras     shamtree/src/KarrasRadixTree.cpp:45-143
//   AABB/field shamtree/src/KarrasRadixTreeAABB.cpp:33-140,
//              shamtree/include/shamtree/KarrasRadixTreeField.hpp:134-222,
//              shammodels/sph/src/Solver.cpp:1322-1356
// The reference propagates node boxes with tree_depth full sweeps; here one
// bottom-up pass with arrival counters produces the same exact min/max.

#include "gbsph_ctx.cuh"

#include <type_traits>
#include <utility>

namespace gbsph {

namespace {

// ---------------------------------------------------------------- Morton
template<class K>
struct Morton;
template<>
struct Morton<u32> {
    static constexpr u32 val_count = 1024, max_val = 1023;
    static constexpr u32 err       = 0xFFFFFFFFu;
    __device__ static u32 expand(u32 x) {
        x &= 0x3ffU;
        x = (x | x << 16U) & 0x30000ffU;
        x = (x | x << 8U) & 0x300f00fU;
        x = (x | x << 4U) & 0x30c30c3U;
        x = (x | x << 2U) & 0x9249249U;
        return x;
    }
    __device__ static u32 encode(u32 x, u32 y, u32 z) { return expand(x) * 4 + expand(y) * 2 + expand(z); }
    __device__ static int clz(u32 v) { return __clz(v); }
};
template<>
struct Morton<u64> {
    static constexpr u32 val_count = 2097152, max_val = 2097151;
    static constexpr u64 err       = 0xFFFFFFFFFFFFFFFFull;
    __device__ static u64 expand(u64 x) {
        x &= 0x1fffffULL;
        x = (x | x << 32ULL) & 0x1f00000000ffffULL;
        x = (x | x << 16ULL) & 0x1f0000ff0000ffULL;
        x = (x | x << 8ULL) & 0x100f00f00f00f00fULL;
        x = (x | x << 4ULL) & 0x10c30c30c30c30c3ULL;
        x = (x | x << 2ULL) & 0x1249249249249249ULL;
        return x;
    }
    __device__ static u64 encode(u64 x, u64 y, u64 z) { return expand(x) * 4 + expand(y) * 2 + expand(z); }
    __device__ static int clz(u64 v) { return __clzll((long long) v); }
};

__global__ void k_bbox_fact(BBox *bb, u32 val_count) {
    if (threadIdx.x < 3) {
        int c       = threadIdx.x;
        bb->fact[c] = __ddiv_rn(__dsub_rn(bb->hi[c], bb->lo[c]), (f64) val_count);
    }
}

template<class K>
__global__ void k_morton(const f64 *__restrict__ x, const f64 *__restrict__ y,
                         const f64 *__restrict__ z, u32 n, u32 P, const BBox *__restrict__ bb,
                         K *__restrict__ keys, u32 *__restrict__ vals) {
    u32 i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    vals[i] = i;
    if (i >= n) {
        keys[i] = Morton<K>::err;
        return;
    }
    const f64 p[3] = {x[i], y[i], z[i]};
    u32 g[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
        f64 r = fmin(fmax(p[c], bb->lo[c]), bb->hi[c]);
        u32 gi = __double2uint_rz(__ddiv_rn(__dsub_rn(r, bb->lo[c]), bb->fact[c]));
        g[c]   = min(gi, Morton<K>::max_val);
    }
    keys[i] = Morton<K>::encode(g[0], g[1], g[2]);
}

// ---------------------------------------------------------------- bitonic sort
// Compare-exchange of the reference network (bitonicSort_updated_usm.cpp:29-39):
// swap iff reverse ^ (a < b), reverse = ((length << 1) & i) == 0.
template<class K>
__device__ __forceinline__ void cmpx(K &a, K &b, u32 &va, u32 &vb, bool reverse) {
    bool swap = reverse ^ (a < b);
    if (swap) {
        K t = a;
        a   = b;
        b   = t;
        u32 tv = va;
        va     = vb;
        vb     = tv;
    }
}

template<class K, int TILE>
__global__ void __launch_bounds__(512) k_bitonic_smem(K *__restrict__ keys, u32 *__restrict__ vals,
                                                      u32 tile, u32 length_lo, u32 length_hi,
                                                      u32 inc_start) {
    __shared__ K sk[TILE];
    __shared__ u32 sv[TILE];
    u32 base = blockIdx.x * tile;
    for (u32 k = threadIdx.x; k < tile; k += blockDim.x) {
        sk[k] = keys[base + k];
        sv[k] = vals[base + k];
    }
    __syncthreads();
    for (u32 length = length_lo; length < length_hi; length <<= 1) {
        u32 dir = length << 1;
        for (u32 inc = (length == length_lo) ? inc_start : length; inc > 0; inc >>= 1) {
            for (u32 j = threadIdx.x; j < tile / 2; j += blockDim.x) {
                u32 low = j & (inc - 1);
                u32 i   = (j << 1) - low;
                bool reverse = (dir & (base + i)) == 0;
                K a = sk[i], b = sk[i + inc];
                u32 va = sv[i], vb = sv[i + inc];
                cmpx(a, b, va, vb, reverse);
                sk[i]       = a;
                sk[i + inc] = b;
                sv[i]       = va;
                sv[i + inc] = vb;
            }
            __syncthreads();
        }
    }
    for (u32 k = threadIdx.x; k < tile; k += blockDim.x) {
        keys[base + k] = sk[k];
        vals[base + k] = sv[k];
    }
}

// LEVELS consecutive stages (inc, inc/2, ...) of one merge step in registers,
// as the reference's order_kernel<2^LEVELS> (bitonicSort_updated_usm.cpp:111-281).
template<class K, int LEVELS>
__global__ void __launch_bounds__(256) k_bitonic_global(K *__restrict__ keys, u32 *__restrict__ vals,
                                                        u32 nthreads, u32 length, u32 inc) {
    constexpr int S = 1 << LEVELS;
    u32 t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nthreads) return;
    u32 sub  = inc >> (LEVELS - 1);
    u32 low  = t & (sub - 1);
    u32 i    = ((t - low) << LEVELS) + low;
    bool reverse = ((length << 1) & i) == 0;
    K x[S];
    u32 v[S];
#pragma unroll
    for (int k = 0; k < S; k++) {
        x[k] = keys[i + k * sub];
        v[k] = vals[i + k * sub];
    }
#pragma unroll
    for (int d = S / 2; d >= 1; d >>= 1) {
#pragma unroll
        for (int k = 0; k < S; k++) {
            if ((k & d) == 0) cmpx(x[k], x[k + d], v[k], v[k + d], reverse);
        }
    }
#pragma unroll
    for (int k = 0; k < S; k++) {
        keys[i + k * sub] = x[k];
        vals[i + k * sub] = v[k];
    }
}

template<class K>
cudaError_t bitonic_sort(K *keys, u32 *vals, u32 len, cudaStream_t s) {
    constexpr int TILE = (sizeof(K) == 4) ? 4096 : 2048;
    if (len <= 1) return cudaSuccess;
    u32 tile = len < (u32) TILE ? len : (u32) TILE;
    { k_bitonic_smem<K, TILE><<<len / tile, 512, 0, s>>>(keys, vals, tile, 1, tile, 1); GBSPH_COUNTED; }
    for (u32 length = TILE; length < len; length <<= 1) {
        u32 inc = length;
        while (inc >= (u32) TILE) {
            int avail  = __builtin_ctz(inc) - __builtin_ctz((u32) TILE) + 1;
            int levels = avail < 4 ? avail : 4;
            u32 nth    = len >> levels;
            u32 blocks = div_up(nth, 256);
            switch (levels) {
            case 4: { k_bitonic_global<K, 4><<<blocks, 256, 0, s>>>(keys, vals, nth, length, inc); GBSPH_COUNTED; } break;
            case 3: { k_bitonic_global<K, 3><<<blocks, 256, 0, s>>>(keys, vals, nth, length, inc); GBSPH_COUNTED; } break;
            case 2: { k_bitonic_global<K, 2><<<blocks, 256, 0, s>>>(keys, vals, nth, length, inc); GBSPH_COUNTED; } break;
            default: { k_bitonic_global<K, 1><<<blocks, 256, 0, s>>>(keys, vals, nth, length, inc); GBSPH_COUNTED; } break;
            }
            inc >>= levels;
        }
        { k_bitonic_smem<K, TILE><<<len / TILE, 512, 0, s>>>(keys, vals, TILE, length, length << 1,
                                                          TILE / 2); GBSPH_COUNTED; }
    }
    return cudaGetLastError();
}

// ---------------------------------------------------------------- radix sort
// Stable LSD radix sort of n u32 keys with u32 values, four 8-bit digits.  Per pass: a
// per-block digit histogram (bucket-major), its exclusive scan (the global start of each
// block's elements of each digit), and a scatter that walks the block's tile in index
// order, 256 elements per round: lanes with equal digits are ranked with a warp match,
// warps by an exclusive prefix of their per-warp counts, so every pass is stable.  With
// distinct keys the result is the unique sorted order, hence the bitonic network's.
constexpr u32 kRadixItems = 8, kRadixTile = 256 * kRadixItems;

__global__ void __launch_bounds__(256) k_radix_hist(const u32 *__restrict__ keys, u32 n, int shift,
                                                    u32 nblocks, u32 *__restrict__ hist) {
    __shared__ u32 h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const u32 base = blockIdx.x * kRadixTile;
#pragma unroll
    for (u32 r = 0; r < kRadixItems; r++) {
        const u32 i = base + r * 256 + threadIdx.x;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[threadIdx.x * nblocks + blockIdx.x] = h[threadIdx.x];
}

__global__ void __launch_bounds__(256) k_radix_scatter(const u32 *__restrict__ kin,
                                                       const u32 *__restrict__ vin, u32 n, int shift,
                                                       u32 nblocks, const u32 *__restrict__ offs,
                                                       u32 *__restrict__ kout, u32 *__restrict__ vout) {
    __shared__ u32 cnt[256];   // next output slot of each digit for this block
    __shared__ u32 wc[8][256]; // per-warp digit counts, then their exclusive prefix
    const u32 t = threadIdx.x, lane = t & 31u, w = t >> 5;
    cnt[t]         = offs[t * nblocks + blockIdx.x];
    const u32 base = blockIdx.x * kRadixTile;
    for (u32 r = 0; r < kRadixItems; r++) {
        for (u32 k = lane; k < 256; k += 32) wc[w][k] = 0;
        __syncthreads();
        const u32 i     = base + r * 256 + t;
        const bool valid = i < n;
        const u32 key   = valid ? kin[i] : 0u;
        const u32 val   = valid ? vin[i] : 0u;
        const u32 d     = (key >> shift) & 255u;
        // invalid lanes match only themselves (values above 255)
        const u32 peers = __match_any_sync(0xffffffffu, valid ? d : (0x100u | lane));
        const u32 lower = __popc(peers & ((1u << lane) - 1u));
        if (valid && lower == 0) wc[w][d] = __popc(peers);
        __syncthreads();
        u32 run = cnt[t];
#pragma unroll
        for (u32 ww = 0; ww < 8; ww++) {
            const u32 c = wc[ww][t];
            wc[ww][t]   = run;
            run += c;
        }
        cnt[t] = run;
        __syncthreads();
        if (valid) {
            const u32 pos = wc[w][d] + lower;
            kout[pos]     = key;
            vout[pos]     = val;
        }
        __syncthreads();
    }
}

__global__ void k_adjacent_dup(const u32 *__restrict__ keys, u32 n, u32 *__restrict__ flag) {
    u32 i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i + 1 < n && keys[i] == keys[i + 1]) atomicOr(flag, 1u);
}

// sorts keys[0..n) / vals[0..n) in place (four passes end in the input buffers)
cudaError_t radix_sort_u32(Ctx &c, u32 *keys, u32 *vals, u32 n, cudaStream_t s) {
    cudaError_t e;
    if (n < 2) return cudaSuccess;
    const u32 nb = div_up(n, kRadixTile);
    if ((e = c.radix_k.ensure(sizeof(u32) * (size_t) n, s)) != cudaSuccess) return e;
    if ((e = c.radix_v.ensure(sizeof(u32) * (size_t) n, s)) != cudaSuccess) return e;
    if ((e = c.radix_hist.ensure(sizeof(u32) * 256 * (size_t) nb, s)) != cudaSuccess) return e;
    if ((e = c.radix_off.ensure(sizeof(u32) * 256 * (size_t) nb, s)) != cudaSuccess) return e;
    Scalars *dsc = c.d_scalars.as<Scalars>();
    u32 *ka = keys, *va = vals, *kb = c.radix_k.as<u32>(), *vb = c.radix_v.as<u32>();
    for (int shift = 0; shift < 32; shift += 8) {
        { k_radix_hist<<<nb, 256, 0, s>>>(ka, n, shift, nb, c.radix_hist.as<u32>()); GBSPH_COUNTED; }
        if ((e = scan_exclusive_u32(c.radix_hist.as<u32>(), c.radix_off.as<u32>(), 256 * nb,
                                    &dsc->total2, c.scan_scratch, s)) != cudaSuccess)
            return e;
        { k_radix_scatter<<<nb, 256, 0, s>>>(ka, va, n, shift, nb, c.radix_off.as<u32>(), kb, vb); GBSPH_COUNTED; }
        std::swap(ka, kb);
        std::swap(va, vb);
    }
    return cudaGetLastError();
}

// ---------------------------------------------------------------- leaf reduction
template<class K>
__device__ __forceinline__ i32 karras_delta(i32 x, i32 y, u32 len, const K *__restrict__ m) {
    if ((u32) y > len - 1 || y < 0) return -1;
    return Morton<K>::clz(m[x] ^ m[y]);
}

template<class K>
__global__ void k_split(const K *__restrict__ m, u32 cnt, u8 *__restrict__ out) {
    u32 i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cnt) return;
    out[i] = (i > 0) ? ((m[i - 1] != m[i]) ? 1 : 0) : 1;
}

template<class K>
__global__ void k_reduce_iter(const K *__restrict__ m, u32 cnt, const u8 *__restrict__ in,
                              u8 *__restrict__ out) {
    u32 i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cnt) return;
    u32 before1 = i - 1;
    while (before1 <= cnt - 1 && !in[before1]) before1--;
    u32 before2 = before1 - 1;
    while (before2 <= cnt - 1 && !in[before2]) before2--;
    u32 next1 = i + 1;
    while (next1 <= cnt - 1 && !in[next1]) next1++;
    i32 delt_0  = karras_delta<K>((i32) i, (i32) next1, cnt, m);
    i32 delt_m  = karras_delta<K>((i32) i, (i32) before1, cnt, m);
    i32 delt_mm = karras_delta<K>((i32) before1, (i32) before2, cnt, m);
    out[i] = (!(delt_0 < delt_m && delt_mm < delt_m) && in[i]) ? 1 : 0;
}

template<class K>
__global__ void k_compact_leaves(const u8 *__restrict__ flags, const u32 *__restrict__ offs, u32 cnt,
                                 const K *__restrict__ m, u32 *__restrict__ reduc,
                                 K *__restrict__ reduced) {
    u32 i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cnt) return;
    if (flags[i]) {
        u32 o      = offs[i];
        reduc[o]   = i;
        reduced[o] = m[i];
    }
}

__global__ void k_reduc_tail(u32 *reduc, const u32 *L, u32 cnt) {
    reduc[*L]     = cnt;
    reduc[*L + 1] = 0;
}

// ---------------------------------------------------------------- Karras
template<class K>
__global__ void k_karras(const K *__restrict__ m, u32 L, u32 *__restrict__ lchild,
                         u32 *__restrict__ rchild, u8 *__restrict__ lflag, u8 *__restrict__ rflag,
                         u32 *__restrict__ endrange, u32 *__restrict__ parent) {
    u32 ui = blockIdx.x * blockDim.x + threadIdx.x;
    if (ui == 0) parent[0] = kNone;
    if (ui + 1 >= L) return;
    i32 i = (i32) ui;
    auto DELTA = [&](i32 a, i32 b) { return karras_delta<K>(a, b, L, m); };
    i32 ddelta    = DELTA(i, i + 1) - DELTA(i, i - 1);
    i32 d         = (ddelta == 0) ? 0 : ((ddelta > 0) ? 1 : -1);
    i32 delta_min = DELTA(i, i - d);
    i32 lmax      = 2;
    while (DELTA(i, i + lmax * d) > delta_min) lmax *= 2;
    i32 l = 0;
    i32 t = lmax / 2;
    while (t > 0) {
        if (DELTA(i, i + (l + t) * d) > delta_min) l = l + t;
        t = t / 2;
    }
    u32 j          = (u32) (i + l * d);
    endrange[i]    = j;
    i32 delta_node = DELTA(i, (i32) j);
    i32 s          = 0;
    float div      = 2;
    t              = (i32) ceilf(__fdiv_rn((float) l, div));
    while (true) {
        i32 tmp_ = i + (s + t) * d;
        if (DELTA(i, tmp_) > delta_node) s = s + t;
        if (t <= 1) break;
        div *= 2;
        t = (i32) ceilf(__fdiv_rn((float) l, div));
    }
    i32 gamma  = i + s * d + min(d, 0);
    u32 off    = L - 1;
    bool lleaf = (min(ui, j) == (u32) gamma);
    bool rleaf = (max(ui, j) == (u32) (gamma + 1));
    lchild[i]  = (u32) gamma;
    lflag[i]   = lleaf ? 1 : 0;
    rchild[i]  = (u32) (gamma + 1);
    rflag[i]   = rleaf ? 1 : 0;
    parent[(u32) gamma + (lleaf ? off : 0)]       = ui;
    parent[(u32) (gamma + 1) + (rleaf ? off : 0)] = ui;
}

// ---------------------------------------------------------------- rank-order copies
__global__ void k_permute(const u32 *__restrict__ sort_index, u32 n, const f64 *__restrict__ x,
                          const f64 *__restrict__ y, const f64 *__restrict__ z,
                          const f64 *__restrict__ h, f64 *__restrict__ sx, f64 *__restrict__ sy,
                          f64 *__restrict__ sz, f64 *__restrict__ sh, u32 *__restrict__ rank_of) {
    u32 r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    u32 id     = sort_index[r];
    sx[r]      = x[id];
    sy[r]      = y[id];
    sz[r]      = z[id];
    if (h) sh[r] = h[id];
    rank_of[id] = r;
}

// ---------------------------------------------------------------- node boxes
__device__ __forceinline__ void store_box(NodeBox *b, const f64 lo[3], const f64 hi[3], f64 rint) {
    double2 *p = (double2 *) b;
    p[0]       = make_double2(lo[0], lo[1]);
    p[1]       = make_double2(lo[2], rint);
    p[2]       = make_double2(hi[0], hi[1]);
    p[3]       = make_double2(hi[2], 0.0);
}
__device__ __forceinline__ void load_box_cg(const NodeBox *b, f64 lo[3], f64 hi[3], f64 &rint) {
    const double2 *p = (const double2 *) b;
    double2 a = __ldcg(p), c = __ldcg(p + 1), d = __ldcg(p + 2), e = __ldcg(p + 3);
    lo[0] = a.x;
    lo[1] = a.y;
    lo[2] = c.x;
    rint  = c.y;
    hi[0] = d.x;
    hi[1] = d.y;
    hi[2] = e.x;
}

__global__ void k_leaf_boxes_up(const u32 *__restrict__ reduc, u32 L, const f64 *__restrict__ sx,
                                const f64 *__restrict__ sy, const f64 *__restrict__ sz,
                                const f64 *__restrict__ sh, f64 htol, const u32 *__restrict__ lchild,
                                const u32 *__restrict__ rchild, const u8 *__restrict__ lflag,
                                const u8 *__restrict__ rflag, const u32 *__restrict__ parent,
                                u32 *__restrict__ visit, NodeBox *__restrict__ boxes) {
    u32 l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= L) return;
    const f64 big = 1.7976931348623157e308;
    f64 lo[3] = {big, big, big}, hi[3] = {-big, -big, -big};
    f64 hm = -big;
    for (u32 r = reduc[l]; r < reduc[l + 1]; r++) {
        f64 p[3] = {sx[r], sy[r], sz[r]};
#pragma unroll
        for (int c = 0; c < 3; c++) {
            lo[c] = fmin(lo[c], p[c]);
            hi[c] = fmax(hi[c], p[c]);
        }
        if (sh) hm = fmax(hm, sh[r]);
    }
    f64 rint = sh ? __dmul_rn(hm, htol) : 0.0;
    u32 off  = L - 1;
    u32 node = off + l;
    store_box(&boxes[node], lo, hi, rint);
    __threadfence();
    u32 p = parent[node];
    while (p != kNone) {
        if (atomicAdd(&visit[p], 1u) == 0) return;
        __threadfence();
        u32 a = lchild[p] + off * (u32) lflag[p];
        u32 b = rchild[p] + off * (u32) rflag[p];
        f64 alo[3], ahi[3], blo[3], bhi[3], ar, br;
        load_box_cg(&boxes[a], alo, ahi, ar);
        load_box_cg(&boxes[b], blo, bhi, br);
#pragma unroll
        for (int c = 0; c < 3; c++) {
            lo[c] = fmin(alo[c], blo[c]);
            hi[c] = fmax(ahi[c], bhi[c]);
        }
        store_box(&boxes[p], lo, hi, fmax(ar, br));
        __threadfence();
        p = parent[p];
    }
}

// ---------------------------------------------------------------- bbox of merged positions
__global__ void k_bbox_init(Scalars *sc) {
    if (threadIdx.x < 3) {
        sc->bbox_min[threadIdx.x] = ~0ull;
        sc->bbox_max[threadIdx.x] = 0ull;
    }
}

__global__ void k_bbox_reduce(const f64 *__restrict__ x, const f64 *__restrict__ y,
                              const f64 *__restrict__ z, u32 n, Scalars *sc) {
    u64 mn[3] = {~0ull, ~0ull, ~0ull}, mx[3] = {0, 0, 0};
    for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        u64 o[3] = {f64_to_ordered(x[i]), f64_to_ordered(y[i]), f64_to_ordered(z[i])};
#pragma unroll
        for (int c = 0; c < 3; c++) {
            mn[c] = o[c] < mn[c] ? o[c] : mn[c];
            mx[c] = o[c] > mx[c] ? o[c] : mx[c];
        }
    }
#pragma unroll
    for (int c = 0; c < 3; c++) {
        u64 a = block_reduce(mn[c], OpMinU64{}, ~0ull);
        u64 b = block_reduce(mx[c], OpMaxU64{}, 0ull);
        if (threadIdx.x == 0) {
            atomicMin((unsigned long long *) &sc->bbox_min[c], (unsigned long long) a);
            atomicMax((unsigned long long *) &sc->bbox_max[c], (unsigned long long) b);
        }
    }
}

// nextafter widening (BuildTrees.cpp:50-55) + Morton grid step
__global__ void k_bbox_finalize(const Scalars *sc, BBox *bb, u32 val_count) {
    int c = threadIdx.x;
    if (c >= 3) return;
    f64 lo    = ordered_to_f64(sc->bbox_min[c]);
    f64 hi    = ordered_to_f64(sc->bbox_max[c]);
    lo        = nextafter(lo, -__longlong_as_double(0x7ff0000000000000ll));
    hi        = nextafter(hi, __longlong_as_double(0x7ff0000000000000ll));
    bb->lo[c] = lo;
    bb->hi[c] = hi;
    bb->fact[c] = __ddiv_rn(__dsub_rn(hi, lo), (f64) val_count);
}

template<class K>
cudaError_t tree_build_impl(Ctx &c, const f64 *x, const f64 *y, const f64 *z, const f64 *h, u32 n,
                            u32 level, f64 htol, u32 morton_count, bool fast_sort) {
    cudaStream_t s = c.stream;
    cudaError_t e;
    u32 P = morton_count;
    if (P == 0) {
        P = 1;
        while (P < n) P <<= 1;
    }
    c.n_obj        = n;
    c.morton_count = P;
    c.key_bits     = (int) sizeof(K) * 8;
    c.has_rint     = (h != nullptr);
#define ENS(buf, bytes)                                                                          \
    if ((e = (buf).ensure((bytes), s)) != cudaSuccess) return e;
    ENS(c.keys, sizeof(K) * P);
    ENS(c.sort_index, sizeof(u32) * P);
    ENS(c.flags_a, n);
    ENS(c.flags_b, n);
    ENS(c.offsets, sizeof(u32) * (size_t) n);
    ENS(c.reduc, sizeof(u32) * ((size_t) n + 2));
    ENS(c.reduced, sizeof(K) * (size_t) n);
    ENS(c.rank_of, sizeof(u32) * (size_t) n);
    ENS(c.sx, sizeof(f64) * (size_t) n);
    ENS(c.sy, sizeof(f64) * (size_t) n);
    ENS(c.sz, sizeof(f64) * (size_t) n);
    ENS(c.sh, sizeof(f64) * (size_t) n);

    K *keys = c.keys.as<K>();
    u32 *vals = c.sort_index.as<u32>();
    const u32 T = 256;
    Scalars *dsc = c.d_scalars.as<Scalars>();
    u8 *fa = c.flags_a.as<u8>(), *fb = c.flags_b.as<u8>();
    u8 *fin = (level % 2 == 0) ? fa : fb;
    // The radix sort is tried first when allowed; equal keys (whose order is the
    // network's) send the build back to the bitonic sort, found at the sync below.
    const bool radix = fast_sort && std::is_same<K, u32>::value;
    for (int attempt = radix ? 0 : 1; attempt < 2; attempt++) {
        {
            ProfScope ps(c, kProfSort, P);
            { k_morton<K><<<div_up(P, T), T, 0, s>>>(x, y, z, n, P, c.d_bbox.as<BBox>(), keys, vals); GBSPH_COUNTED; }
            if (attempt == 0) {
                if ((e = cudaMemsetAsync(&dsc->dup_keys, 0, sizeof(u32), s)) != cudaSuccess) return e;
                if ((e = radix_sort_u32(c, (u32 *) keys, vals, n, s)) != cudaSuccess) return e;
                { k_adjacent_dup<<<div_up(n, T), T, 0, s>>>((const u32 *) keys, n, &dsc->dup_keys); GBSPH_COUNTED; }
            } else {
                if ((e = bitonic_sort<K>(keys, vals, P, s)) != cudaSuccess) return e;
            }
        }
        int prof_tree = c.prof.on ? prof_begin(c, kProfTree, n) : -1;
        // leaf reduction: ping-pong split tables, final table is a for even levels
        { k_split<K><<<div_up(n, T), T, 0, s>>>(keys, n, fa); GBSPH_COUNTED; }
        for (u32 it = 1; it <= level; it++) {
            if (it % 2 == 0) { k_reduce_iter<K><<<div_up(n, T), T, 0, s>>>(keys, n, fb, fa); GBSPH_COUNTED; }
            else { k_reduce_iter<K><<<div_up(n, T), T, 0, s>>>(keys, n, fa, fb); GBSPH_COUNTED; }
        }
        if ((e = scan_exclusive_flags(fin, c.offsets.as<u32>(), n, &dsc->total, c.scan_scratch, s)) !=
            cudaSuccess)
            return e;
        { k_compact_leaves<K><<<div_up(n, T), T, 0, s>>>(fin, c.offsets.as<u32>(), n, keys,
                                                       c.reduc.as<u32>(), c.reduced.as<K>()); GBSPH_COUNTED; }
        { k_reduc_tail<<<1, 1, 0, s>>>(c.reduc.as<u32>(), &dsc->total, n); GBSPH_COUNTED; }
        if (prof_tree >= 0) prof_end(c, prof_tree);
        if ((e = sync_scalars(c)) != cudaSuccess) return e;
        if (attempt == 0 && !c.h_scalars->dup_keys) break;
    }
    ProfScope ps_tree(c, kProfTree, 0);
    u32 L        = c.h_scalars->total;
    c.leaf_count = L;
    u32 I        = L - 1;
    u32 Tn       = 2 * L - 1;
    ENS(c.lchild, sizeof(u32) * (I + 1));
    ENS(c.rchild, sizeof(u32) * (I + 1));
    ENS(c.lflag, I + 1);
    ENS(c.rflag, I + 1);
    ENS(c.endrange, sizeof(u32) * (I + 1));
    ENS(c.parent, sizeof(u32) * Tn);
    ENS(c.visit, sizeof(u32) * (I + 1));
    ENS(c.boxes, sizeof(NodeBox) * Tn);
#undef ENS
    { k_karras<K><<<div_up(L, T), T, 0, s>>>(c.reduced.as<K>(), L, c.lchild.as<u32>(),
                                           c.rchild.as<u32>(), c.lflag.as<u8>(), c.rflag.as<u8>(),
                                           c.endrange.as<u32>(), c.parent.as<u32>()); GBSPH_COUNTED; }
    { k_permute<<<div_up(n, T), T, 0, s>>>(vals, n, x, y, z, h, c.sx.as<f64>(), c.sy.as<f64>(),
                                         c.sz.as<f64>(), c.sh.as<f64>(), c.rank_of.as<u32>()); GBSPH_COUNTED; }
    if ((e = cudaMemsetAsync(c.visit.p, 0, sizeof(u32) * (I + 1), s)) != cudaSuccess) return e;
    { k_leaf_boxes_up<<<div_up(L, T), T, 0, s>>>(
        c.reduc.as<u32>(), L, c.sx.as<f64>(), c.sy.as<f64>(), c.sz.as<f64>(),
        h ? c.sh.as<f64>() : nullptr, htol, c.lchild.as<u32>(), c.rchild.as<u32>(),
        c.lflag.as<u8>(), c.rflag.as<u8>(), c.parent.as<u32>(), c.visit.as<u32>(),
        c.boxes.as<NodeBox>()); GBSPH_COUNTED; }
    return cudaGetLastError();
}

} // namespace

cudaError_t sync_scalars(Ctx &c) {
    cudaError_t e = cudaMemcpyAsync(c.h_scalars, c.d_scalars.p, sizeof(Scalars),
                                    cudaMemcpyDeviceToHost, c.stream);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(c.stream);
}

cudaError_t set_bbox_host(Ctx &c, const f64 *bmin, const f64 *bmax) {
    BBox b{};
    for (int k = 0; k < 3; k++) {
        b.lo[k] = bmin[k];
        b.hi[k] = bmax[k];
    }
    cudaError_t e = cudaMemcpyAsync(c.d_bbox.p, &b, sizeof(BBox), cudaMemcpyHostToDevice, c.stream);
    if (e != cudaSuccess) return e;
    // grid step for both key widths is filled by tree_build (depends on key width)
    return cudaStreamSynchronize(c.stream);
}

cudaError_t bbox_from_merged(Ctx &c, u32 n) {
    Scalars *dsc = c.d_scalars.as<Scalars>();
    ProfScope ps(c, kProfMerge, 0);
    { k_bbox_init<<<1, 32, 0, c.stream>>>(dsc); GBSPH_COUNTED; }
    u32 blocks = div_up(n, 256);
    if (blocks > 1216) blocks = 1216;
    if (blocks == 0) blocks = 1;
    { k_bbox_reduce<<<blocks, 256, 0, c.stream>>>(c.mx.as<f64>(), c.my.as<f64>(), c.mz.as<f64>(), n,
                                                dsc); GBSPH_COUNTED; }
    { k_bbox_finalize<<<1, 32, 0, c.stream>>>(dsc, c.d_bbox.as<BBox>(), Morton<u32>::val_count); GBSPH_COUNTED; }
    return cudaGetLastError();
}

cudaError_t tree_build(Ctx &c, const f64 *x, const f64 *y, const f64 *z, const f64 *h, u32 n,
                       u32 level, f64 htol, int key_bits, u32 morton_count, bool fast_sort) {
    if (key_bits == 64) {
        { k_bbox_fact<<<1, 32, 0, c.stream>>>(c.d_bbox.as<BBox>(), Morton<u64>::val_count); GBSPH_COUNTED; }
        return tree_build_impl<u64>(c, x, y, z, h, n, level, htol, morton_count, false);
    }
    { k_bbox_fact<<<1, 32, 0, c.stream>>>(c.d_bbox.as<BBox>(), Morton<u32>::val_count); GBSPH_COUNTED; }
    return tree_build_impl<u32>(c, x, y, z, h, n, level, htol, morton_count, fast_sort);
}

// explicit entry points for module-level exports (driver.cu)
template<class K>
cudaError_t sort_keys_dev(K *keys, u32 *vals, u32 len, cudaStream_t s) {
    return bitonic_sort<K>(keys, vals, len, s);
}
template cudaError_t sort_keys_dev<u32>(u32 *, u32 *, u32, cudaStream_t);
template cudaError_t sort_keys_dev<u64>(u64 *, u32 *, u32, cudaStream_t);

} // namespace gbsph

namespace gbsph {

namespace {
template<class K>
__global__ void k_morton_only(const f64 *__restrict__ x, const f64 *__restrict__ y,
                              const f64 *__restrict__ z, u32 n, u32 P, const BBox *__restrict__ bb,
                              K *__restrict__ keys) {
    u32 i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    if (i >= n) {
        keys[i] = Morton<K>::err;
        return;
    }
    const f64 p[3] = {x[i], y[i], z[i]};
    u32 g[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
        f64 r  = fmin(fmax(p[c], bb->lo[c]), bb->hi[c]);
        u32 gi = __double2uint_rz(__ddiv_rn(__dsub_rn(r, bb->lo[c]), bb->fact[c]));
        g[c]   = min(gi, Morton<K>::max_val);
    }
    keys[i] = Morton<K>::encode(g[0], g[1], g[2]);
}

__global__ void k_export_boxes(const NodeBox *__restrict__ b, u32 T, f64 *__restrict__ mn,
                               f64 *__restrict__ mx, f64 *__restrict__ rint) {
    u32 i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= T) return;
    NodeBox v = b[i];
    if (mn) {
        mn[3 * i] = v.lo[0];
        mn[3 * i + 1] = v.lo[1];
        mn[3 * i + 2] = v.lo[2];
    }
    if (mx) {
        mx[3 * i] = v.hi[0];
        mx[3 * i + 1] = v.hi[1];
        mx[3 * i + 2] = v.hi[2];
    }
    if (rint) rint[i] = v.rint;
}
} // namespace

cudaError_t morton_codes_dev(Ctx &c, const f64 *x, const f64 *y, const f64 *z, u32 n, u32 P,
                             int key_bits, void *out) {
    if (key_bits == 64) {
        { k_bbox_fact<<<1, 32, 0, c.stream>>>(c.d_bbox.as<BBox>(), Morton<u64>::val_count); GBSPH_COUNTED; }
        { k_morton_only<u64><<<div_up(P, 256), 256, 0, c.stream>>>(x, y, z, n, P, c.d_bbox.as<BBox>(),
                                                                 (u64 *) out); GBSPH_COUNTED; }
    } else {
        { k_bbox_fact<<<1, 32, 0, c.stream>>>(c.d_bbox.as<BBox>(), Morton<u32>::val_count); GBSPH_COUNTED; }
        { k_morton_only<u32><<<div_up(P, 256), 256, 0, c.stream>>>(x, y, z, n, P, c.d_bbox.as<BBox>(),
                                                                 (u32 *) out); GBSPH_COUNTED; }
    }
    return cudaGetLastError();
}

cudaError_t export_boxes(Ctx &c, f64 *mn, f64 *mx, f64 *rint) {
    u32 T = 2 * c.leaf_count - 1;
    { k_export_boxes<<<div_up(T, 256), 256, 0, c.stream>>>(c.boxes.as<NodeBox>(), T, mn, mx, rint); GBSPH_COUNTED; }
    return cudaGetLastError();
}

} // namespace gbsph
