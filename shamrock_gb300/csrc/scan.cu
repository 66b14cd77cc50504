// Device-wide exclusive prefix sums used by leaf compaction, CSR offsets and ghost
// selection (the role of shamalgs::numeric::scan_exclusive / stream_compact,
// shamalgs/src/details/numeric/numeric.cpp:48-92).
//
// Reduce-then-scan in three launches: per-tile totals, one block scanning the tile
// totals, per-tile scan plus tile offset.  A tile is 256 threads x 8 items.  Each item is
// read and written by the same thread, so the u32 scan may run in place (in == out).

#include "gbsph_internal.cuh"

namespace gbsph {

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems   = 8;
constexpr u32 kScanTile    = kScanThreads * kScanItems;

template<class In>
__device__ __forceinline__ void load_items(const In *in, u32 n, u32 base, u32 v[kScanItems]) {
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        u32 i = base + k;
        v[k]  = (i < n) ? (u32) in[i] : 0u;
    }
}

// inclusive warp scan
__device__ __forceinline__ u32 warp_incl_scan(u32 v) {
    int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        u32 t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// exclusive block scan of one value per thread; returns exclusive prefix, *total = sum
__device__ __forceinline__ u32 block_excl_scan(u32 v, u32 *total) {
    __shared__ u32 warp_sums[33];
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    u32 inc = warp_incl_scan(v);
    if (lane == 31) warp_sums[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        int nw  = blockDim.x >> 5;
        u32 ws  = (lane < nw) ? warp_sums[lane] : 0;
        u32 wsi = warp_incl_scan(ws);
        if (lane < nw) warp_sums[lane] = wsi - ws;
        if (lane == nw - 1) warp_sums[32] = wsi;
    }
    __syncthreads();
    u32 res = warp_sums[wid] + inc - v;
    *total  = warp_sums[32];
    __syncthreads();
    return res;
}

template<class In>
__global__ void k_tile_sums(const In *in, u32 n, u32 *tile_sums) {
    u32 base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    u32 v[kScanItems];
    load_items(in, n, base, v);
    u32 s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) s += v[k];
    s = block_reduce(s, OpAddU32{}, 0u);
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = s;
}

// one block: exclusive scan of the tile sums in place, grand total to *total
__global__ void k_scan_tiles(u32 *tile_sums, u32 ntiles, u32 *total) {
    u32 carry = 0;
    for (u32 base = 0; base < ntiles; base += blockDim.x) {
        u32 i = base + threadIdx.x;
        u32 v = (i < ntiles) ? tile_sums[i] : 0;
        u32 tot;
        u32 ex = block_excl_scan(v, &tot);
        if (i < ntiles) tile_sums[i] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) *total = carry;
}

template<class In>
__global__ void k_scan_apply(const In *in, u32 *out, u32 n, const u32 *tile_offsets) {
    u32 base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    u32 v[kScanItems];
    load_items(in, n, base, v);
    u32 s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) s += v[k];
    u32 tot;
    u32 ex  = block_excl_scan(s, &tot) + tile_offsets[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        u32 i = base + k;
        if (i < n) out[i] = ex;
        ex += v[k];
    }
}

template<class In>
cudaError_t scan_impl(const In *in, u32 *out, u32 n, u32 *total_dev, DevBuf &scratch,
                      cudaStream_t s) {
    u32 ntiles = div_up(n, kScanTile);
    if (ntiles == 0) ntiles = 1;
    cudaError_t e = scratch.ensure(sizeof(u32) * ntiles, s);
    if (e != cudaSuccess) return e;
    u32 *tiles = scratch.as<u32>();
    { k_tile_sums<In><<<ntiles, kScanThreads, 0, s>>>(in, n, tiles); GBSPH_COUNTED; }
    { k_scan_tiles<<<1, 1024, 0, s>>>(tiles, ntiles, total_dev); GBSPH_COUNTED; }
    if (n) { k_scan_apply<In><<<ntiles, kScanThreads, 0, s>>>(in, out, n, tiles); GBSPH_COUNTED; }
    return cudaGetLastError();
}

} // namespace

cudaError_t scan_exclusive_u32(
    const u32 *in, u32 *out, u32 n, u32 *total_dev, DevBuf &scratch, cudaStream_t s) {
    return scan_impl<u32>(in, out, n, total_dev, scratch, s);
}

cudaError_t scan_exclusive_flags(
    const u8 *in, u32 *out, u32 n, u32 *total_dev, DevBuf &scratch, cudaStream_t s) {
    return scan_impl<u8>(in, out, n, total_dev, scratch, s);
}

} // namespace gbsph
