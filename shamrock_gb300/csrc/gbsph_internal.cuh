// Internal declarations shared by the GB300 SPH hot-path translation units.
//
// Index spaces used throughout:
//   local id   : position of a particle in the caller's arrays, [0, n_local)
//   merged id  : locals then periodic ghosts, [0, N) with N = n_local + n_ghost
//                (the reference's merged_xyzh order, BasicSPHGhosts.hpp:452-517)
//   rank       : position in Morton-sorted order, [0, N); sort_index[rank] = merged id
//   row        : position of a local particle in rank order, [0, n_local);
//                row_rank[row] = its rank, row_local[row] = its local id.
// Pair kernels run one thread per row so that neighbouring threads touch
// neighbouring particles; all per-particle fields they read are gathered into
// rank order first.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <string>

typedef uint8_t u8;
typedef uint32_t u32;
typedef uint64_t u64;
typedef int32_t i32;
typedef int64_t i64;
typedef double f64;
typedef float f32;

#define GBSPH_OK 0
#define GBSPH_ERR_ARG 1
#define GBSPH_ERR_CUDA 2
#define GBSPH_ERR_CAPACITY 3
#define GBSPH_ERR_NOT_CONVERGED 4
#define GBSPH_ERR_STATE 5

namespace gbsph {

// Process-wide count of kernel launches issued by this library (every launch site is
// followed by GBSPH_COUNTED); read through gbsph_kernel_launches().  Atomic: contexts
// on different host threads, and the context-free entry point, count into it at once.
extern std::atomic<unsigned long long> g_kernel_launches;
#define GBSPH_COUNTED (::gbsph::g_kernel_launches.fetch_add(1, std::memory_order_relaxed))

// ------------------------------------------------------------------ constants
// M4 cubic spline, shammath/include/shammath/sphkernels.hpp:29-72
constexpr f64 kRkern   = 2.0;
constexpr f64 kHfact   = 1.2;
constexpr f64 kPi      = 3.141592653589793;
constexpr f64 kNorm3d  = 1 / kPi;

constexpr u32 kNone = 0xFFFFFFFFu;

// ------------------------------------------------------------------ exact FP64 helpers
// Round-to-nearest intrinsics are never contracted into FMA, so these give the same
// bits as the oracle's -ffp-contract=off arithmetic in every translation unit.
__device__ __forceinline__ f64 dot3_rn(f64 x, f64 y, f64 z) {
    return __dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z));
}

// ------------------------------------------------------------------ wide loads
// A 32-byte record fetched with one 256-bit read-only load (sm_100 and later): one L1
// request per lane instead of two 128-bit ones.  The pointer must be 32-byte aligned.
struct __align__(32) F8 {
    float4 a, b;
};
__device__ __forceinline__ F8 ldg256(const void *p) {
    F8 r;
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(r.a.x), "=f"(r.a.y), "=f"(r.a.z), "=f"(r.a.w), "=f"(r.b.x), "=f"(r.b.y),
          "=f"(r.b.z), "=f"(r.b.w)
        : "l"(p));
    return r;
}

// double <-> order-preserving u64 (for atomic min/max on doubles)
__device__ __forceinline__ u64 f64_to_ordered(f64 v) {
    u64 b = (u64) __double_as_longlong(v);
    return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}
__host__ __device__ inline f64 ordered_to_f64(u64 o) {
    union {
        u64 u;
        f64 d;
    } c;
    c.u = (o & 0x8000000000000000ull) ? (o & 0x7FFFFFFFFFFFFFFFull) : ~o;
    return c.d;
}

// ------------------------------------------------------------------ warp/block reductions
template<class T, class Op>
__device__ __forceinline__ T warp_reduce(T v, Op op) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = op(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// block-wide reduction; result valid in thread 0. blockDim.x multiple of 32, <= 1024.
template<class T, class Op, class I>
__device__ __forceinline__ T block_reduce(T v, Op op, I ident_) {
    const T ident = (T) ident_;
    __shared__ T sh[32];
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    v = warp_reduce(v, op);
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    int nw = (blockDim.x + 31) >> 5;
    v      = (threadIdx.x < nw) ? sh[threadIdx.x] : ident;
    if (wid == 0) v = warp_reduce(v, op);
    return v;
}

struct OpMaxU64 {
    __device__ u64 operator()(u64 a, u64 b) const { return a > b ? a : b; }
};
struct OpMinU64 {
    __device__ u64 operator()(u64 a, u64 b) const { return a < b ? a : b; }
};
struct OpAddF64 {
    __device__ f64 operator()(f64 a, f64 b) const { return a + b; }
};
struct OpAddF32 {
    __device__ float operator()(float a, float b) const { return a + b; }
};
struct OpAddU32 {
    __device__ u32 operator()(u32 a, u32 b) const { return a + b; }
};
struct OpAddU64 {
    __device__ u64 operator()(u64 a, u64 b) const { return a + b; }
};

inline u32 div_up(u64 a, u64 b) { return (u32) ((a + b - 1) / b); }

// ------------------------------------------------------------------ device buffers
// Growable stream-ordered device allocation owned by a context.
struct DevBuf {
    void *p     = nullptr;
    size_t size = 0;
    cudaError_t ensure(size_t bytes, cudaStream_t s) {
        if (bytes <= size) return cudaSuccess;
        if (p) {
            cudaError_t e = cudaFreeAsync(p, s);
            if (e != cudaSuccess) return e;
            p = nullptr;
        }
        size_t nb = bytes + bytes / 4 + 256;
        cudaError_t e = cudaMallocAsync(&p, nb, s);
        if (e != cudaSuccess) {
            size = 0;
            return e;
        }
        size = nb;
        return cudaSuccess;
    }
    void release(cudaStream_t s) {
        if (p) cudaFreeAsync(p, s);
        p    = nullptr;
        size = 0;
    }
    template<class T>
    T *as() const {
        return (T *) p;
    }
};

// Node box of the compressed-leaf BVH: AABB and interaction radius (max h x htol),
// 64 bytes so one node is two 32-byte sectors.
struct __align__(16) NodeBox {
    f64 lo[3];
    f64 rint;
    f64 hi[3];
    f64 pad;
};

// ------------------------------------------------------------------ scan helpers (scan.cu)
// Exclusive prefix sum of n u32 values; writes the grand total to *total_dev.
cudaError_t scan_exclusive_u32(
    const u32 *in, u32 *out, u32 n, u32 *total_dev, DevBuf &scratch, cudaStream_t s);
// Exclusive prefix sum of n u8 flags into u32 offsets (+ total).
cudaError_t scan_exclusive_flags(
    const u8 *in, u32 *out, u32 n, u32 *total_dev, DevBuf &scratch, cudaStream_t s);

} // namespace gbsph
