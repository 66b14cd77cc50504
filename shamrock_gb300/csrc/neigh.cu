// Two-stage neighbour cache over the compressed-leaf BVH —
//   shammodels/sph/src/modules/NeighbourCache.cpp:223-596 (start_neighbors_cache_2stages),
//   traversal shamtree/include/shamtree/KarrasTreeTraverser.hpp:70-118 (left-first DFS),
//   criteria shamtree/include/shamtree/kernels/geometry_utils.hpp:62-135,
//   CSR layout shamtree/include/shamtree/TreeTraversal.hpp:375-526.
//
// Stage 1: leaf -> candidate leaves (extended-AABB overlap, both directions), stored
//          as rank ranges: consecutive leaves cover consecutive ranks, so runs of
//          consecutive candidates merge and stage 2 walks fewer, longer runs.
// Owner:   local particle -> leaf (the last leaf, in DFS order, whose box holds it).
// Stage 2: local particle -> interacting particles, pair test
//          !(r^2 > (h_a htol)^2 R^2 && r^2 > (h_b htol)^2 R^2).
// Rows are local particles in Morton order; entries are ranks, so a row lists its
// neighbours in exactly the reference order (ascending leaf, then in-leaf order).

#include "gbsph_ctx.cuh"
#include "split64.cuh"

#include <cmath>
#include <cstddef>
#include <type_traits>

namespace gbsph {

namespace {

constexpr int kStack   = 64;
// Initial one-pass slots: stage-1 leaves per leaf, stage-2 entries per row (multiple of
// 4).  A build that overflows records its largest row and is rerun, still in one pass,
// with slots that fit; the context keeps the grown sizes for later builds.
constexpr u32 kLeafCap = 256;
constexpr u32 kRowCap  = 192;
// Beyond this many slot bytes (or u32 offsets) the exact two-pass builds run instead.
constexpr u64 kMaxSlotBytes = 24ull << 30;

__device__ __forceinline__ void load_box(const NodeBox *__restrict__ b, f64 lo[3], f64 hi[3],
                                         f64 &rint) {
    const double2 *p = (const double2 *) b;
    double2 a = __ldg(p), c = __ldg(p + 1), d = __ldg(p + 2), e = __ldg(p + 3);
    lo[0] = a.x;
    lo[1] = a.y;
    lo[2] = c.x;
    rint  = c.y;
    hi[0] = d.x;
    hi[1] = d.y;
    hi[2] = e.x;
}

struct TreeView {
    const u32 *lchild, *rchild;
    const u8 *lflag, *rflag;
    const NodeBox *boxes;
    const u32 *reduc;
    u32 L;
    __device__ u32 off() const { return L - 1; }
    __device__ u32 left(u32 n) const { return lchild[n] + off() * (u32) lflag[n]; }
    __device__ u32 right(u32 n) const { return rchild[n] + off() * (u32) rflag[n]; }
};

// left-first stack DFS; on_leaf(leaf_index) in ascending leaf order
template<class Crit, class OnLeaf>
__device__ __forceinline__ bool dfs(const TreeView &t, Crit &&crit, OnLeaf &&on_leaf) {
    u32 stack[kStack];
    int top      = 0;
    stack[top++] = 0;
    u32 off      = t.off();
    while (top > 0) {
        u32 node = stack[--top];
        if (!crit(node)) continue;
        if (node >= off) {
            on_leaf(node - off);
        } else {
            if (top + 2 > kStack) return false;
            stack[top++] = t.right(node);
            stack[top++] = t.left(node);
        }
    }
    return true;
}

// Candidate leaves arrive in ascending order; a leaf following the previous run
// directly extends it.  A run of leaves [l0, l1) is stored as its rank range
// [reduc[l0], reduc[l1]).  `c` counts runs; only the first `cap` are stored.
struct RangeWriter {
    uint2 *out;
    const u32 *reduc;
    u32 base, cap, c;
    uint2 cur;
    bool open;
    __device__ RangeWriter(uint2 *o, const u32 *rd, u32 b, u32 cp)
        : out(o), reduc(rd), base(b), cap(cp), c(0), open(false) {}
    __device__ __forceinline__ void add(u32 r0, u32 r1) {
        if (open && cur.y == r0) {
            cur.y = r1;
            return;
        }
        flush();
        cur  = make_uint2(r0, r1);
        open = true;
    }
    __device__ __forceinline__ void flush() {
        if (!open) return;
        if (out && c < cap) out[base + c] = make_uint2(reduc[cur.x], reduc[cur.y]);
        c++;
        open = false;
    }
};

// ---- stage 1 criterion (NeighbourCache.cpp:289-334)
__device__ __forceinline__ bool cella_neigh_b(const f64 amin[3], const f64 amax[3],
                                              const f64 bmin[3], const f64 bmax[3]) {
    return (fmax(amin[0], bmin[0]) <= fmin(amax[0], bmax[0]))
           && (fmax(amin[1], bmin[1]) <= fmin(amax[1], bmax[1]))
           && (fmax(amin[2], bmin[2]) <= fmin(amax[2], bmax[2]));
}

struct LeafCrit {
    const TreeView &t;
    f64 amin[3], amax[3], amin_ext[3], amax_ext[3];
    __device__ LeafCrit(const TreeView &tv, u32 leaf) : t(tv) {
        f64 r;
        load_box(&t.boxes[t.off() + leaf], amin, amax, r);
        f64 ra = __dmul_rn(r, kRkern);
#pragma unroll
        for (int c = 0; c < 3; c++) {
            amin_ext[c] = __dsub_rn(amin[c], ra);
            amax_ext[c] = __dadd_rn(amax[c], ra);
        }
    }
    __device__ bool operator()(u32 node) const {
        f64 nlo[3], nhi[3], r;
        load_box(&t.boxes[node], nlo, nhi, r);
        f64 rn = __dmul_rn(r, kRkern);
        f64 emin[3], emax[3];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            emin[c] = __dsub_rn(nlo[c], rn);
            emax[c] = __dadd_rn(nhi[c], rn);
        }
        return cella_neigh_b(amin, amax, emin, emax) || cella_neigh_b(amin_ext, amax_ext, nlo, nhi);
    }
};

// The same criterion with the leaf's FP64 box loaded at each call: for the one-pass
// traversal, which decides almost every node in FP32 and calls this only inside the
// rounding band, keeping twelve doubles out of its registers.
struct LazyLeafCrit {
    const TreeView &t;
    u32 leaf_node;
    __device__ LazyLeafCrit(const TreeView &tv, u32 leaf) : t(tv), leaf_node(tv.off() + leaf) {}
    __device__ bool operator()(u32 node) const {
        const LeafCrit eager(t, leaf_node - t.off());
        return eager(node);
    }
};

// exact two-pass stage 1: range counts, then ranges at the scanned offsets
__global__ void k_leaf_count(TreeView t, u32 *__restrict__ cnt, u32 *__restrict__ flags) {
    u32 l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= t.L) return;
    LeafCrit crit(t, l);
    RangeWriter w(nullptr, t.reduc, 0, 0);
    bool ok = dfs(t, crit, [&](u32 leaf) { w.add(leaf, leaf + 1); });
    w.flush();
    if (!ok) atomicOr(flags, kFlagStackOverflow);
    cnt[l] = w.c;
}

__global__ void k_leaf_fill(TreeView t, const u32 *__restrict__ off, uint2 *__restrict__ ent) {
    u32 l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= t.L) return;
    LeafCrit crit(t, l);
    RangeWriter w(ent, t.reduc, off[l], 0xffffffffu);
    dfs(t, crit, [&](u32 leaf) { w.add(leaf, leaf + 1); });
    w.flush();
}

// ---- stage 1, one pass into `cap` slots per leaf, optional FP32 pre-test.
// For boxes a (the leaf) and n (a node) the criterion is
//   C1 || C2,  C1 = a overlaps n grown by r_n,  C2 = a grown by r_a overlaps n,
// which in exact arithmetic is  max_axis s <= max(r_n, r_a)  with the per-axis
// separation s = max(n.lo - a.hi, a.lo - n.hi).  The FP32 estimate of s carries at most
// ~2e-7 of the largest coordinate M plus 1e-7 relative; outside a band of
// 1e-6 (M + R) the FP32 answer is certain, inside it the FP64 criterion decides.
__global__ void k_boxes_f32(const NodeBox *__restrict__ b, u32 T, NodeBoxF *__restrict__ f) {
    u32 i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= T) return;
    NodeBox v = b[i];
    f[i].lo = make_float4(__double2float_rn(v.lo[0]), __double2float_rn(v.lo[1]),
                          __double2float_rn(v.lo[2]), __double2float_rn(__dmul_rn(v.rint, kRkern)));
    f[i].hi = make_float4(__double2float_rn(v.hi[0]), __double2float_rn(v.hi[1]),
                          __double2float_rn(v.hi[2]), 0.f);
}

__global__ void k_node_pairs(TreeView t, const NodeBoxF *__restrict__ fb, NodePairF *__restrict__ rec) {
    u32 n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= t.off()) return; // internal nodes 0 .. L - 2
    u32 l = t.left(n), r = t.right(n);
    NodeBoxF bl = fb[l], br = fb[r];
    bl.hi.w = __uint_as_float(l);
    br.hi.w = __uint_as_float(r);
    rec[n]  = NodePairF{bl, br};
}

// Stage 1 over the child-pair records.  A popped internal node loads both children's
// boxes in one record and tests them together, pushing those that pass (right, then
// left, so the left subtree is walked first); a popped leaf has passed and is
// reported.  Every node is tested once, when its parent is expanded, so the leaves and
// their order are those of dfs() with the same criterion; per step the traversal waits
// on one record load instead of a box load and a child-index load per node.
// leaf_thr (optional, see k_owner): a leaf owning no row gets an empty list, and a
// candidate leaf that no owned row can pair with is dropped (the cache is unchanged).
__global__ void __launch_bounds__(128) k_leaf_lists(TreeView t, const NodeBoxF *__restrict__ fb,
                                                    const NodePairF *__restrict__ rec,
                                                    u32 *__restrict__ cnt, u32 *__restrict__ off,
                                                    uint2 *__restrict__ ent, u32 cap, Scalars *sc,
                                                    const u32 *__restrict__ leaf_thr) {
    u32 l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= t.L) return;
    u32 base = l * cap;
    float thr_own = 0.f;
    if (leaf_thr) {
        const u32 tb = leaf_thr[l];
        if (tb == 0) { // no row is owned by this leaf: stage 2 never reads its list
            cnt[l] = 0;
            off[l] = base;
            return;
        }
        thr_own = __uint_as_float(tb);
    }
    LazyLeafCrit crit(t, l);
    const u32 offn = t.off();
    F8 fa = ldg256(&fb[offn + l]), fr = ldg256(&fb[0]);
    const float4 alo = fa.a, ahi = fa.b, rlo = fr.a, rhi = fr.b;
    float M = fmaxf(fmaxf(fmaxf(fabsf(rlo.x), fabsf(rlo.y)), fmaxf(fabsf(rlo.z), fabsf(rhi.x))),
                    fmaxf(fabsf(rhi.y), fabsf(rhi.z)));
    float band_abs = 1e-6f * M;
    // the criterion with an FP32 decision outside the rounding band
    auto test = [&](u32 node, const float4 &nlo, const float4 &nhi) -> bool {
        float sx = fmaxf(nlo.x - ahi.x, alo.x - nhi.x);
        float sy = fmaxf(nlo.y - ahi.y, alo.y - nhi.y);
        float sz = fmaxf(nlo.z - ahi.z, alo.z - nhi.z);
        float sm = fmaxf(fmaxf(sx, sy), sz);
        float R  = fmaxf(nlo.w, alo.w);
        float band = band_abs + 1e-6f * R;
        if (sm < R - band) return true;
        if (sm > R + band) return false;
        return crit(node);
    };
    // Exact pruning for stage 2: every row owned by this leaf lies in its box, so a
    // pair (a, b) with b in the candidate leaf has r_ab at least the Euclidean gap D
    // between the boxes.  With thr_own >= thr_a of every owned row and
    // (r_leaf R)^2 >= thr_b, D^2 > max of the two makes every pair test fail.  The FP32
    // gaps are shrunk by the rounding band and the bound carries a 1e-5 margin, so the
    // skip is certain.
    auto keep = [&](const float4 &nlo, const float4 &nhi) -> bool {
        if (!leaf_thr) return true;
        float gx = fmaxf(fmaxf(nlo.x - ahi.x, alo.x - nhi.x) - band_abs, 0.f);
        float gy = fmaxf(fmaxf(nlo.y - ahi.y, alo.y - nhi.y) - band_abs, 0.f);
        float gz = fmaxf(fmaxf(nlo.z - ahi.z, alo.z - nhi.z) - band_abs, 0.f);
        float d2 = gx * gx + gy * gy + gz * gz;
        float tb = fmaxf(thr_own, nlo.w * nlo.w * 1.000001f);
        return !(d2 > tb * 1.00001f);
    };
    u32 stack[kStack];
    int top = 0;
    bool ok = true;
    RangeWriter w(ent, t.reduc, base, cap);
    if (test(0, rlo, rhi) && (offn > 0 || keep(rlo, rhi))) stack[top++] = 0;
    while (top > 0) {
        const u32 n = stack[--top];
        if (n >= offn) {
            w.add(n - offn, n - offn + 1);
            continue;
        }
        const F8 bl = ldg256(&rec[n].l), br = ldg256(&rec[n].r);
        const u32 li = __float_as_uint(bl.b.w), ri = __float_as_uint(br.b.w);
        bool pl = test(li, bl.a, bl.b), pr = test(ri, br.a, br.b);
        if (pl && li >= offn) pl = keep(bl.a, bl.b);
        if (pr && ri >= offn) pr = keep(br.a, br.b);
        if (top + 2 > kStack) {
            ok = false;
            break;
        }
        if (pr) stack[top++] = ri;
        if (pl) stack[top++] = li;
    }
    w.flush();
    const u32 c = w.c;
    if (!ok) atomicOr(&sc->flags, kFlagStackOverflow);
    if (c > cap) {
        atomicOr(&sc->flags, kFlagLeafCap);
        atomicMax(&sc->leaf_cnt_max, c);
    }
    cnt[l] = c;
    off[l] = base;
}

// ---- rows: local particles in rank order
__global__ void k_row_flags(const u32 *__restrict__ sort_index, u32 N, u32 n_local,
                            u8 *__restrict__ flags) {
    u32 r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= N) return;
    flags[r] = sort_index[r] < n_local ? 1 : 0;
}
__global__ void k_rows(const u32 *__restrict__ sort_index, const u8 *__restrict__ flags,
                       const u32 *__restrict__ offs, u32 N, u32 *__restrict__ row_rank,
                       u32 *__restrict__ row_local) {
    u32 r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= N || !flags[r]) return;
    u32 row        = offs[r];
    row_rank[row]  = r;
    row_local[row] = sort_index[r];
}

// ---- owner leaf: max leaf index whose box contains the point (inclusive bounds),
// i.e. the last leaf the reference's left-first DFS reports (NeighbourCache.cpp:419-443).
// Right-first traversal over the child-pair records (the first leaf reached is the
// largest); containment is decided in FP32 outside a rounding band, else in FP64.
// leaf_thr (optional): per leaf, the FP32 bits (rounded up) of the largest pair-test
// threshold thr_a = ((h_a htol)^2) R^2 over the rows it owns, 0 for a leaf owning none.
// The exact containment test inside the FP32 band compares the doubles' ordered bit
// patterns with integer operations (the FP64 pipe is scarce on GB300; particles lie on
// their own leaf's faces, so the band is met often).
__device__ __forceinline__ long long ord64(f64 v) {
    long long b = __double_as_longlong(v);
    if (b == (long long) 0x8000000000000000ull) b = 0; // -0 orders as +0
    return b < 0 ? (b ^ 0x7fffffffffffffffll) : b;
}

__global__ void __launch_bounds__(128) k_owner(TreeView t, const NodeBoxF *__restrict__ fb,
                                               const NodePairF *__restrict__ rec,
                                               const u32 *__restrict__ row_rank, u32 n_rows,
                                               const f64 *__restrict__ sx, const f64 *__restrict__ sy,
                                               const f64 *__restrict__ sz, u32 *__restrict__ owner,
                                               u32 *__restrict__ flags, const f64 *__restrict__ sh,
                                               float h_tol_up, u32 *__restrict__ leaf_thr) {
    u32 row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= n_rows) return;
    u32 r    = row_rank[row];
    const f64 p[3] = {sx[r], sy[r], sz[r]};
    const long long op[3] = {ord64(p[0]), ord64(p[1]), ord64(p[2])};
    float px, py, pz, lo_unused;
    split64(p[0], px, lo_unused);
    split64(p[1], py, lo_unused);
    split64(p[2], pz, lo_unused);
    const F8 fr = ldg256(&fb[0]);
    float M = fmaxf(fmaxf(fmaxf(fabsf(fr.a.x), fabsf(fr.a.y)), fmaxf(fabsf(fr.a.z), fabsf(fr.b.x))),
                    fmaxf(fabsf(fr.b.y), fabsf(fr.b.z)));
    const float band = 1e-6f * M;
    auto inside = [&](u32 node, const float4 &lo, const float4 &hi) -> bool {
        float m = fminf(fminf(fminf(px - lo.x, py - lo.y), fminf(pz - lo.z, hi.x - px)),
                        fminf(hi.y - py, hi.z - pz));
        if (m > band) return true;
        if (m < -band) return false;
        f64 l64[3], h64[3], rr;
        load_box(&t.boxes[node], l64, h64, rr);
        return (ord64(l64[0]) <= op[0]) && (op[0] <= ord64(h64[0])) && (ord64(l64[1]) <= op[1])
               && (op[1] <= ord64(h64[1])) && (ord64(l64[2]) <= op[2]) && (op[2] <= ord64(h64[2]));
    };
    const u32 offn = t.off();
    u32 stack[kStack];
    int top   = 0;
    u32 found = kNone;
    if (inside(0, fr.a, fr.b)) stack[top++] = 0;
    while (top > 0) {
        const u32 n = stack[--top];
        if (n >= offn) {
            found = n - offn;
            break;
        }
        const F8 bl = ldg256(&rec[n].l), br = ldg256(&rec[n].r);
        const u32 li = __float_as_uint(bl.b.w), ri = __float_as_uint(br.b.w);
        const bool cl = inside(li, bl.a, bl.b), cr = inside(ri, br.a, br.b);
        if (top + 2 > kStack) {
            atomicOr(flags, kFlagStackOverflow);
            break;
        }
        if (cl) stack[top++] = li;
        if (cr) stack[top++] = ri;
    }
    if (found == kNone) {
        atomicOr(flags, kFlagOwnerMissing);
        found = 0;
    } else if (leaf_thr) {
        // an FP32 upper bound of thr_a = fl64(fl64(h htol)^2 R^2): every factor rounded up
        // (a float at or above a real number is at or above its nearest double)
        const float rint = __fmul_ru(__double2float_ru(sh[r]), h_tol_up);
        const float thr  = __fmul_ru(__fmul_ru(rint, rint), (float) (kRkern * kRkern));
        atomicMax(&leaf_thr[found], __float_as_uint(thr));
    }
    owner[row] = found;
}

// ---- stage 2 (NeighbourCache.cpp:492-591)
// MODE kCount: per-row count, and the count rounded up to 4 into off[] (scanned in
// place into offsets); kFill: entries at off[row]; kOnePass: entries straight into
// `cap` slots per row (off[row] = row * cap), flagging kFlagCsrCap when a row
// overflows so the host reruns the two-pass build.  Either way every row starts on a
// 16-byte boundary, so readers may fetch entries four at a time.
//
// F32: the pair test is r^2 <= max(thr_a, thr_b), thr = ((h htol)^2) R^2 in FP64.  r^2
// is estimated in FP32 from hi/lo-split positions (relative error below ~3e-7) and
// compared with the FP32 rounding of max(thr_a, thr_b) carried in the position record;
// outside a +-1e-5 relative band the answer is certain, inside it the exact FP64 test
// decides.  The cache is therefore identical to the FP64 one.
enum CacheMode { kCount = 0, kFill = 1, kOnePass = 2 };

template<int MODE, bool F32>
__global__ void __launch_bounds__(256) k_part_cache(
    const u32 *__restrict__ row_rank, u32 n_rows, const u32 *__restrict__ owner,
    const u32 *__restrict__ leaf_cnt, const u32 *__restrict__ leaf_off,
    const uint2 *__restrict__ leaf_ent, const float4 *__restrict__ P,
    const f64 *__restrict__ sx, const f64 *__restrict__ sy, const f64 *__restrict__ sz,
    const f64 *__restrict__ sh, f64 h_tol, u32 *__restrict__ cnt, u32 *__restrict__ off,
    u32 *__restrict__ ent, Scalars *sc, u32 cap) {
    u32 row = blockIdx.x * blockDim.x + threadIdx.x;
    u32 c   = 0;
    if (row < n_rows) {
        u32 ra     = row_rank[row];
        f64 xa     = sx[ra], ya = sy[ra], za = sz[ra];
        f64 rint_a = __dmul_rn(sh[ra], h_tol);
        f64 thr_a  = __dmul_rn(__dmul_rn(rint_a, rint_a), kRkern * kRkern);
        float4 Aa = make_float4(0, 0, 0, 0), Ba = Aa;
        if (F32) {
            F8 pa = ldg256(&P[2 * (size_t) ra]);
            Aa    = pa.a;
            Ba    = pa.b;
        }
        const float lo_f = 1.f - 1e-5f, hi_f = 1.f + 1e-5f;
        u32 leaf = owner[row];
        u32 k0 = leaf_off[leaf], k1 = k0 + leaf_cnt[leaf];
        u32 w = (MODE == kFill) ? off[row] : ((MODE == kOnePass) ? row * cap : 0);
        // one flat loop over the row's candidates (rows of a warp with different owner
        // leaves then stay converged); the next range is fetched one range ahead
        uint2 g  = (k0 < k1) ? leaf_ent[k0] : make_uint2(0, 0);
        u32 k    = k0 + 1;
        uint2 gn = (k < k1) ? leaf_ent[k] : g;
        u32 rb   = g.x;
        bool more = true;
        while (true) {
            while (rb >= g.y) {
                if (k >= k1) {
                    more = false;
                    break;
                }
                g  = gn;
                rb = g.x;
                k++;
                if (k < k1) gn = leaf_ent[k];
            }
            if (!more) break;
            {
                int decided = -1;
                if (F32) {
                    F8 pb = ldg256(&P[2 * (size_t) rb]);
                    const float4 Ab = pb.a, Bb = pb.b;
                    float dx = __fadd_rn(__fsub_rn(Aa.x, Ab.x), __fsub_rn(Ba.x, Bb.x));
                    float dy = __fadd_rn(__fsub_rn(Aa.y, Ab.y), __fsub_rn(Ba.y, Bb.y));
                    float dz = __fadd_rn(__fsub_rn(Aa.z, Ab.z), __fsub_rn(Ba.z, Bb.z));
                    float r2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
                    float tm = fmaxf(Ba.w, Bb.w);
                    decided  = (r2 < tm * lo_f) ? 1 : ((r2 > tm * hi_f) ? 0 : -1);
                }
                bool in;
                if (decided >= 0) {
                    in = decided == 1;
                } else {
                    f64 dx = __dsub_rn(xa, sx[rb]), dy = __dsub_rn(ya, sy[rb]),
                        dz = __dsub_rn(za, sz[rb]);
                    f64 rab2   = dot3_rn(dx, dy, dz);
                    f64 rint_b = __dmul_rn(sh[rb], h_tol);
                    f64 thr_b  = __dmul_rn(__dmul_rn(rint_b, rint_b), kRkern * kRkern);
                    in = !(rab2 > thr_a && rab2 > thr_b);
                }
                if (in) {
                    if (MODE == kFill) ent[w + c] = rb;
                    if (MODE == kOnePass && c < cap) ent[w + c] = rb;
                    c++;
                }
            }
            rb++;
        }
        if (MODE != kFill) cnt[row] = c;
        if (MODE == kCount) off[row] = (c + 3u) & ~3u;
        if (MODE == kOnePass) {
            off[row] = w;
            if (c > cap) atomicOr(&sc->flags, kFlagCsrCap);
        }
    }
    // the largest row of the build (sizes the slots of the next one)
    {
        u64 m = block_reduce((u64) c, OpMaxU64{}, 0ull);
        if (threadIdx.x == 0 && m) atomicMax(&sc->row_cnt_max, (u32) m);
    }
    if (MODE != kCount) {
        u64 tot = block_reduce((u64) c, OpAddU64{}, 0ull);
        if (threadIdx.x == 0) atomicAdd((unsigned long long *) &sc->csr_entries, (unsigned long long) tot);
    }
}

// ---- generic object query (CLBVHObjectIterator::rtree_for, CLBVHObjectIterator.hpp:127-169)
template<bool FILL>
__global__ void k_query(TreeView t, const f64 *__restrict__ qx, const f64 *__restrict__ qy,
                        const f64 *__restrict__ qz, u32 nq, int mode, f64 s,
                        const u32 *__restrict__ sort_index, const f64 *__restrict__ sx,
                        const f64 *__restrict__ sy, const f64 *__restrict__ sz,
                        u32 *__restrict__ counts, const u32 *__restrict__ offs, u32 *__restrict__ out,
                        u32 *__restrict__ flags) {
    u32 q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nq) return;
    f64 lo[3] = {__dadd_rn(qx[q], -s), __dadd_rn(qy[q], -s), __dadd_rn(qz[q], -s)};
    f64 hi[3] = {__dadd_rn(qx[q], s), __dadd_rn(qy[q], s), __dadd_rn(qz[q], s)};
    u32 c = 0, w = FILL ? offs[q] : 0;
    bool ok = dfs(
        t,
        [&](u32 node) {
            if (mode == 0) return true;
            f64 nl[3], nh[3], r;
            load_box(&t.boxes[node], nl, nh, r);
            for (int k = 0; k < 3; k++)
                if (!(fmin(nh[k], hi[k]) >= fmax(nl[k], lo[k]))) return false;
            return true;
        },
        [&](u32 leaf) {
            for (u32 rr = t.reduc[leaf]; rr < t.reduc[leaf + 1]; rr++) {
                bool in = true;
                if (mode == 1) {
                    f64 p[3] = {sx[rr], sy[rr], sz[rr]};
                    for (int k = 0; k < 3; k++)
                        if (!(fmin(p[k], hi[k]) >= fmax(p[k], lo[k]))) in = false;
                }
                if (in) {
                    if (FILL) out[w++] = sort_index[rr];
                    c++;
                }
            }
        });
    if (!ok) atomicOr(flags, kFlagStackOverflow);
    if (!FILL) counts[q] = c;
}

// the smallest float at or above v (host)
float up_f32(f64 v) {
    float f = (float) v;
    if ((f64) f < v) f = std::nextafter(f, INFINITY);
    return f;
}

TreeView view(const Ctx &c) {
    return TreeView{c.lchild.as<u32>(), c.rchild.as<u32>(), c.lflag.as<u8>(), c.rflag.as<u8>(),
                    c.boxes.as<NodeBox>(), c.reduc.as<u32>(), c.leaf_count};
}

} // namespace

cudaError_t build_rows(Ctx &c, u32 n_local) {
    cudaStream_t s = c.stream;
    cudaError_t e;
    u32 N = c.n_obj;
    if ((e = c.row_flags.ensure(N, s)) != cudaSuccess) return e;
    if ((e = c.row_offsets.ensure(sizeof(u32) * (size_t) N, s)) != cudaSuccess) return e;
    if ((e = c.row_rank.ensure(sizeof(u32) * (size_t) n_local, s)) != cudaSuccess) return e;
    if ((e = c.row_local.ensure(sizeof(u32) * (size_t) n_local, s)) != cudaSuccess) return e;
    { k_row_flags<<<div_up(N, 256), 256, 0, s>>>(c.sort_index.as<u32>(), N, n_local,
                                               c.row_flags.as<u8>()); GBSPH_COUNTED; }
    Scalars *dsc = c.d_scalars.as<Scalars>();
    if ((e = scan_exclusive_flags(c.row_flags.as<u8>(), c.row_offsets.as<u32>(), N, &dsc->total2,
                                  c.scan_scratch, s)) != cudaSuccess)
        return e;
    { k_rows<<<div_up(N, 256), 256, 0, s>>>(c.sort_index.as<u32>(), c.row_flags.as<u8>(),
                                          c.row_offsets.as<u32>(), N, c.row_rank.as<u32>(),
                                          c.row_local.as<u32>()); GBSPH_COUNTED; }
    c.n_local = n_local;
    return cudaGetLastError();
}

cudaError_t neigh_cache_build(Ctx &c, f64 h_tol, const float4 *P) {
    cudaStream_t s = c.stream;
    cudaError_t e;
    u32 L = c.leaf_count, n = c.n_local;
    if (L == 0) {
        c.err = "neighbour cache: the tree has no leaves";
        return cudaErrorInvalidValue;
    }
    TreeView t = view(c);
    Scalars *dsc = c.d_scalars.as<Scalars>();
    if ((e = c.leaf_cnt.ensure(sizeof(u32) * (size_t) L, s)) != cudaSuccess) return e;
    if ((e = c.leaf_off.ensure(sizeof(u32) * (size_t) L, s)) != cudaSuccess) return e;
    // Stage 1 in one pass into c.leaf_cap slots per leaf; if a leaf has more candidates
    // the pass is rerun with slots that fit, or, past the slot budget, the exact
    // two-pass build runs.
    // flags, leaf_cnt_max and row_cnt_max are adjacent u32 fields of Scalars
    static_assert(offsetof(Scalars, leaf_cnt_max) == offsetof(Scalars, flags) + 4 &&
                      offsetof(Scalars, row_cnt_max) == offsetof(Scalars, flags) + 8,
                  "Scalars field order");
    if ((e = cudaMemsetAsync(&dsc->flags, 0, 3 * sizeof(u32), s)) != cudaSuccess) return e;
    if (c.leaf_cap == 0) c.leaf_cap = kLeafCap;
    const u64 budget = c.slot_budget ? c.slot_budget : kMaxSlotBytes;
    auto slots_ok = [&](u64 rows, u32 cap, u64 esize = 4) {
        return rows * cap < 0xffffffffull && rows * cap * esize <= budget;
    };
    const bool s1_one_pass = slots_ok(L, c.leaf_cap, sizeof(uint2));
    // FP32 node boxes and the child-pair records the traversals read (the FP64 boxes
    // decide inside the rounding band)
    const u32 T = 2 * L - 1;
    if ((e = c.fboxes.ensure(sizeof(NodeBoxF) * (size_t) T, s)) != cudaSuccess) return e;
    if ((e = c.fpairs.ensure(sizeof(NodePairF) * (size_t) L, s)) != cudaSuccess) return e;
    { k_boxes_f32<<<div_up(T, 256), 256, 0, s>>>(c.boxes.as<NodeBox>(), T, c.fboxes.as<NodeBoxF>()); GBSPH_COUNTED; }
    const NodeBoxF *fb = c.fboxes.as<NodeBoxF>();
    const NodePairF *rec = c.fpairs.as<NodePairF>();
    if (L > 1) { k_node_pairs<<<div_up(L - 1, 256), 256, 0, s>>>(t, fb, c.fpairs.as<NodePairF>()); GBSPH_COUNTED; }
    // Owner leaves first: they also record, per leaf, the largest threshold of the rows
    // it owns, which lets stage 1 drop leaves that no owned row can pair with (and skip
    // leaves that own no row); the cache is unchanged.
    if ((e = c.owner.ensure(sizeof(u32) * (size_t) n, s)) != cudaSuccess) return e;
    if ((e = c.leaf_thr.ensure(sizeof(u32) * (size_t) L, s)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(c.leaf_thr.p, 0, sizeof(u32) * (size_t) L, s)) != cudaSuccess) return e;
    u32 *leaf_thr = c.leaf_thr.as<u32>();
    if (n) {
        ProfScope ps(c, kProfOwner, n);
        { k_owner<<<div_up(n, 128), 128, 0, s>>>(t, fb, rec, c.row_rank.as<u32>(), n, c.sx.as<f64>(),
                                               c.sy.as<f64>(), c.sz.as<f64>(), c.owner.as<u32>(),
                                               &dsc->flags, c.sh.as<f64>(), up_f32(h_tol), leaf_thr); GBSPH_COUNTED; }
    }
    auto stage1 = [&]() -> cudaError_t {
        cudaError_t err = c.leaf_ent.ensure(sizeof(uint2) * ((size_t) L * c.leaf_cap + 1), s);
        if (err != cudaSuccess) return err;
        ProfScope ps(c, kProfStage1, L);
        { k_leaf_lists<<<div_up(L, 128), 128, 0, s>>>(t, fb, rec, c.leaf_cnt.as<u32>(), c.leaf_off.as<u32>(),
                                                    c.leaf_ent.as<uint2>(), c.leaf_cap, dsc, leaf_thr); GBSPH_COUNTED; }
        return cudaGetLastError();
    };
    if (s1_one_pass) {
        if ((e = stage1()) != cudaSuccess) return e;
    } else {
        // slots beyond the budget: flag the overflow so the exact build below runs
        const u32 ovf = kFlagLeafCap;
        if ((e = cudaMemcpyAsync(&dsc->flags, &ovf, sizeof(u32), cudaMemcpyHostToDevice, s)) != cudaSuccess) return e;
        if ((e = cudaMemcpyAsync(&dsc->leaf_cnt_max, &c.leaf_cap, sizeof(u32), cudaMemcpyHostToDevice, s)) != cudaSuccess) return e;
    }
    if ((e = sync_scalars(c)) != cudaSuccess) return e;
    if (c.h_scalars->flags & (kFlagStackOverflow | kFlagOwnerMissing)) {
        c.err = "neighbour cache: tree traversal failed (stack overflow or particle outside every leaf box)";
        return cudaErrorUnknown;
    }
    c.leaf_csr_total = 0;
    if (c.h_scalars->flags & kFlagLeafCap) {
        const u32 cap = (c.h_scalars->leaf_cnt_max + 31u) & ~31u;
        const bool fits = s1_one_pass && slots_ok(L, cap, sizeof(uint2));
        if ((e = cudaMemsetAsync(&dsc->flags, 0, sizeof(u32), s)) != cudaSuccess) return e;
        if (fits) {
            // one pass again with slots that hold the largest list
            c.leaf_cap = cap;
            if ((e = stage1()) != cudaSuccess) return e;
        } else {
            // exact two-pass build
            ProfScope ps(c, kProfStage1, 0);
            { k_leaf_count<<<div_up(L, 128), 128, 0, s>>>(t, c.leaf_cnt.as<u32>(), &dsc->flags); GBSPH_COUNTED; }
            if ((e = scan_exclusive_u32(c.leaf_cnt.as<u32>(), c.leaf_off.as<u32>(), L, &dsc->total,
                                        c.scan_scratch, s)) != cudaSuccess)
                return e;
            if ((e = sync_scalars(c)) != cudaSuccess) return e;
            c.leaf_csr_total = c.h_scalars->total;
            if ((e = c.leaf_ent.ensure(sizeof(uint2) * (c.leaf_csr_total + 1), s)) != cudaSuccess) return e;
            { k_leaf_fill<<<div_up(L, 128), 128, 0, s>>>(t, c.leaf_off.as<u32>(), c.leaf_ent.as<uint2>()); GBSPH_COUNTED; }
        }
    }

    if ((e = c.csr_cnt.ensure(sizeof(u32) * ((size_t) n + 1), s)) != cudaSuccess) return e;
    if ((e = c.csr_off.ensure(sizeof(u32) * ((size_t) n + 1), s)) != cudaSuccess) return e;
    // the padded one-pass layout needs row * cap to fit the u32 offsets
    if (c.row_cap == 0) c.row_cap = kRowCap;
    auto slots_fit = [&](u32 cap) { return slots_ok(n, cap); };
    // slots that no longer fit (more rows than before): size them from the largest row
    // of the last build, with a quarter of margin, before falling back to two passes
    if (!slots_fit(c.row_cap) && c.row_seen > 0) {
        const u32 cap = (c.row_seen + c.row_seen / 4 + 7u) & ~3u;
        if (cap < c.row_cap && slots_fit(cap)) c.row_cap = cap;
    }
    bool one_pass = slots_fit(c.row_cap);
    if (one_pass)
        if ((e = c.csr_ent.ensure(sizeof(u32) * ((size_t) n * c.row_cap + 4), s)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(&dsc->csr_entries, 0, sizeof(u64), s)) != cudaSuccess) return e;
    // launch helper for the stage-2 kernel family
    auto part = [&](auto mode_tag, u32 *cnt, u32 *off, u32 *ent) {
        constexpr int MODE = decltype(mode_tag)::value;
        if (P) {
            { k_part_cache<MODE, true><<<div_up(n, 256), 256, 0, s>>>(
                c.row_rank.as<u32>(), n, c.owner.as<u32>(), c.leaf_cnt.as<u32>(),
                c.leaf_off.as<u32>(), c.leaf_ent.as<uint2>(), P, c.sx.as<f64>(),
                c.sy.as<f64>(), c.sz.as<f64>(), c.sh.as<f64>(), h_tol, cnt, off, ent, dsc, c.row_cap); GBSPH_COUNTED; }
        } else {
            { k_part_cache<MODE, false><<<div_up(n, 256), 256, 0, s>>>(
                c.row_rank.as<u32>(), n, c.owner.as<u32>(), c.leaf_cnt.as<u32>(),
                c.leaf_off.as<u32>(), c.leaf_ent.as<uint2>(), nullptr,
                c.sx.as<f64>(), c.sy.as<f64>(), c.sz.as<f64>(), c.sh.as<f64>(), h_tol, cnt, off,
                ent, dsc, c.row_cap); GBSPH_COUNTED; }
        }
    };
    using OnePass = std::integral_constant<int, kOnePass>;
    using Count   = std::integral_constant<int, kCount>;
    using Fill    = std::integral_constant<int, kFill>;
    if (n && one_pass) {
        ProfScope ps(c, kProfCacheFill, n);
        part(OnePass{}, c.csr_cnt.as<u32>(), c.csr_off.as<u32>(), c.csr_ent.as<u32>());
    }
    if ((e = sync_scalars(c)) != cudaSuccess) return e;
    c.csr_total = c.h_scalars->csr_entries;
    if (n && one_pass && (c.h_scalars->flags & kFlagCsrCap)) {
        // a row overflowed: one pass again with slots that hold the largest row
        const u32 cap = (c.h_scalars->row_cnt_max + 3u) & ~3u;
        if (slots_fit(cap)) {
            c.row_cap = cap;
            if ((e = c.csr_ent.ensure(sizeof(u32) * ((size_t) n * cap + 4), s)) != cudaSuccess) return e;
            if ((e = cudaMemsetAsync(&dsc->csr_entries, 0, sizeof(u64), s)) != cudaSuccess) return e;
            if ((e = cudaMemsetAsync(&dsc->flags, 0, sizeof(u32), s)) != cudaSuccess) return e;
            {
                ProfScope ps(c, kProfCacheFill, n);
                part(OnePass{}, c.csr_cnt.as<u32>(), c.csr_off.as<u32>(), c.csr_ent.as<u32>());
            }
            if ((e = sync_scalars(c)) != cudaSuccess) return e;
            c.csr_total = c.h_scalars->csr_entries;
        } else {
            one_pass = false;
        }
    }
    if (n && (!one_pass || (c.h_scalars->flags & kFlagCsrCap))) {
        // slots beyond the budget: exact two-pass build into a compact CSR
        {
            ProfScope ps(c, kProfCacheCount, n);
            part(Count{}, c.csr_cnt.as<u32>(), c.csr_off.as<u32>(), nullptr);
        }
        // rows padded to multiples of 4 entries, scanned in place
        if ((e = scan_exclusive_u32(c.csr_off.as<u32>(), c.csr_off.as<u32>(), n, &dsc->total,
                                    c.scan_scratch, s)) != cudaSuccess)
            return e;
        if ((e = cudaMemsetAsync(&dsc->csr_entries, 0, sizeof(u64), s)) != cudaSuccess) return e;
        if ((e = sync_scalars(c)) != cudaSuccess) return e;
        u64 padded = c.h_scalars->total;
        if ((e = c.csr_ent.ensure(sizeof(u32) * (padded + 4), s)) != cudaSuccess) return e;
        {
            ProfScope ps(c, kProfCacheFill, 0);
            part(Fill{}, nullptr, c.csr_off.as<u32>(), c.csr_ent.as<u32>());
        }
        if ((e = sync_scalars(c)) != cudaSuccess) return e;
        c.csr_total = c.h_scalars->csr_entries;
    }
    c.row_seen    = c.h_scalars->row_cnt_max;
    c.cache_valid = true;
    return cudaGetLastError();
}

cudaError_t tree_query(Ctx &c, const f64 *qx, const f64 *qy, const f64 *qz, u32 nq, int mode,
                       f64 s, u32 *counts, u32 *offsets, u32 *out, bool fill) {
    TreeView t = view(c);
    Scalars *dsc = c.d_scalars.as<Scalars>();
    if (fill)
        { k_query<true><<<div_up(nq, 128), 128, 0, c.stream>>>(
            t, qx, qy, qz, nq, mode, s, c.sort_index.as<u32>(), c.sx.as<f64>(), c.sy.as<f64>(),
            c.sz.as<f64>(), nullptr, offsets, out, &dsc->flags); GBSPH_COUNTED; }
    else
        { k_query<false><<<div_up(nq, 128), 128, 0, c.stream>>>(
            t, qx, qy, qz, nq, mode, s, c.sort_index.as<u32>(), c.sx.as<f64>(), c.sy.as<f64>(),
            c.sz.as<f64>(), counts, nullptr, nullptr, &dsc->flags); GBSPH_COUNTED; }
    return cudaGetLastError();
}

} // namespace gbsph
