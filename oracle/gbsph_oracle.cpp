// ORACLE — TEST INFRASTRUCTURE ONLY.
//
// CPU FP64 restatement of the Shamrock SPH timestep hot path (Morton keys, bitonic
// sort, leaf reduction, Karras radix tree, tree AABB / interaction-radius fields,
// two-stage neighbour cache, h-rho Newton iteration, Omega, adiabatic EOS,
// constant-AV derivatives, v_sig / CFL, leapfrog KDK with corrector, periodic
// ghosts).  Only the test suite, the smoke check and the CPU-baseline leg of the
// benchmark load this library, as the checker; the product path never does.
//
// Evaluation-order contract (shared with the FP64 CUDA path, which is compiled with
// fused multiply-add disabled): every expression is evaluated left to right exactly
// as written in the cited reference line, dot products as x*x + y*y + z*z, and this
// file is compiled with -ffp-contract=off.
//
// Pinned against the reference's own golden vectors (Morton codes, sorted codes and
// sort permutation, reduced set, Karras topology, ordered object-iterator lists,
// h-iteration sequences, kernel identities); see tests/golden/.
//
// All citations are paths inside the Shamrock source tree.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef uint8_t u8;
typedef uint32_t u32;
typedef uint64_t u64;
typedef int32_t i32;
typedef int64_t i64;
typedef double f64;

namespace orc {

// =================================================================================
// bit helpers
// =================================================================================

// sycl::clz semantics: clz(0) == bit width (shambackends/math.hpp:742-783)
inline int clz_key(u32 v) { return v == 0 ? 32 : __builtin_clz(v); }
inline int clz_key(u64 v) { return v == 0 ? 64 : __builtin_clzll(v); }

// shammath/sfc/bmi.hpp:43-51 (10-bit value, two zero bits between payload bits)
inline u32 expand_bits_10(u32 x) {
    x &= 0x3ffU;
    x = (x | x << 16U) & 0x30000ffU;
    x = (x | x << 8U) & 0x300f00fU;
    x = (x | x << 4U) & 0x30c30c3U;
    x = (x | x << 2U) & 0x9249249U;
    return x;
}
// shammath/sfc/bmi.hpp:31-40 (21-bit value)
inline u64 expand_bits_21(u64 x) {
    x &= 0x1fffffULL;
    x = (x | x << 32ULL) & 0x1f00000000ffffULL;
    x = (x | x << 16ULL) & 0x1f0000ff0000ffULL;
    x = (x | x << 8ULL) & 0x100f00f00f00f00fULL;
    x = (x | x << 4ULL) & 0x10c30c30c30c30c3ULL;
    x = (x | x << 2ULL) & 0x1249249249249249ULL;
    return x;
}

template<class K>
struct MortonTraits;
// shammath/sfc/morton.hpp:46-112 (MortonCodes<u32,3>): 10 bits per axis, grid 1024
template<>
struct MortonTraits<u32> {
    static constexpr u32 val_count = 1024;
    static constexpr u32 max_val   = 1023;
    static constexpr u32 err_code  = 0xFFFFFFFFu;
    static inline u32 encode(u32 x, u32 y, u32 z) {
        return expand_bits_10(x) * 4 + expand_bits_10(y) * 2 + expand_bits_10(z);
    }
};
// shammath/sfc/morton.hpp:114-180 (MortonCodes<u64,3>): 21 bits per axis
template<>
struct MortonTraits<u64> {
    static constexpr u32 val_count = 2097152;
    static constexpr u32 max_val   = 2097151;
    static constexpr u64 err_code  = 0xFFFFFFFFFFFFFFFFull;
    static inline u64 encode(u64 x, u64 y, u64 z) {
        return expand_bits_21(x) * 4 + expand_bits_21(y) * 2 + expand_bits_21(z);
    }
};

// =================================================================================
// Morton code set — shamtree/src/MortonCodeSet.cpp:63-118
//   position clamped to the AABB (shammath/AABB.hpp:320-322, sycl::clamp),
//   grid = static_cast of (p - bmin) / fact with fact = (bmax - bmin) / val_count
//   (shammath/src/CoordRangeTransform.cpp:169-184, CoordRangeTransform.hpp:114-122),
//   clamped to max_val (morton.hpp:213-224), interleaved x*4 + y*2 + z;
//   slots [n, morton_count) padded with err_code (MortonCodeSet.cpp:101-111).
// =================================================================================
template<class K>
void morton_codes(
    const f64 *pos, u32 n, u32 morton_count, const f64 *bmin, const f64 *bmax, K *out) {
    f64 fact[3];
    for (int c = 0; c < 3; c++) {
        fact[c] = (bmax[c] - bmin[c]) / (f64) MortonTraits<K>::val_count;
    }
#pragma omp parallel for schedule(static)
    for (i64 i = 0; i < (i64) n; i++) {
        u32 g[3];
        for (int c = 0; c < 3; c++) {
            f64 r = std::fmin(std::fmax(pos[3 * i + c], bmin[c]), bmax[c]);
            u32 gi = (u32) ((r - bmin[c]) / fact[c]);
            g[c]   = std::min(gi, MortonTraits<K>::max_val);
        }
        out[i] = MortonTraits<K>::encode(g[0], g[1], g[2]);
    }
    for (u32 i = n; i < morton_count; i++) {
        out[i] = MortonTraits<K>::err_code;
    }
}

// =================================================================================
// Bitonic key/value sort — shamalgs/src/details/algorithm/bitonicSort_updated_usm.cpp
//   compare-exchange (:29-39): swap = reverse ^ (a < b); direction
//   reverse = ((length << 1) & i) == 0 with i the lower index of the pair;
//   stage loop (:298-395): for length = 1,2,4..<len, for inc = length..1.
// The stencil kernels (:146-281) fuse several inc levels per pass; they execute the
// same compare-exchange network, so the plain per-stage form below is the same
// function (bitonic_sort_stencil16 re-creates the fused form to show it).
// =================================================================================
template<class K>
void bitonic_sort(K *keys, u32 *vals, u32 len) {
    for (u32 length = 1; length < len; length <<= 1) {
        for (u32 inc = length; inc > 0; inc >>= 1) {
#pragma omp parallel for schedule(static)
            for (i64 t = 0; t < (i64) (len / 2); t++) {
                u32 low      = (u32) t & (inc - 1);
                u32 i        = ((u32) t << 1) - low;
                bool reverse = ((length << 1) & i) == 0;
                K a = keys[i], b = keys[i + inc];
                bool swap = reverse ^ (a < b);
                if (swap) {
                    keys[i]       = b;
                    keys[i + inc] = a;
                    u32 tv        = vals[i];
                    vals[i]       = vals[i + inc];
                    vals[i + inc] = tv;
                }
            }
        }
    }
}

// The reference's fused-stencil pass structure (bitonicSort_updated_usm.cpp:146-281,
// 298-395 with MaxStencilSize 16), restated to check the equivalence claim above.
template<class K>
static void order_pair(K *x, u32 *v, u32 a, u32 b, bool reverse) {
    bool swap = reverse ^ (x[a] < x[b]);
    if (swap) {
        std::swap(x[a], x[b]);
        std::swap(v[a], v[b]);
    }
}
template<class K>
static void order_stencil(K *x, u32 *v, u32 base, u32 size, bool reverse) {
    if (size < 2) return;
    u32 half = size / 2;
    for (u32 k = 0; k < half; k++) order_pair(x, v, base + k, base + k + half, reverse);
    order_stencil(x, v, base, half, reverse);
    order_stencil(x, v, base + half, half, reverse);
}
template<class K>
void bitonic_sort_stencil16(K *m, u32 *id, u32 len) {
    for (u32 length = 1; length < len; length <<= 1) {
        u32 inc = length;
        while (inc > 0) {
            u32 ninc = 0;
            if (inc >= 8) ninc = 4;
            else if (inc >= 4) ninc = 3;
            else if (inc >= 2) ninc = 2;
            else ninc = 1;
            u32 stencil  = 1u << ninc;
            u32 nthreads = len >> ninc;
            u32 sub_inc  = inc >> (ninc - 1);
#pragma omp parallel for schedule(static)
            for (i64 tt = 0; tt < (i64) nthreads; tt++) {
                i32 t        = (i32) tt;
                i32 low      = t & (i32) (sub_inc - 1);
                i32 i        = ((t - low) << ninc) + low;
                bool reverse = (((length << 1) & (u32) i) == 0);
                K x[16];
                u32 v[16];
                for (u32 k = 0; k < stencil; k++) {
                    x[k] = m[k * sub_inc + i];
                    v[k] = id[k * sub_inc + i];
                }
                order_stencil(x, v, 0, stencil, reverse);
                for (u32 k = 0; k < stencil; k++) {
                    m[k * sub_inc + i]  = x[k];
                    id[k * sub_inc + i] = v[k];
                }
            }
            inc >>= ninc;
        }
    }
}

// =================================================================================
// Karras delta — shambackends/math.hpp:826-828.  The y bound test compares y as
// unsigned against morton_length - 1, so any y outside [0, len) yields -1.
// =================================================================================
template<class K>
inline i32 karras_delta(i32 x, i32 y, u32 len, const K *m) {
    if ((u32) y > len - 1 || y < 0) return -1;
    return clz_key((K) (m[x] ^ m[y]));
}

// =================================================================================
// Leaf reduction — shamtree/src/kernels/reduction_alg.cpp
//   split table (:62-85), reduction iteration (:196-244), ping-pong over
//   reduction_level iterations (:413-456), stream compaction + tail
//   [..., morton_count, 0] (:274-295, :357-373).  morton_count here is the object
//   count (MortonReducedSet.cpp:34-38 passes cnt_obj).
// =================================================================================
template<class K>
u32 reduction_alg(const K *m, u32 cnt, u32 level, std::vector<u32> &reduc_index_map) {
    std::vector<u32> s1(cnt), s2(cnt);
    for (u32 i = 0; i < cnt; i++) {
        s1[i] = (i > 0) ? ((m[i - 1] != m[i]) ? 1 : 0) : 1;
    }
    for (u32 iter = 1; iter <= level; iter++) {
        const std::vector<u32> &in = (iter % 2 == 0) ? s2 : s1;
        std::vector<u32> &out      = (iter % 2 == 0) ? s1 : s2;
#pragma omp parallel for schedule(static)
        for (i64 ii = 0; ii < (i64) cnt; ii++) {
            u32 i       = (u32) ii;
            u32 before1 = i - 1;
            while (before1 <= cnt - 1 && !in[before1]) before1--;
            u32 before2 = before1 - 1;
            while (before2 <= cnt - 1 && !in[before2]) before2--;
            u32 next1 = i + 1;
            while (next1 <= cnt - 1 && !in[next1]) next1++;
            i32 delt_0  = karras_delta((i32) i, (i32) next1, cnt, m);
            i32 delt_m  = karras_delta((i32) i, (i32) before1, cnt, m);
            i32 delt_mm = karras_delta((i32) before1, (i32) before2, cnt, m);
            out[i] = (!(delt_0 < delt_m && delt_mm < delt_m) && in[i]) ? 1 : 0;
        }
    }
    const std::vector<u32> &fin = (level % 2 == 0) ? s1 : s2;
    reduc_index_map.clear();
    for (u32 i = 0; i < cnt; i++) {
        if (fin[i]) reduc_index_map.push_back(i);
    }
    u32 leaves = (u32) reduc_index_map.size();
    reduc_index_map.push_back(cnt);
    reduc_index_map.push_back(0);
    return leaves;
}

// =================================================================================
// Karras 2012 radix tree — shamtree/src/KarrasRadixTree.cpp:45-143
// =================================================================================
template<class K>
void karras_tree(
    const K *m, u32 L, u32 *lchild, u32 *rchild, u8 *lflag, u8 *rflag, u32 *endrange) {
    if (L <= 1) return;
    u32 internal = L - 1;
#pragma omp parallel for schedule(static)
    for (i64 ii = 0; ii < (i64) internal; ii++) {
        i32 i       = (i32) ii;
        auto DELTA  = [&](i32 x, i32 y) { return karras_delta(x, y, L, m); };
        i32 ddelta  = DELTA(i, i + 1) - DELTA(i, i - 1);
        i32 d       = (ddelta == 0) ? 0 : ((ddelta > 0) ? 1 : -1);
        i32 delta_min = DELTA(i, i - d);
        i32 lmax      = 2;
        while (DELTA(i, i + lmax * d) > delta_min) lmax *= 2;
        i32 l = 0;
        i32 t = lmax / 2;
        while (t > 0) {
            if (DELTA(i, i + (l + t) * d) > delta_min) l = l + t;
            t = t / 2;
        }
        u32 j           = (u32) (i + l * d);
        endrange[i]     = j;
        i32 delta_node  = DELTA(i, (i32) j);
        i32 s           = 0;
        float div       = 2;
        t               = (i32) std::ceil((float) l / div);
        while (true) {
            i32 tmp_ = i + (s + t) * d;
            if (DELTA(i, tmp_) > delta_node) s = s + t;
            if (t <= 1) break;
            div *= 2;
            t = (i32) std::ceil((float) l / div);
        }
        i32 gamma  = i + s * d + std::min(d, 0);
        u32 ui     = (u32) i;
        lchild[i]  = (u32) gamma;
        lflag[i]   = (std::min(ui, j) == (u32) gamma) ? 1 : 0;
        rchild[i]  = (u32) (gamma + 1);
        rflag[i]   = (std::max(ui, j) == (u32) (gamma + 1)) ? 1 : 0;
    }
}

// =================================================================================
// CompressedLeafBVH — shamtree/src/CompressedLeafBVH.cpp:32-95
//   morton set over roundup_pow2(n) slots, sort, reduce, Karras, then
//   leaf AABBs from member positions (KarrasRadixTreeAABB.cpp:92-140, init +/-max)
//   and bottom-up union (the reference's tree_depth Jacobi passes :33-73 converge to
//   the exact subtree min/max).  Node numbering: internal [0, L-1), leaves at
//   offset L-1 (KarrasTreeTraverser.hpp:46-64).
// =================================================================================
inline u32 roundup_pow2(u32 v) {
    u32 p = 1;
    while (p < v) p <<= 1;
    return p;
}

struct Tree {
    int key_bits = 32;
    u32 n_obj = 0, morton_count = 0, leaf_count = 0;
    std::vector<u64> sorted_keys;  // [P] (u32 keys widened)
    std::vector<u32> sort_index;   // [P]
    std::vector<u32> reduc;        // [L+2]
    std::vector<u64> reduced;      // [L]
    std::vector<u32> lchild, rchild, endrange;
    std::vector<u8> lflag, rflag;
    std::vector<f64> bmin, bmax;   // 3*(2L-1)
    std::vector<f64> rint;         // 2L-1 (optional)

    u32 offset_leaf() const { return leaf_count - 1; }
    u32 total_nodes() const { return 2 * leaf_count - 1; }
    bool is_leaf(u32 id) const { return id >= offset_leaf(); }
    u32 left(u32 id) const { return lchild[id] + offset_leaf() * (u32) lflag[id]; }
    u32 right(u32 id) const { return rchild[id] + offset_leaf() * (u32) rflag[id]; }

    // stack DFS, left child first (KarrasTreeTraverser.hpp:70-118)
    template<class Crit, class Leaf>
    void traverse(Crit &&crit, Leaf &&on_leaf) const {
        u32 stack[70];
        int top      = 0;
        stack[top++] = 0;
        while (top > 0) {
            u32 node = stack[--top];
            if (crit(node)) {
                if (is_leaf(node)) {
                    on_leaf(node);
                } else {
                    stack[top++] = right(node);
                    stack[top++] = left(node);
                }
            }
        }
    }
};

template<class K>
void build_tree_impl(
    Tree &t, const f64 *pos, const f64 *h, u32 n, const f64 *bmin, const f64 *bmax, u32 level,
    f64 htol, u32 morton_count = 0) {
    t.key_bits     = (int) (sizeof(K) * 8);
    t.n_obj        = n;
    t.morton_count = morton_count ? morton_count : roundup_pow2(n);
    u32 P          = t.morton_count;
    std::vector<K> keys(P);
    morton_codes<K>(pos, n, P, bmin, bmax, keys.data());
    t.sort_index.resize(P);
    for (u32 i = 0; i < P; i++) t.sort_index[i] = i;
    bitonic_sort<K>(keys.data(), t.sort_index.data(), P);
    t.sorted_keys.assign(keys.begin(), keys.end());
    t.leaf_count = reduction_alg<K>(keys.data(), n, level, t.reduc);
    u32 L        = t.leaf_count;
    std::vector<K> red(L);
    for (u32 l = 0; l < L; l++) red[l] = keys[t.reduc[l]];
    t.reduced.assign(red.begin(), red.end());
    u32 I = (L > 0) ? L - 1 : 0;
    t.lchild.assign(I, 0);
    t.rchild.assign(I, 0);
    t.endrange.assign(I, 0);
    t.lflag.assign(I, 0);
    t.rflag.assign(I, 0);
    karras_tree<K>(red.data(), L, t.lchild.data(), t.rchild.data(), t.lflag.data(), t.rflag.data(),
                   t.endrange.data());

    u32 T = 2 * L - 1;
    t.bmin.assign(3 * (size_t) T, 0);
    t.bmax.assign(3 * (size_t) T, 0);
    t.rint.assign(T, 0);
    u32 off = I;
    const f64 fmax = std::numeric_limits<f64>::max();
#pragma omp parallel for schedule(static)
    for (i64 ll = 0; ll < (i64) L; ll++) {
        u32 l = (u32) ll;
        f64 lo[3] = {fmax, fmax, fmax}, hi[3] = {-fmax, -fmax, -fmax};
        f64 hm = std::numeric_limits<f64>::lowest();
        for (u32 s = t.reduc[l]; s < t.reduc[l + 1]; s++) {
            u32 id = t.sort_index[s];
            for (int c = 0; c < 3; c++) {
                lo[c] = std::fmin(lo[c], pos[3 * id + c]);
                hi[c] = std::fmax(hi[c], pos[3 * id + c]);
            }
            if (h) hm = std::fmax(hm, h[id]);
        }
        for (int c = 0; c < 3; c++) {
            t.bmin[3 * (off + l) + c] = lo[c];
            t.bmax[3 * (off + l) + c] = hi[c];
        }
        t.rint[off + l] = hm;
    }
    // bottom-up: internal node ids are not topologically ordered, recurse from root
    if (I > 0) {
        std::vector<u32> order;
        order.reserve(I);
        std::vector<u32> st;
        st.push_back(0);
        while (!st.empty()) {
            u32 nd = st.back();
            st.pop_back();
            order.push_back(nd);
            u32 a = t.left(nd), b = t.right(nd);
            if (!t.is_leaf(a)) st.push_back(a);
            if (!t.is_leaf(b)) st.push_back(b);
        }
        for (size_t k = order.size(); k-- > 0;) {
            u32 nd = order[k];
            u32 a = t.left(nd), b = t.right(nd);
            for (int c = 0; c < 3; c++) {
                t.bmin[3 * nd + c] = std::fmin(t.bmin[3 * a + c], t.bmin[3 * b + c]);
                t.bmax[3 * nd + c] = std::fmax(t.bmax[3 * a + c], t.bmax[3 * b + c]);
            }
            t.rint[nd] = std::fmax(t.rint[a], t.rint[b]);
        }
    }
    // interaction radius field x htol (shammodels/sph/src/Solver.cpp:1322-1356)
    if (h) {
        for (u32 k = 0; k < T; k++) t.rint[k] *= htol;
    }
}

// =================================================================================
// Neighbour cache, two stages —
//   shammodels/sph/src/modules/NeighbourCache.cpp:223-596,
//   ObjectCache/prepare_object_cache shamtree/include/shamtree/TreeTraversal.hpp:375-485,
//   cella_neigh_b / is_coord_in_range_incl_max
//   shamtree/include/shamtree/kernels/geometry_utils.hpp:62-135
// =================================================================================
inline bool cella_neigh_b(const f64 *amin, const f64 *amax, const f64 *bmin, const f64 *bmax) {
    return (std::fmax(amin[0], bmin[0]) <= std::fmin(amax[0], bmax[0]))
           && (std::fmax(amin[1], bmin[1]) <= std::fmin(amax[1], bmax[1]))
           && (std::fmax(amin[2], bmin[2]) <= std::fmin(amax[2], bmax[2]));
}
inline bool coord_in_incl(const f64 *p, const f64 *lo, const f64 *hi) {
    return (lo[0] <= p[0]) && (p[0] <= hi[0]) && (lo[1] <= p[1]) && (p[1] <= hi[1])
           && (lo[2] <= p[2]) && (p[2] <= hi[2]);
}

struct CSR {
    std::vector<u32> cnt, scanned, entries;
    u64 total = 0;
    void finish_counts() {
        scanned.resize(cnt.size());
        u64 acc = 0;
        for (size_t i = 0; i < cnt.size(); i++) {
            scanned[i] = (u32) acc;
            acc += cnt[i];
        }
        total = acc;
        entries.assign(total, 0);
    }
};

struct NeighCache {
    CSR leaf;                  // stage 1: leaf -> leaf node ids
    std::vector<u32> owner;    // local particle -> leaf id
    CSR part;                  // stage 2: local particle -> merged ids
};

static const f64 Rkern = 2.0; // KernelDefM4::Rkern, shammath/sphkernels.hpp:31

void neigh_cache(
    const Tree &t, const f64 *xyz, const f64 *h, u32 n_local, f64 h_tolerance, NeighCache &nc) {
    u32 L   = t.leaf_count;
    u32 off = t.offset_leaf();
    auto leaf_crit = [&](u32 l, u32 node) {
        f64 ra = t.rint[off + l] * Rkern;
        const f64 *amin = &t.bmin[3 * (off + l)], *amax = &t.bmax[3 * (off + l)];
        f64 amin_ext[3], amax_ext[3];
        for (int c = 0; c < 3; c++) {
            amin_ext[c] = amin[c] - ra;
            amax_ext[c] = amax[c] + ra;
        }
        f64 rn = t.rint[node] * Rkern;
        const f64 *nmin = &t.bmin[3 * node], *nmax = &t.bmax[3 * node];
        f64 ext_min[3], ext_max[3];
        for (int c = 0; c < 3; c++) {
            ext_min[c] = nmin[c] - rn;
            ext_max[c] = nmax[c] + rn;
        }
        return cella_neigh_b(amin, amax, ext_min, ext_max)
               || cella_neigh_b(amin_ext, amax_ext, nmin, nmax);
    };
    nc.leaf.cnt.assign(L, 0);
#pragma omp parallel for schedule(dynamic, 256)
    for (i64 ll = 0; ll < (i64) L; ll++) {
        u32 l = (u32) ll, c = 0;
        t.traverse([&](u32 node) { return leaf_crit(l, node); }, [&](u32) { c++; });
        nc.leaf.cnt[l] = c;
    }
    nc.leaf.finish_counts();
#pragma omp parallel for schedule(dynamic, 256)
    for (i64 ll = 0; ll < (i64) L; ll++) {
        u32 l = (u32) ll, c = nc.leaf.scanned[l];
        t.traverse([&](u32 node) { return leaf_crit(l, node); },
                   [&](u32 node) { nc.leaf.entries[c++] = node; });
    }
    // particle -> parent leaf: last leaf found in DFS order (NeighbourCache.cpp:419-443)
    nc.owner.assign(n_local, 0);
#pragma omp parallel for schedule(dynamic, 1024)
    for (i64 ii = 0; ii < (i64) n_local; ii++) {
        const f64 *p = &xyz[3 * ii];
        u32 found    = 2147483647u;
        t.traverse([&](u32 node) { return coord_in_incl(p, &t.bmin[3 * node], &t.bmax[3 * node]); },
                   [&](u32 node) { found = node - off; });
        nc.owner[ii] = found;
    }
    const f64 Rker2 = Rkern * Rkern;
    auto for_each_candidate = [&](u32 a, auto &&fn) {
        u32 lo = nc.leaf.scanned[nc.owner[a]];
        u32 hi = lo + nc.leaf.cnt[nc.owner[a]];
        for (u32 k = lo; k < hi; k++) {
            u32 lb = nc.leaf.entries[k] - off;
            for (u32 s = t.reduc[lb]; s < t.reduc[lb + 1]; s++) fn(t.sort_index[s]);
        }
    };
    auto interact = [&](u32 a, u32 b) {
        f64 rint_a = h[a] * h_tolerance;
        f64 dx = xyz[3 * a] - xyz[3 * b], dy = xyz[3 * a + 1] - xyz[3 * b + 1],
            dz = xyz[3 * a + 2] - xyz[3 * b + 2];
        f64 rab2   = dx * dx + dy * dy + dz * dz;
        f64 rint_b = h[b] * h_tolerance;
        bool no_interact = rab2 > rint_a * rint_a * Rker2 && rab2 > rint_b * rint_b * Rker2;
        return !no_interact;
    };
    nc.part.cnt.assign(n_local, 0);
#pragma omp parallel for schedule(dynamic, 1024)
    for (i64 ii = 0; ii < (i64) n_local; ii++) {
        u32 a = (u32) ii, c = 0;
        for_each_candidate(a, [&](u32 b) { c += interact(a, b) ? 1 : 0; });
        nc.part.cnt[a] = c;
    }
    nc.part.finish_counts();
#pragma omp parallel for schedule(dynamic, 1024)
    for (i64 ii = 0; ii < (i64) n_local; ii++) {
        u32 a = (u32) ii, c = nc.part.scanned[a];
        for_each_candidate(a, [&](u32 b) {
            if (interact(a, b)) nc.part.entries[c++] = b;
        });
    }
}

// =================================================================================
// M4 cubic spline — shammath/include/shammath/sphkernels.hpp:29-72, 2286-2343
// =================================================================================
static const f64 norm_3d = 1 / 3.141592653589793; // KernelDefM4::norm_3d
static const f64 hfactd  = 1.2;                   // KernelDefM4::hfactd

inline f64 m4_f(f64 q) {
    f64 t1 = 2 - q;
    f64 t2 = 1 - q;
    t1     = t1 * t1 * t1;
    t2     = t2 * t2 * t2;
    const f64 div1_4 = (1. / 4.);
    t1 *= div1_4;
    t2 *= -1;
    if (q < 1) return t1 + t2;
    else if (q < 2) return t1;
    return 0;
}
inline f64 m4_df(f64 q) {
    const f64 div9_4 = (9. / 4.);
    const f64 div3_4 = (3. / 4.);
    if (q < 1) return -3 * q + div9_4 * q * q;
    else if (q < 2) return -3 + 3 * q - div3_4 * q * q;
    return 0;
}
inline f64 W_3d(f64 r, f64 h) { return norm_3d * m4_f(r / h) / (h * h * h); }
inline f64 dW_3d(f64 r, f64 h) { return norm_3d * m4_df(r / h) / (h * h * h * h); }
inline f64 dhW_3d(f64 r, f64 h) {
    return -(norm_3d) * (3 * m4_f(r / h) + (r / h) * m4_df(r / h)) / (h * h * h * h);
}

// shammodels/sph/include/shammodels/sph/math/density.hpp:22-41
inline f64 rho_h(f64 m, f64 h, f64 hfact) { return m * (hfact / h) * (hfact / h) * (hfact / h); }
inline f64 newton_iterate_new_h(f64 rho_ha, f64 rho_sum, f64 sumdWdh, f64 h_a) {
    f64 f_iter  = rho_sum - rho_ha;
    f64 df_iter = sumdWdh + 3 * rho_ha / h_a;
    return h_a - f_iter / df_iter;
}

// =================================================================================
// One h-rho Newton iteration —
//   shammodels/sph/src/modules/IterateSmoothingLengthDensity.cpp:52-119
// =================================================================================
void h_iterate_once(
    u32 n_local, const u32 *cnt, const u32 *scanned, const u32 *entries, const f64 *r,
    const f64 *h_old, f64 *h_new, f64 *eps, f64 pmass, f64 h_evol_max, f64 h_evol_iter_max) {
    const f64 h_max_tot_max_evol = h_evol_max;
    const f64 h_max_evol_p       = h_evol_iter_max;
    const f64 h_max_evol_m       = 1 / h_evol_iter_max;
#pragma omp parallel for schedule(dynamic, 1024)
    for (i64 ii = 0; ii < (i64) n_local; ii++) {
        u32 a = (u32) ii;
        if (!(eps[a] > 1e-6)) continue;
        f64 h_a  = h_new[a];
        f64 dint = h_a * h_a * Rkern * Rkern;
        f64 rho_sum = 0, sumdWdh = 0;
        for (u32 k = scanned[a]; k < scanned[a] + cnt[a]; k++) {
            u32 b  = entries[k];
            f64 dx = r[3 * a] - r[3 * b], dy = r[3 * a + 1] - r[3 * b + 1],
                dz = r[3 * a + 2] - r[3 * b + 2];
            f64 rab2 = dx * dx + dy * dy + dz * dz;
            if (rab2 > dint) continue;
            f64 rab = std::sqrt(rab2);
            rho_sum += pmass * W_3d(rab, h_a);
            sumdWdh += pmass * dhW_3d(rab, h_a);
        }
        f64 rho_ha = rho_h(pmass, h_a, hfactd);
        f64 new_h  = newton_iterate_new_h(rho_ha, rho_sum, sumdWdh, h_a);
        if (new_h < h_a * h_max_evol_m) new_h = h_max_evol_m * h_a;
        if (new_h > h_a * h_max_evol_p) new_h = h_max_evol_p * h_a;
        f64 ha_0 = h_old[a];
        if (new_h < ha_0 * h_max_tot_max_evol) {
            h_new[a] = new_h;
            eps[a]   = std::fabs(new_h - h_a) / ha_0;
        } else {
            h_new[a] = ha_0 * h_max_tot_max_evol;
            eps[a]   = -1;
        }
    }
}

// Omega — shammodels/sph/src/modules/ComputeOmega.cpp:36-73
void compute_omega(
    u32 n_local, const u32 *cnt, const u32 *scanned, const u32 *entries, const f64 *r,
    const f64 *h, f64 pmass, f64 *omega) {
#pragma omp parallel for schedule(dynamic, 1024)
    for (i64 ii = 0; ii < (i64) n_local; ii++) {
        u32 a    = (u32) ii;
        f64 h_a  = h[a];
        f64 dint = h_a * h_a * Rkern * Rkern;
        f64 rho_sum = 0, part_omega_sum = 0;
        for (u32 k = scanned[a]; k < scanned[a] + cnt[a]; k++) {
            u32 b  = entries[k];
            f64 dx = r[3 * a] - r[3 * b], dy = r[3 * a + 1] - r[3 * b + 1],
                dz = r[3 * a + 2] - r[3 * b + 2];
            f64 rab2 = dx * dx + dy * dy + dz * dz;
            if (rab2 > dint) continue;
            f64 rab = std::sqrt(rab2);
            rho_sum += pmass * W_3d(rab, h_a);
            part_omega_sum += pmass * dhW_3d(rab, h_a);
        }
        f64 rho_ha  = rho_h(pmass, h_a, hfactd);
        f64 omega_a = 1 + (h_a / (3 * rho_ha)) * part_omega_sum;
        omega[a]    = omega_a;
    }
}

// Adiabatic EOS from h — shammodels/common ComputeEOSAdiabatic
//   (shammodels/sph/src/modules/ComputeEos.cpp:162-172, 219-236;
//    shamphys/include/shamphys/eos.hpp:45-54)
void eos_adiabatic(u32 n, const f64 *h, const f64 *u, f64 pmass, f64 gamma, f64 *P, f64 *cs) {
#pragma omp parallel for schedule(static)
    for (i64 i = 0; i < (i64) n; i++) {
        f64 rho = rho_h(pmass, h[i], hfactd);
        f64 Pa  = (gamma - 1) * rho * u[i];
        P[i]    = Pa;
        cs[i]   = std::sqrt(gamma * Pa / rho);
    }
}

// Locally isothermal EOS (LP07) — shammodels/sph/src/modules/ComputeEos.cpp:725-798,
// shamphys/include/shamphys/eos.hpp:87-98: c_s^2 = cs0^2 (R^2 / r0^2)^(-q) at the merged
// position R, P = c_s^2 rho.
void eos_locally_isothermal(u32 n, const f64 *xyz, const f64 *h, f64 pmass, f64 cs0, f64 r0,
                            f64 q, f64 *P, f64 *cs) {
    const f64 r0sq = r0 * r0, mq = -q;
#pragma omp parallel for schedule(static)
    for (i64 i = 0; i < (i64) n; i++) {
        f64 x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
        f64 Rsq   = x * x + y * y + z * z;
        f64 cs_sq = (cs0 * cs0) * std::pow(Rsq / r0sq, mq);
        f64 rho   = rho_h(pmass, h[i], hfactd);
        P[i]      = cs_sq * rho;
        cs[i]     = std::sqrt(cs_sq);
    }
}

// Central point mass at the origin — shammodels/common/src/modules/AddForceCentralGravPotential.cpp:37-48:
// a_ext = (-M G) r / |r|^3, evaluated after the predictor's drift (ExternalForces.cpp,
// compute_ext_forces_indep_v, called from Solver.cpp:2035) and added to the hydro
// acceleration of every corrector evaluation (ExternalForces.cpp:342-359).
void point_mass_accel(u32 n, const f64 *xyz, f64 central_mass, f64 G, f64 *aext) {
    const f64 mGM = -central_mass * G;
    for (u32 i = 0; i < n; i++) {
        f64 x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
        f64 r   = std::sqrt(x * x + y * y + z * z);
        f64 r3  = r * r * r;
        aext[3 * i]     = mGM * x / r3;
        aext[3 * i + 1] = mGM * y / r3;
        aext[3 * i + 2] = mGM * z / r3;
    }
}

inline f64 inv_sat_positive(f64 v) { return (v >= 1e-9) ? 1. / v : 0.; }
inline f64 inv_sat_zero(f64 v) { return (v != 0 && v == v) ? 1. / v : 0.; }

// Constant-AV derivatives —
//   shammodels/sph/src/modules/UpdateDerivs.cpp:176-271,
//   shammodels/sph/include/shammodels/sph/math/forces.hpp:24-226, q_ab.hpp:36-39
void derivs_constAV(
    u32 n_local, const u32 *cnt, const u32 *scanned, const u32 *entries, const f64 *xyz,
    const f64 *vxyz, const f64 *hpart, const f64 *omega, const f64 *u, const f64 *pressure,
    const f64 *cs, f64 pmass, f64 alpha_u, f64 alpha_AV, f64 beta_AV, f64 *axyz, f64 *du,
    const f64 *alpha = nullptr) {
    // alpha (merged index space) != null: the varying-AV form, alpha_a and alpha_b per
    // particle (NodeUpdateDerivsVaryingAlphaAV.cpp:45-125), otherwise alpha_AV for both
    const f64 Rker2 = Rkern * Rkern;
#pragma omp parallel for schedule(dynamic, 1024)
    for (i64 ii = 0; ii < (i64) n_local; ii++) {
        u32 a = (u32) ii;
        f64 h_a = hpart[a];
        const f64 *xa = &xyz[3 * a], *va = &vxyz[3 * a];
        f64 P_a = pressure[a], omega_a = omega[a];
        const f64 u_a = u[a];
        f64 rho_a             = rho_h(pmass, h_a, hfactd);
        f64 rho_a_sq          = rho_a * rho_a;
        f64 rho_a_inv         = 1. / rho_a;
        f64 omega_a_rho_a_inv = 1 / (omega_a * rho_a);
        f64 cs_a              = cs[a];
        const f64 alpha_a     = alpha ? alpha[a] : alpha_AV;
        f64 fx = 0, fy = 0, fz = 0, tdu = 0;
        for (u32 k = scanned[a]; k < scanned[a] + cnt[a]; k++) {
            u32 b    = entries[k];
            f64 dx   = xa[0] - xyz[3 * b], dy = xa[1] - xyz[3 * b + 1],
                dz   = xa[2] - xyz[3 * b + 2];
            f64 rab2 = dx * dx + dy * dy + dz * dz;
            f64 h_b  = hpart[b];
            if (rab2 > h_a * h_a * Rker2 && rab2 > h_b * h_b * Rker2) continue;
            f64 rab       = std::sqrt(rab2);
            const f64 u_b = u[b];
            f64 rho_b   = rho_h(pmass, h_b, hfactd);
            f64 P_b     = pressure[b];
            f64 omega_b = omega[b];
            f64 cs_b    = cs[b];
            f64 Fab_a   = dW_3d(rab, h_a);
            f64 Fab_b   = dW_3d(rab, h_b);
            f64 vx = va[0] - vxyz[3 * b], vy = va[1] - vxyz[3 * b + 1], vz = va[2] - vxyz[3 * b + 2];
            f64 inv  = inv_sat_positive(rab);
            f64 rx = dx * inv, ry = dy * inv, rz = dz * inv;
            f64 v_ab_r_ab     = vx * rx + vy * ry + vz * rz;
            f64 abs_v_ab_r_ab = std::fabs(v_ab_r_ab);
            const f64 alpha_b = alpha ? alpha[b] : alpha_AV;
            f64 vsig_a = alpha_a * cs_a + beta_AV * abs_v_ab_r_ab;
            f64 vsig_b = alpha_b * cs_b + beta_AV * abs_v_ab_r_ab;
            // vsig_u (forces.hpp:35-41)
            f64 rho_avg = (rho_a + rho_b) * 0.5;
            f64 abs_dp  = std::fabs(P_a - P_b);
            f64 vsig_u  = std::sqrt(abs_dp / rho_avg);
            // q_av (q_ab.hpp:36-39)
            f64 qa_ab = std::fmax(-f64(0.5) * rho_a * vsig_a * v_ab_r_ab, f64(0));
            f64 qb_ab = std::fmax(-f64(0.5) * rho_b * vsig_b * v_ab_r_ab, f64(0));
            // add_to_derivs_sph_artif_visco_cond (forces.hpp:172-226)
            f64 AV_P_a = P_a + qa_ab;
            f64 AV_P_b = P_b + qb_ab;
            f64 sub_fact_a = rho_a_sq * omega_a;
            f64 sub_fact_b = (rho_b * rho_b) * omega_b;
            f64 ca = AV_P_a * inv_sat_zero(sub_fact_a);
            f64 cb = AV_P_b * inv_sat_zero(sub_fact_b);
            f64 nax = rx * Fab_a, nay = ry * Fab_a, naz = rz * Fab_a;
            f64 nbx = rx * Fab_b, nby = ry * Fab_b, nbz = rz * Fab_b;
            f64 mb = -pmass;
            fx += mb * (ca * nax + cb * nbx);
            fy += mb * (ca * nay + cb * nby);
            fz += mb * (ca * naz + cb * nbz);
            f64 dotvg = vx * nax + vy * nay + vz * naz;
            tdu += AV_P_a * (omega_a_rho_a_inv * rho_a_inv) * pmass * dotvg;
            f64 Fa = Fab_a * omega_a_rho_a_inv;
            f64 Fb = Fab_b / (rho_b * omega_b);
            tdu += pmass * alpha_u * vsig_u * (u_a - u_b) * f64(0.5) * (Fa + Fb);
        }
        axyz[3 * a]     = fx;
        axyz[3 * a + 1] = fy;
        axyz[3 * a + 2] = fz;
        du[a]           = tdu;
    }
}

// Velocity-gradient estimates of the varying (CD10) viscosity, per local particle a over
// its cache row, pairs inside max(h_a, h_b) R and grad W taken with h_a:
//  - div v, curl v: -1/(Omega_a rho_a) sum m (v_a - v_b) . / x grad W
//    (shammodels/sph/src/modules/DiffOperator.cpp:95-140, 200-245);
//  - d(div v)/dt = tr(G(a)) - tr(G(v) G(v)) with the linearly corrected gradients
//    G(f) = R^-1 D(f), R_ij = -sum m r_ab,i gradW_j, D(f)_jk = -sum m f_ab,k gradW_j
//    (DiffOperatorDtDivv.cpp:116-210, 3x3 inverse by cofactors, matrix_legacy.hpp:25-95).
// The three share one pass over the row; each sum keeps the reference's order.
inline void inv33(const f64 m[3][3], f64 r[3][3]) {
    const f64 a00 = m[0][0], a01 = m[0][1], a02 = m[0][2];
    const f64 a10 = m[1][0], a11 = m[1][1], a12 = m[1][2];
    const f64 a20 = m[2][0], a21 = m[2][1], a22 = m[2][2];
    const f64 det = (((((-a02 * a11) * a20 + (a01 * a12) * a20) + (a02 * a10) * a21)
                      - (a00 * a12) * a21) - (a01 * a10) * a22) + (a00 * a11) * a22;
    r[0][0] = (-a12 * a21 + a11 * a22) / det;
    r[0][1] = (a02 * a21 - a01 * a22) / det;
    r[0][2] = (-a02 * a11 + a01 * a12) / det;
    r[1][0] = (a12 * a20 - a10 * a22) / det;
    r[1][1] = (-a02 * a20 + a00 * a22) / det;
    r[1][2] = (a02 * a10 - a00 * a12) / det;
    r[2][0] = (-a11 * a20 + a10 * a21) / det;
    r[2][1] = (a01 * a20 - a00 * a21) / det;
    r[2][2] = (-a01 * a10 + a00 * a11) / det;
}
inline void mul33(const f64 a[3][3], const f64 b[3][3], f64 c[3][3]) {
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) c[i][j] = (a[i][0] * b[0][j] + a[i][1] * b[1][j]) + a[i][2] * b[2][j];
}

void velocity_gradients(
    u32 n_local, const u32 *cnt, const u32 *scanned, const u32 *entries, const f64 *xyz,
    const f64 *vxyz, const f64 *axyz, const f64 *hpart, const f64 *omega, f64 pmass, f64 *divv,
    f64 *curlv, f64 *dtdivv) {
    const f64 Rker2 = Rkern * Rkern;
#pragma omp parallel for schedule(dynamic, 1024)
    for (i64 ii = 0; ii < (i64) n_local; ii++) {
        u32 a = (u32) ii;
        const f64 h_a = hpart[a];
        const f64 *xa = &xyz[3 * a], *va = &vxyz[3 * a], *aa = &axyz[3 * a];
        const f64 rho_a = rho_h(pmass, h_a, hfactd);
        const f64 inv_rho_omega_a = 1. / (omega[a] * rho_a);
        f64 sdiv = 0, sc[3] = {0, 0, 0};
        f64 R[3][3] = {}, Dv[3][3] = {}, Da[3][3] = {};
        for (u32 k = scanned[a]; k < scanned[a] + cnt[a]; k++) {
            u32 b = entries[k];
            const f64 r[3] = {xa[0] - xyz[3 * b], xa[1] - xyz[3 * b + 1], xa[2] - xyz[3 * b + 2]};
            const f64 rab2 = (r[0] * r[0] + r[1] * r[1]) + r[2] * r[2];
            const f64 h_b  = hpart[b];
            if (rab2 > h_a * h_a * Rker2 && rab2 > h_b * h_b * Rker2) continue;
            const f64 rab = std::sqrt(rab2);
            const f64 v[3] = {va[0] - vxyz[3 * b], va[1] - vxyz[3 * b + 1], va[2] - vxyz[3 * b + 2]};
            const f64 w[3] = {aa[0] - axyz[3 * b], aa[1] - axyz[3 * b + 1], aa[2] - axyz[3 * b + 2]};
            f64 e[3] = {r[0] / rab, r[1] / rab, r[2] / rab};
            if (rab < 1e-9) e[0] = e[1] = e[2] = 0;
            const f64 F = dW_3d(rab, h_a);
            const f64 g[3] = {F * e[0], F * e[1], F * e[2]};
            sdiv = sdiv + pmass * ((v[0] * g[0] + v[1] * g[1]) + v[2] * g[2]);
            sc[0] = sc[0] + pmass * (v[1] * g[2] - v[2] * g[1]);
            sc[1] = sc[1] + pmass * (v[2] * g[0] - v[0] * g[2]);
            sc[2] = sc[2] + pmass * (v[0] * g[1] - v[1] * g[0]);
            const f64 mg[3] = {g[0] * pmass, g[1] * pmass, g[2] * pmass};
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) {
                    R[i][j]  = R[i][j] - r[i] * mg[j];
                    Dv[j][i] = Dv[j][i] - v[i] * mg[j];
                    Da[j][i] = Da[j][i] - w[i] * mg[j];
                }
        }
        divv[a] = -inv_rho_omega_a * sdiv;
        for (int c = 0; c < 3; c++) curlv[3 * a + c] = -inv_rho_omega_a * sc[c];
        f64 Ri[3][3], Gv[3][3], Ga[3][3];
        inv33(R, Ri);
        mul33(Ri, Dv, Gv);
        mul33(Ri, Da, Ga);
        const f64 div_a = (Ga[0][0] + Ga[1][1]) + Ga[2][2];
        const f64 tens  = ((((((((Gv[0][0] * Gv[0][0] + Gv[1][0] * Gv[0][1]) + Gv[2][0] * Gv[0][2])
                                + Gv[0][1] * Gv[1][0]) + Gv[1][1] * Gv[1][1]) + Gv[2][1] * Gv[1][2])
                             + Gv[0][2] * Gv[2][0]) + Gv[1][2] * Gv[2][1]) + Gv[2][2] * Gv[2][2]);
        dtdivv[a] = div_a - tens;
    }
}

// Cullen & Dehnen (2010) viscosity switch, one implicit-Euler relaxation step
// (shammodels/sph/src/modules/UpdateViscosity.cpp:170-215); cs is the sound speed kept
// from the previous step's last EOS evaluation.
void cd10_update(u32 n, const f64 *divv, const f64 *curlv, const f64 *dtdivv, const f64 *cs,
                 const f64 *h, const f64 *alpha, f64 dt, f64 sigma_decay, f64 alpha_min,
                 f64 alpha_max, f64 *alpha_new) {
    const f64 eps = std::numeric_limits<f64>::epsilon();
#pragma omp parallel for schedule(static)
    for (i64 ii = 0; ii < (i64) n; ii++) {
        const u32 i = (u32) ii;
        const f64 cs_a = cs[i], h_a = h[i], alpha_a = alpha[i];
        const f64 inv_tau = cs_a * sigma_decay / h_a;
        const f64 fact_t  = dt * inv_tau;
        const f64 euler   = 1 / (1 + fact_t);
        // max / min written as comparisons (NaN and signed-zero cases fixed, as on the GPU)
        const f64 md = -divv[i];
        f64 fac      = (md > 0) ? md : f64(0);
        fac          = fac * fac;
        const f64 traceS = (curlv[3 * i] * curlv[3 * i] + curlv[3 * i + 1] * curlv[3 * i + 1])
                           + curlv[3 * i + 2] * curlv[3 * i + 2];
        const f64 balsara = (fac + traceS > eps) ? fac / (fac + traceS) : f64(1);
        const f64 mdt     = -dtdivv[i];
        const f64 A       = balsara * ((mdt > 0) ? mdt : f64(0));
        const f64 temp    = cs_a * cs_a;
        f64 alpha_loc     = (cs_a > 0) ? 10 * h_a * h_a * A / temp : alpha_min;
        alpha_loc         = (alpha_loc < alpha_max) ? alpha_loc : alpha_max;
        alpha_loc     = (temp > eps) ? alpha_loc : alpha_min;
        f64 na = (alpha_a + alpha_loc * fact_t) * euler;
        if (alpha_loc > alpha_a) na = alpha_loc;
        alpha_new[i] = na;
    }
}

// Morris & Monaghan (1997) switch, one implicit-Euler step towards alpha_min with the
// source max(-div v, 0) (UpdateViscosity.cpp:53-118)
void mm97_update(u32 n, const f64 *divv, const f64 *cs, const f64 *h, const f64 *alpha, f64 dt,
                 f64 sigma_decay, f64 alpha_min, f64 alpha_max, f64 *alpha_new) {
#pragma omp parallel for schedule(static)
    for (i64 ii = 0; ii < (i64) n; ii++) {
        const u32 i      = (u32) ii;
        const f64 inv_tau = cs[i] * sigma_decay / h[i];
        const f64 fact_t  = dt * inv_tau;
        const f64 euler   = 1 / (1 + fact_t);
        const f64 md      = -divv[i];
        const f64 source  = (md > 0) ? md : f64(0);
        const f64 na      = (alpha[i] + source * dt + fact_t * alpha_min) * euler;
        alpha_new[i]      = (na < alpha_max) ? na : alpha_max;
    }
}

// v_sig — shammodels/sph/src/Solver.cpp:2716-2788 (alpha_AV = 1, beta_AV = 2 fixed)
void vsig_max(
    u32 n_local, const u32 *cnt, const u32 *scanned, const u32 *entries, const f64 *xyz,
    const f64 *vxyz, const f64 *hpart, const f64 *cs, f64 *vsig) {
    const f64 Rker2 = Rkern * Rkern, alpha_AV = 1.0, beta_AV = 2.0;
#pragma omp parallel for schedule(dynamic, 1024)
    for (i64 ii = 0; ii < (i64) n_local; ii++) {
        u32 a = (u32) ii;
        f64 h_a = hpart[a];
        const f64 *xa = &xyz[3 * a], *va = &vxyz[3 * a];
        f64 cs_a = cs[a], vmax = 0;
        for (u32 k = scanned[a]; k < scanned[a] + cnt[a]; k++) {
            u32 b    = entries[k];
            f64 dx   = xa[0] - xyz[3 * b], dy = xa[1] - xyz[3 * b + 1],
                dz   = xa[2] - xyz[3 * b + 2];
            f64 rab2 = dx * dx + dy * dy + dz * dz;
            f64 h_b  = hpart[b];
            if (rab2 > h_a * h_a * Rker2 && rab2 > h_b * h_b * Rker2) continue;
            f64 rab = std::sqrt(rab2);
            f64 vx = va[0] - vxyz[3 * b], vy = va[1] - vxyz[3 * b + 1], vz = va[2] - vxyz[3 * b + 2];
            f64 rx = dx / rab, ry = dy / rab, rz = dz / rab;
            if (rab < 1e-9) rx = ry = rz = 0;
            f64 v_ab_r_ab = vx * rx + vy * ry + vz * rz;
            f64 vsig_a    = alpha_AV * cs_a + beta_AV * std::fabs(v_ab_r_ab);
            vmax          = std::fmax(vmax, vsig_a);
        }
        vsig[a] = vmax;
    }
}

// CFL — shammodels/sph/include/shammodels/sph/modules/ComputeCFLCourant.hpp:45-60,
//       ComputeCFLForce.hpp:50-62; global min (Solver.cpp:3046-3119)
f64 cfl_min(u32 n, const f64 *h, const f64 *vsig, const f64 *axyz, f64 C_cour, f64 C_force,
            f64 *dt_part) {
    f64 m = std::numeric_limits<f64>::infinity();
    for (u32 a = 0; a < n; a++) {
        f64 dt   = std::numeric_limits<f64>::infinity();
        f64 dt_c = C_cour * h[a] / vsig[a];
        dt       = std::fmin(dt, dt_c);
        f64 ax = axyz[3 * a], ay = axyz[3 * a + 1], az = axyz[3 * a + 2];
        f64 abs_a = std::sqrt(ax * ax + ay * ay + az * az);
        f64 dt_f  = C_force * std::sqrt(h[a] / abs_a);
        dt        = std::fmin(dt, dt_f);
        if (dt_part) dt_part[a] = dt;
        m = std::fmin(m, dt);
    }
    return m;
}

// Leapfrog predictor — shamrock/src/math/integrators.cpp:27-86 via Solver.cpp:390-524:
// v += dt/2 a, u += dt/2 du (half step 1), x += dt v, then the second half step, and the
// periodic wrap of the positions (integrators.cpp:207-237).
void leapfrog_predict(u32 n, f64 *xyz, f64 *vxyz, f64 *u, const f64 *axyz, const f64 *du, f64 dt,
                      u32 periodic, const f64 *bmin, const f64 *bmax, f64 *aext_out = nullptr,
                      f64 central_mass = 0, f64 G = 0) {
    const f64 dt_half = dt / 2;
    for (u32 i = 0; i < n; i++) {
        for (int c = 0; c < 3; c++) vxyz[3 * i + c] = vxyz[3 * i + c] + dt_half * axyz[3 * i + c];
        u[i] = u[i] + dt_half * du[i];
    }
    for (u32 i = 0; i < 3 * n; i++) xyz[i] = xyz[i] + dt * vxyz[i];
    for (u32 i = 0; i < n; i++) {
        for (int c = 0; c < 3; c++) vxyz[3 * i + c] = vxyz[3 * i + c] + dt_half * axyz[3 * i + c];
        u[i] = u[i] + dt_half * du[i];
    }
    // velocity-independent external forces at the drifted positions, before the wrap
    if (aext_out) point_mass_accel(n, xyz, central_mass, G, aext_out);
    if (periodic) {
        for (u32 i = 0; i < n; i++)
            for (int c = 0; c < 3; c++) {
                f64 delt = bmax[c] - bmin[c];
                f64 r    = xyz[3 * i + c] - bmin[c];
                r        = std::fmod(r, delt);
                r += delt;
                r = std::fmod(r, delt);
                r += bmin[c];
                xyz[3 * i + c] = r;
            }
    }
}

// Leapfrog corrector — integrators.cpp:88-120, Solver.cpp:2506-2616: v += dt/2 (a_new -
// a_old), u += dt/2 (du_new - du_old); returns eps_v = max|dv| / sqrt(sum v^2 / n) (0
// when the mean vanishes), the rerun test of the corrector loop.
f64 leapfrog_correct(u32 n, f64 *vxyz, f64 *u, const f64 *a_new, const f64 *a_old,
                     const f64 *du_new, const f64 *du_old, f64 dt) {
    f64 hdt     = dt / 2;
    f64 max_ev2 = 0;
    for (u32 i = 0; i < n; i++) {
        f64 ix = hdt * (a_new[3 * i] - a_old[3 * i]);
        f64 iy = hdt * (a_new[3 * i + 1] - a_old[3 * i + 1]);
        f64 iz = hdt * (a_new[3 * i + 2] - a_old[3 * i + 2]);
        vxyz[3 * i]     = vxyz[3 * i] + ix;
        vxyz[3 * i + 1] = vxyz[3 * i + 1] + iy;
        vxyz[3 * i + 2] = vxyz[3 * i + 2] + iz;
        max_ev2         = std::fmax(max_ev2, ix * ix + iy * iy + iz * iz);
        f64 iu          = hdt * (du_new[i] - du_old[i]);
        u[i]            = u[i] + iu;
    }
    f64 sum_vsq = 0;
    for (u32 i = 0; i < n; i++)
        sum_vsq += vxyz[3 * i] * vxyz[3 * i] + vxyz[3 * i + 1] * vxyz[3 * i + 1]
                   + vxyz[3 * i + 2] * vxyz[3 * i + 2];
    f64 rank_veps_v = std::sqrt(max_ev2);
    f64 vmean       = std::sqrt(sum_vsq / f64(n));
    f64 eps_v       = rank_veps_v / vmean;
    if (vmean <= 0) eps_v = 0;
    return eps_v;
}

// =================================================================================
// Periodic ghosts, one patch covering the box —
//   find_interfaces shammodels/sph/src/BasicSPHGhosts.cpp:260-360 (27 offsets, x
//   outer .. z inner, self offset skipped), interaction range
//   SPHUtilities.hpp:79-95 (max h * htol * Rkern), interface volume
//   sender ∩ (receiver expanded - offset), selection by half-open box
//   (shamrock/patch/Patch.hpp:210-215, BasicSPHGhosts.cpp:512-530), ghosts appended
//   in interface order after the locals (BasicSPHGhosts.hpp:452-517).
// =================================================================================
void periodic_ghosts(
    u32 n_local, const f64 *xyz, const f64 *h, const f64 *bmin, const f64 *bmax, f64 htol,
    std::vector<u32> &src, std::vector<f64> &offs) {
    src.clear();
    offs.clear();
    f64 hmax = std::numeric_limits<f64>::lowest();
    for (u32 i = 0; i < n_local; i++) hmax = std::fmax(hmax, h[i]);
    f64 R = hmax * htol * Rkern;
    f64 bsize[3] = {bmax[0] - bmin[0], bmax[1] - bmin[1], bmax[2] - bmin[2]};
    for (i32 xo = -1; xo <= 1; xo++)
        for (i32 yo = -1; yo <= 1; yo++)
            for (i32 zo = -1; zo <= 1; zo++) {
                if (xo == 0 && yo == 0 && zo == 0) continue;
                f64 off[3] = {xo * bsize[0], yo * bsize[1], zo * bsize[2]};
                f64 vlo[3], vhi[3];
                for (int c = 0; c < 3; c++) {
                    f64 rlo = (bmin[c] - R) + (-off[c]);
                    f64 rhi = (bmax[c] + R) + (-off[c]);
                    vlo[c]  = std::fmax(bmin[c], rlo);
                    vhi[c]  = std::fmin(bmax[c], rhi);
                }
                for (u32 i = 0; i < n_local; i++) {
                    const f64 *p = &xyz[3 * i];
                    if ((vlo[0] <= p[0]) && (p[0] < vhi[0]) && (vlo[1] <= p[1]) && (p[1] < vhi[1])
                        && (vlo[2] <= p[2]) && (p[2] < vhi[2])) {
                        src.push_back(i);
                        offs.push_back(off[0]);
                        offs.push_back(off[1]);
                        offs.push_back(off[2]);
                    }
                }
            }
}

// =================================================================================
// Full step — shammodels/sph/src/Solver.cpp:1942-3272 (evolve_once),
//   predictor graph :390-524 + ForwardEuler (shammodels/common ForwardEuler.hpp:62-84),
//   periodic wrap (shamrock/src/math/integrators.cpp:207-237), sph_prestep :1060-1304,
//   corrector (integrators.cpp:88-120, Solver.cpp:2506-2616), CFL and multiplier
//   update :3253-3263.
// =================================================================================
struct Config {
    f64 gamma;
    f64 pmass;
    f64 alpha_u, alpha_AV, beta_AV;
    f64 cfl_cour, cfl_force, cfl_mult_stiffness;
    f64 htol_up_coarse, htol_up_fine;
    f64 epsilon_h;
    u32 h_iter_per_subcycles, h_max_subcycles;
    u32 tree_reduction_level;
    u32 periodic;
    f64 bmin[3], bmax[3];
    u32 eos_kind; // 0 adiabatic, 1 locally isothermal (LP07)
    u32 ext_kind; // 0 none, 1 central point mass
    f64 cs0, eos_r0, eos_q;        // LP07: c_s^2 = cs0^2 (R^2 / r0^2)^(-q)
    f64 central_mass, constant_G;  // point mass at the origin
    u32 av_kind;  // 0 constant, 1 varying CD10 (Cullen & Dehnen 2010), 2 varying MM97
    u32 pad;
    f64 alpha_min, alpha_max, sigma_decay;
};

struct StepLog {
    f64 t, dt, next_dt, cfl_mult;
    u32 n_local, n_ghost, leaf_count, h_subcycles, h_iterations, corrector_iters;
    u64 cache_size;
    f64 eps_v, max_eps_h;
};

struct Sim {
    Config cfg;
    u32 n;
    std::vector<f64> xyz, vxyz, axyz, h, u, du, omega;
    f64 t = 0, dt = 0, cfl_mult = 1e-2;
    // last-step artefacts (merged index space) kept for inspection
    std::vector<u32> ghost_src;
    std::vector<f64> ghost_off;
    Tree tree;
    NeighCache cache;
    std::vector<f64> P, cs, vsig;
    // varying AV state (alpha_AV, the sound speed of the last EOS) and its diagnostics
    std::vector<f64> alpha_AV, soundspeed, divv, curlv, dtdivv;
};

void merge_positions(Sim &s, std::vector<f64> &mxyz, std::vector<f64> &mh) {
    u32 n = s.n, g = (u32) s.ghost_src.size();
    mxyz.resize(3 * (size_t) (n + g));
    mh.resize(n + g);
    std::memcpy(mxyz.data(), s.xyz.data(), sizeof(f64) * 3 * n);
    std::memcpy(mh.data(), s.h.data(), sizeof(f64) * n);
    for (u32 k = 0; k < g; k++) {
        u32 i = s.ghost_src[k];
        for (int c = 0; c < 3; c++) mxyz[3 * (n + k) + c] = s.xyz[3 * i + c] + s.ghost_off[3 * k + c];
        mh[n + k] = s.h[i];
    }
}

template<class T>
void merge_field(const Sim &s, const std::vector<T> &f, int comps, std::vector<T> &out) {
    u32 n = s.n, g = (u32) s.ghost_src.size();
    out.resize((size_t) comps * (n + g));
    std::memcpy(out.data(), f.data(), sizeof(T) * comps * n);
    for (u32 k = 0; k < g; k++)
        for (int c = 0; c < comps; c++) out[comps * (n + k) + c] = f[comps * s.ghost_src[k] + c];
}

void evolve_once(Sim &s, StepLog &log) {
    const Config &cfg = s.cfg;
    u32 n             = s.n;
    f64 dt            = s.dt;
    log               = StepLog{};
    log.t             = s.t;
    log.dt            = dt;
    log.n_local       = n;

    std::vector<f64> aext;
    if (cfg.ext_kind == 1) aext.assign(3 * (size_t) n, 0);
    leapfrog_predict(n, s.xyz.data(), s.vxyz.data(), s.u.data(), s.axyz.data(), s.du.data(), dt,
                     cfg.periodic, cfg.bmin, cfg.bmax, cfg.ext_kind == 1 ? aext.data() : nullptr,
                     cfg.central_mass, cfg.constant_G);

    // sph_prestep
    std::vector<f64> mxyz, mh;
    u32 hstep = 0;
    for (; hstep < cfg.h_max_subcycles; hstep++) {
        if (cfg.periodic) {
            periodic_ghosts(n, s.xyz.data(), s.h.data(), cfg.bmin, cfg.bmax, cfg.htol_up_coarse,
                            s.ghost_src, s.ghost_off);
        } else {
            s.ghost_src.clear();
            s.ghost_off.clear();
        }
        merge_positions(s, mxyz, mh);
        u32 N = (u32) mh.size();
        // BuildTrees.cpp:26-59
        f64 bmn[3], bmx[3];
        for (int c = 0; c < 3; c++) {
            bmn[c] = std::numeric_limits<f64>::max();
            bmx[c] = std::numeric_limits<f64>::lowest();
        }
        for (u32 i = 0; i < N; i++)
            for (int c = 0; c < 3; c++) {
                bmn[c] = std::fmin(bmn[c], mxyz[3 * i + c]);
                bmx[c] = std::fmax(bmx[c], mxyz[3 * i + c]);
            }
        const f64 inf = std::numeric_limits<f64>::infinity();
        for (int c = 0; c < 3; c++) {
            bmn[c] = std::nextafter(bmn[c], -inf);
            bmx[c] = std::nextafter(bmx[c], inf);
        }
        s.tree = Tree{};
        build_tree_impl<u32>(s.tree, mxyz.data(), mh.data(), N, bmn, bmx, cfg.tree_reduction_level,
                             cfg.htol_up_coarse);
        neigh_cache(s.tree, mxyz.data(), mh.data(), n, cfg.htol_up_coarse, s.cache);
        std::vector<f64> eps(n, 100.), h_old(s.h);
        f64 max_eps = std::numeric_limits<f64>::max();
        u32 it      = 0;
        for (; it < cfg.h_iter_per_subcycles; it++) {
            h_iterate_once(n, s.cache.part.cnt.data(), s.cache.part.scanned.data(),
                           s.cache.part.entries.data(), mxyz.data(), h_old.data(), s.h.data(),
                           eps.data(), cfg.pmass, cfg.htol_up_coarse, cfg.htol_up_fine);
            max_eps = *std::max_element(eps.begin(), eps.end());
            log.h_iterations++;
            if (max_eps < cfg.epsilon_h) break;
        }
        f64 min_eps = *std::min_element(eps.begin(), eps.end());
        log.max_eps_h = max_eps;
        bool converged = (max_eps < cfg.epsilon_h) && !(min_eps < 0);
        if (!converged) continue;
        break;
    }
    log.h_subcycles = hstep + 1;
    log.n_ghost     = (u32) s.ghost_src.size();
    log.leaf_count  = s.tree.leaf_count;
    log.cache_size  = s.cache.part.total;
    s.omega.assign(n, 0);
    compute_omega(n, s.cache.part.cnt.data(), s.cache.part.scanned.data(),
                  s.cache.part.entries.data(), mxyz.data(), s.h.data(), cfg.pmass, s.omega.data());

    // corrector loop
    f64 next_cfl   = 0;
    bool rerun     = false;
    u32 corr_iters = 0;
    do {
        std::vector<f64> m_h, m_u, m_v, m_om;
        merge_field(s, s.h, 1, m_h);
        merge_field(s, s.u, 1, m_u);
        merge_field(s, s.vxyz, 3, m_v);
        merge_field(s, s.omega, 1, m_om);
        u32 N = (u32) m_h.size();
        // varying AV (Solver.cpp:2261-2370): div v, curl v, d(div v)/dt with the current
        // velocities and the accelerations of the last evaluation, the switch update from
        // alpha_AV, then alpha on the ghosts
        std::vector<f64> alpha_upd, m_alpha;
        if (cfg.av_kind == 1 || cfg.av_kind == 2) {
            std::vector<f64> m_a;
            merge_field(s, s.axyz, 3, m_a);
            s.divv.assign(n, 0);
            s.curlv.assign(3 * (size_t) n, 0);
            s.dtdivv.assign(n, 0);
            velocity_gradients(n, s.cache.part.cnt.data(), s.cache.part.scanned.data(),
                               s.cache.part.entries.data(), mxyz.data(), m_v.data(), m_a.data(),
                               m_h.data(), m_om.data(), cfg.pmass, s.divv.data(), s.curlv.data(),
                               s.dtdivv.data());
            alpha_upd.assign(n, 0);
            if (cfg.av_kind == 1)
                cd10_update(n, s.divv.data(), s.curlv.data(), s.dtdivv.data(), s.soundspeed.data(),
                            s.h.data(), s.alpha_AV.data(), dt, cfg.sigma_decay, cfg.alpha_min,
                            cfg.alpha_max, alpha_upd.data());
            else
                mm97_update(n, s.divv.data(), s.soundspeed.data(), s.h.data(), s.alpha_AV.data(), dt,
                            cfg.sigma_decay, cfg.alpha_min, cfg.alpha_max, alpha_upd.data());
            merge_field(s, alpha_upd, 1, m_alpha);
        }
        s.P.assign(N, 0);
        s.cs.assign(N, 0);
        if (cfg.eos_kind == 1)
            eos_locally_isothermal(N, mxyz.data(), m_h.data(), cfg.pmass, cfg.cs0, cfg.eos_r0,
                                   cfg.eos_q, s.P.data(), s.cs.data());
        else
            eos_adiabatic(N, m_h.data(), m_u.data(), cfg.pmass, cfg.gamma, s.P.data(), s.cs.data());
        std::vector<f64> old_a(s.axyz), old_du(s.du);
        derivs_constAV(n, s.cache.part.cnt.data(), s.cache.part.scanned.data(),
                       s.cache.part.entries.data(), mxyz.data(), m_v.data(), m_h.data(),
                       m_om.data(), m_u.data(), s.P.data(), s.cs.data(), cfg.pmass, cfg.alpha_u,
                       cfg.alpha_AV, cfg.beta_AV, s.axyz.data(), s.du.data(),
                       cfg.av_kind != 0 ? m_alpha.data() : nullptr);
        if (cfg.ext_kind == 1)
            for (size_t k = 0; k < 3 * (size_t) n; k++) s.axyz[k] = s.axyz[k] + aext[k];
        f64 eps_v = leapfrog_correct(n, s.vxyz.data(), s.u.data(), s.axyz.data(), old_a.data(),
                                     s.du.data(), old_du.data(), dt);
        log.eps_v = eps_v;
        if (eps_v > 1e-2) {
            rerun = true;
            s.cfl_mult = s.cfl_mult / 2;
        } else {
            rerun = false;
            if (cfg.av_kind != 0) {
                // write back (Solver.cpp:2620-2650, 3125-3160)
                s.alpha_AV = alpha_upd;
                s.soundspeed.assign(s.cs.begin(), s.cs.begin() + n);
            }
            s.vsig.assign(n, 0);
            vsig_max(n, s.cache.part.cnt.data(), s.cache.part.scanned.data(),
                     s.cache.part.entries.data(), mxyz.data(), m_v.data(), m_h.data(), s.cs.data(),
                     s.vsig.data());
            f64 C_cour  = cfg.cfl_cour * s.cfl_mult;
            f64 C_force = cfg.cfl_force * s.cfl_mult;
            next_cfl    = cfl_min(n, s.h.data(), s.vsig.data(), s.axyz.data(), C_cour, C_force, nullptr);
        }
        corr_iters++;
        if (corr_iters >= 50 && rerun) break;
    } while (rerun);
    log.corrector_iters = corr_iters;
    s.dt                = next_cfl;
    s.t                 = s.t + dt;
    f64 stiff           = cfg.cfl_mult_stiffness;
    s.cfl_mult          = (s.cfl_mult * stiff + 1.) / (stiff + 1.);
    log.next_dt         = s.dt;
    log.cfl_mult        = s.cfl_mult;
}

} // namespace orc

// =================================================================================
// C API (ctypes)
// =================================================================================
extern "C" {

void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#endif
}
int orc_get_threads() {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_morton32(const f64 *pos, u32 n, u32 mc, const f64 *bmin, const f64 *bmax, u32 *out) {
    orc::morton_codes<u32>(pos, n, mc, bmin, bmax, out);
}
void orc_morton64(const f64 *pos, u32 n, u32 mc, const f64 *bmin, const f64 *bmax, u64 *out) {
    orc::morton_codes<u64>(pos, n, mc, bmin, bmax, out);
}
void orc_bitonic32(u32 *k, u32 *v, u32 len) { orc::bitonic_sort<u32>(k, v, len); }
void orc_bitonic64(u64 *k, u32 *v, u32 len) { orc::bitonic_sort<u64>(k, v, len); }
void orc_bitonic32_stencil16(u32 *k, u32 *v, u32 len) { orc::bitonic_sort_stencil16<u32>(k, v, len); }
void orc_bitonic64_stencil16(u64 *k, u32 *v, u32 len) { orc::bitonic_sort_stencil16<u64>(k, v, len); }

u32 orc_reduce32(const u32 *m, u32 cnt, u32 level, u32 *out) {
    std::vector<u32> r;
    u32 L = orc::reduction_alg<u32>(m, cnt, level, r);
    std::memcpy(out, r.data(), sizeof(u32) * r.size());
    return L;
}
u32 orc_reduce64(const u64 *m, u32 cnt, u32 level, u32 *out) {
    std::vector<u32> r;
    u32 L = orc::reduction_alg<u64>(m, cnt, level, r);
    std::memcpy(out, r.data(), sizeof(u32) * r.size());
    return L;
}
void orc_karras32(const u32 *m, u32 L, u32 *lc, u32 *rc, u8 *lf, u8 *rf, u32 *er) {
    orc::karras_tree<u32>(m, L, lc, rc, lf, rf, er);
}
void orc_karras64(const u64 *m, u32 L, u32 *lc, u32 *rc, u8 *lf, u8 *rf, u32 *er) {
    orc::karras_tree<u64>(m, L, lc, rc, lf, rf, er);
}

void *orc_tree_build(const f64 *pos, const f64 *h, u32 n, const f64 *bmin, const f64 *bmax,
                     u32 level, int key_bits, f64 htol, u32 morton_count) {
    orc::Tree *t = new orc::Tree();
    if (key_bits == 64) orc::build_tree_impl<u64>(*t, pos, h, n, bmin, bmax, level, htol, morton_count);
    else orc::build_tree_impl<u32>(*t, pos, h, n, bmin, bmax, level, htol, morton_count);
    return t;
}
void orc_tree_free(void *t) { delete (orc::Tree *) t; }
u32 orc_tree_leaf_count(void *t) { return ((orc::Tree *) t)->leaf_count; }
u32 orc_tree_morton_count(void *t) { return ((orc::Tree *) t)->morton_count; }
void orc_tree_export(void *tp, u64 *sorted_keys, u32 *sort_index, u32 *reduc, u64 *reduced, u32 *lc,
                     u32 *rc, u8 *lf, u8 *rf, u32 *er, f64 *aabb_min, f64 *aabb_max, f64 *rint) {
    orc::Tree &t = *(orc::Tree *) tp;
    u32 P = t.morton_count, L = t.leaf_count, I = L - 1, T = 2 * L - 1;
    if (sorted_keys) std::memcpy(sorted_keys, t.sorted_keys.data(), 8 * (size_t) P);
    if (sort_index) std::memcpy(sort_index, t.sort_index.data(), 4 * (size_t) P);
    if (reduc) std::memcpy(reduc, t.reduc.data(), 4 * (size_t) (L + 2));
    if (reduced) std::memcpy(reduced, t.reduced.data(), 8 * (size_t) L);
    if (lc && I) std::memcpy(lc, t.lchild.data(), 4 * (size_t) I);
    if (rc && I) std::memcpy(rc, t.rchild.data(), 4 * (size_t) I);
    if (lf && I) std::memcpy(lf, t.lflag.data(), (size_t) I);
    if (rf && I) std::memcpy(rf, t.rflag.data(), (size_t) I);
    if (er && I) std::memcpy(er, t.endrange.data(), 4 * (size_t) I);
    if (aabb_min) std::memcpy(aabb_min, t.bmin.data(), 8 * 3 * (size_t) T);
    if (aabb_max) std::memcpy(aabb_max, t.bmax.data(), 8 * 3 * (size_t) T);
    if (rint) std::memcpy(rint, t.rint.data(), 8 * (size_t) T);
}

// CLBVHObjectIterator::rtree_for queries (shamtree/include/shamtree/CLBVHObjectIterator.hpp
// :127-169, exercised by src/tests/shamtree/CLBVHObjectIteratorTests.cpp):
// mode 0 = every node accepted; mode 1 = node AABB ∩ [p-s, p+s] non-empty and
// object position inside [p-s, p+s].  Returns entries written (two-pass when out==0).
u64 orc_tree_query(void *tp, const f64 *pos, u32 nq, int mode, f64 s, u32 *counts, u32 *out) {
    orc::Tree &t = *(orc::Tree *) tp;
    u64 w = 0;
    for (u32 q = 0; q < nq; q++) {
        const f64 *p = &pos[3 * q];
        f64 lo[3] = {p[0] + (-s), p[1] + (-s), p[2] + (-s)};
        f64 hi[3] = {p[0] + s, p[1] + s, p[2] + s};
        u32 c = 0;
        t.traverse(
            [&](u32 node) {
                if (mode == 0) return true;
                const f64 *nl = &t.bmin[3 * node], *nh = &t.bmax[3 * node];
                for (int k = 0; k < 3; k++)
                    if (!(std::fmin(nh[k], hi[k]) >= std::fmax(nl[k], lo[k]))) return false;
                return true;
            },
            [&](u32 node) {
                u32 l = node - t.offset_leaf();
                for (u32 sl = t.reduc[l]; sl < t.reduc[l + 1]; sl++) {
                    u32 id = t.sort_index[sl];
                    bool ok = true;
                    if (mode == 1) {
                        const f64 *r2 = &pos[3 * id];
                        for (int k = 0; k < 3; k++)
                            if (!(std::fmin(r2[k], hi[k]) >= std::fmax(r2[k], lo[k]))) ok = false;
                    }
                    if (ok) {
                        if (out) out[w] = id;
                        w++;
                        c++;
                    }
                }
            });
        if (counts) counts[q] = c;
    }
    return w;
}

void *orc_cache_build(void *tp, const f64 *xyz, const f64 *h, u32 n_local, f64 htol) {
    orc::NeighCache *nc = new orc::NeighCache();
    orc::neigh_cache(*(orc::Tree *) tp, xyz, h, n_local, htol, *nc);
    return nc;
}
void orc_cache_free(void *c) { delete (orc::NeighCache *) c; }
u64 orc_cache_total(void *c) { return ((orc::NeighCache *) c)->part.total; }
u64 orc_cache_leaf_total(void *c) { return ((orc::NeighCache *) c)->leaf.total; }
void orc_cache_export(void *cp, u32 *cnt, u32 *scanned, u32 *entries, u32 *owner, u32 *lcnt,
                      u32 *lscanned, u32 *lentries) {
    orc::NeighCache &c = *(orc::NeighCache *) cp;
    if (cnt) std::memcpy(cnt, c.part.cnt.data(), 4 * c.part.cnt.size());
    if (scanned) std::memcpy(scanned, c.part.scanned.data(), 4 * c.part.scanned.size());
    if (entries) std::memcpy(entries, c.part.entries.data(), 4 * c.part.entries.size());
    if (owner) std::memcpy(owner, c.owner.data(), 4 * c.owner.size());
    if (lcnt) std::memcpy(lcnt, c.leaf.cnt.data(), 4 * c.leaf.cnt.size());
    if (lscanned) std::memcpy(lscanned, c.leaf.scanned.data(), 4 * c.leaf.scanned.size());
    if (lentries) std::memcpy(lentries, c.leaf.entries.data(), 4 * c.leaf.entries.size());
}

void orc_h_iterate_once(u32 n, const u32 *cnt, const u32 *sc, const u32 *ent, const f64 *r,
                        const f64 *h_old, f64 *h_new, f64 *eps, f64 pmass, f64 hev, f64 hevi) {
    orc::h_iterate_once(n, cnt, sc, ent, r, h_old, h_new, eps, pmass, hev, hevi);
}
void orc_omega(u32 n, const u32 *cnt, const u32 *sc, const u32 *ent, const f64 *r, const f64 *h,
               f64 pmass, f64 *omega) {
    orc::compute_omega(n, cnt, sc, ent, r, h, pmass, omega);
}
void orc_eos_locally_isothermal(u32 n, const f64 *xyz, const f64 *h, f64 pmass, f64 cs0, f64 r0,
                                f64 q, f64 *P, f64 *cs) {
    orc::eos_locally_isothermal(n, xyz, h, pmass, cs0, r0, q, P, cs);
}
void orc_eos_adiabatic(u32 n, const f64 *h, const f64 *u, f64 pmass, f64 gamma, f64 *P, f64 *cs) {
    orc::eos_adiabatic(n, h, u, pmass, gamma, P, cs);
}
void orc_derivs_constAV(u32 n, const u32 *cnt, const u32 *sc, const u32 *ent, const f64 *xyz,
                        const f64 *v, const f64 *h, const f64 *om, const f64 *u, const f64 *P,
                        const f64 *cs, f64 pmass, f64 alpha_u, f64 alpha_AV, f64 beta_AV,
                        f64 *axyz, f64 *du) {
    orc::derivs_constAV(n, cnt, sc, ent, xyz, v, h, om, u, P, cs, pmass, alpha_u, alpha_AV,
                        beta_AV, axyz, du);
}
void orc_vsig(u32 n, const u32 *cnt, const u32 *sc, const u32 *ent, const f64 *xyz, const f64 *v,
              const f64 *h, const f64 *cs, f64 *vsig) {
    orc::vsig_max(n, cnt, sc, ent, xyz, v, h, cs, vsig);
}
f64 orc_cfl(u32 n, const f64 *h, const f64 *vsig, const f64 *a, f64 cc, f64 cf, f64 *dt_part) {
    return orc::cfl_min(n, h, vsig, a, cc, cf, dt_part);
}
void orc_predict(u32 n, f64 *xyz, f64 *vxyz, f64 *u, const f64 *axyz, const f64 *du, f64 dt,
                 u32 periodic, const f64 *bmin, const f64 *bmax) {
    orc::leapfrog_predict(n, xyz, vxyz, u, axyz, du, dt, periodic, bmin, bmax);
}
f64 orc_correct(u32 n, f64 *vxyz, f64 *u, const f64 *a_new, const f64 *a_old, const f64 *du_new,
                const f64 *du_old, f64 dt) {
    return orc::leapfrog_correct(n, vxyz, u, a_new, a_old, du_new, du_old, dt);
}
u32 orc_periodic_ghosts(u32 n, const f64 *xyz, const f64 *h, const f64 *bmin, const f64 *bmax,
                        f64 htol, u32 *src_out, f64 *off_out, u32 cap) {
    std::vector<u32> src;
    std::vector<f64> off;
    orc::periodic_ghosts(n, xyz, h, bmin, bmax, htol, src, off);
    u32 g = (u32) src.size();
    if (src_out && g <= cap) {
        std::memcpy(src_out, src.data(), 4 * (size_t) g);
        if (off_out) std::memcpy(off_out, off.data(), 8 * 3 * (size_t) g);
    }
    return g;
}

// --- simulation handle ---
void *orc_sim_create(const orc::Config *cfg, u32 n, const f64 *xyz, const f64 *vxyz, const f64 *h,
                     const f64 *u) {
    orc::Sim *s = new orc::Sim();
    s->cfg      = *cfg;
    s->n        = n;
    s->xyz.assign(xyz, xyz + 3 * (size_t) n);
    s->vxyz.assign(vxyz, vxyz + 3 * (size_t) n);
    s->h.assign(h, h + n);
    s->u.assign(u, u + n);
    s->axyz.assign(3 * (size_t) n, 0);
    s->du.assign(n, 0);
    s->omega.assign(n, 1);
    s->alpha_AV.assign(n, cfg->alpha_AV);
    s->soundspeed.assign(n, 0);
    return s;
}
// varying-AV state: alpha_AV and the stored sound speed (in and out), the last step's
// div v, curl v (3 per particle), d(div v)/dt (out)
void orc_sim_set_av(void *sp, const f64 *alpha, const f64 *cs) {
    orc::Sim *s = (orc::Sim *) sp;
    if (alpha) std::memcpy(s->alpha_AV.data(), alpha, 8 * (size_t) s->n);
    if (cs) std::memcpy(s->soundspeed.data(), cs, 8 * (size_t) s->n);
}
void orc_sim_get_av(void *sp, f64 *alpha, f64 *cs, f64 *divv, f64 *curlv, f64 *dtdivv) {
    orc::Sim *s = (orc::Sim *) sp;
    u32 n       = s->n;
    if (alpha) std::memcpy(alpha, s->alpha_AV.data(), 8 * (size_t) n);
    if (cs) std::memcpy(cs, s->soundspeed.data(), 8 * (size_t) n);
    if (divv && s->divv.size() == n) std::memcpy(divv, s->divv.data(), 8 * (size_t) n);
    if (curlv && s->curlv.size() == 3 * (size_t) n) std::memcpy(curlv, s->curlv.data(), 24 * (size_t) n);
    if (dtdivv && s->dtdivv.size() == n) std::memcpy(dtdivv, s->dtdivv.data(), 8 * (size_t) n);
}
void orc_sim_free(void *s) { delete (orc::Sim *) s; }
void orc_sim_set_time(void *sp, f64 t, f64 dt, f64 cfl_mult) {
    orc::Sim *s = (orc::Sim *) sp;
    s->t        = t;
    s->dt       = dt;
    s->cfl_mult = cfl_mult;
}
void orc_sim_get_time(void *sp, f64 *t, f64 *dt, f64 *cfl_mult) {
    orc::Sim *s = (orc::Sim *) sp;
    *t          = s->t;
    *dt         = s->dt;
    *cfl_mult   = s->cfl_mult;
}
void orc_sim_set_derivs(void *sp, const f64 *axyz, const f64 *du) {
    orc::Sim *s = (orc::Sim *) sp;
    std::memcpy(s->axyz.data(), axyz, 8 * 3 * (size_t) s->n);
    std::memcpy(s->du.data(), du, 8 * (size_t) s->n);
}
void orc_sim_evolve_once(void *sp, orc::StepLog *log) { orc::evolve_once(*(orc::Sim *) sp, *log); }
void orc_sim_get(void *sp, f64 *xyz, f64 *vxyz, f64 *h, f64 *u, f64 *axyz, f64 *du, f64 *omega) {
    orc::Sim *s = (orc::Sim *) sp;
    u32 n       = s->n;
    if (xyz) std::memcpy(xyz, s->xyz.data(), 8 * 3 * (size_t) n);
    if (vxyz) std::memcpy(vxyz, s->vxyz.data(), 8 * 3 * (size_t) n);
    if (h) std::memcpy(h, s->h.data(), 8 * (size_t) n);
    if (u) std::memcpy(u, s->u.data(), 8 * (size_t) n);
    if (axyz) std::memcpy(axyz, s->axyz.data(), 8 * 3 * (size_t) n);
    if (du) std::memcpy(du, s->du.data(), 8 * (size_t) n);
    if (omega) std::memcpy(omega, s->omega.data(), 8 * (size_t) n);
}
// last step's merged-space artefacts: ghost list and neighbour cache
u32 orc_sim_ghost_count(void *sp) { return (u32) ((orc::Sim *) sp)->ghost_src.size(); }
void orc_sim_ghosts(void *sp, u32 *src, f64 *off) {
    orc::Sim *s = (orc::Sim *) sp;
    std::memcpy(src, s->ghost_src.data(), 4 * s->ghost_src.size());
    std::memcpy(off, s->ghost_off.data(), 8 * s->ghost_off.size());
}
void *orc_sim_cache(void *sp) { return &((orc::Sim *) sp)->cache; }

} // extern "C"
