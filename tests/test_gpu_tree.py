"""GPU parity of the tree path (Morton keys, bitonic sort, leaf reduction, Karras tree,
AABBs, interaction radii, object queries, periodic ghosts, neighbour cache) against the
reference golden vectors and the oracle.  Integer/index results must be bit-exact."""

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def M():
    from shamrock_gb300 import modules

    return modules


# ----------------------------------------------------------------------------- golden
def test_golden_morton_and_sort(gctx, M, golden):
    """MortonCodeSetTests.cpp:80-125 through the GPU (u64 keys)."""
    g = golden("morton_code_set.json")["file_level"]
    keys = M.morton_codes(gctx, g["partpos"], [0, 0, 0], [1, 1, 1], 16, key_bits=64)
    assert M.unsigned(keys, 64).tolist() == g["test_mortons"]
    sk, perm = M.sort_by_key(gctx, keys, key_bits=64)
    assert M.unsigned(sk, 64).tolist() == g["test_mortons_sorted"]
    assert perm.cpu().numpy().tolist() == g["index_map_obj_idx"]


@pytest.mark.parametrize("test", ["shamtree/MortonReducedSet", "shamtree/MortonReducedSet(single cell)"])
def test_golden_reduced_set(gctx, M, golden, test):
    g = golden("morton_reduced_set.json")["tests"][test]
    v = g["vectors"]
    t = M.Tree(gctx, v["partpos"], [0, 0, 0], [1, 1, 1], g["reduce_morton_set_level"][0],
               key_bits=64, morton_count=16)
    e = t.export()
    assert e["sorted_keys"].tolist() == v["test_mortons_sorted"]
    assert e["sort_index"].tolist() == v["index_map_obj_idx"]
    assert e["reduc"].tolist() == v["buf_reduc_index_map"]
    assert e["reduced"].tolist() == v["reduced_morton_codes"]


@pytest.mark.parametrize("test", ["shamtree/KarrasRadixTreeAABB", "shamtree/KarrasRadixTreeAABB(one-cell)"])
def test_golden_karras_aabb(gctx, M, golden, test):
    g = golden("karras_radix_tree_aabb.json")["tests"][test]
    v = g["vectors"]
    t = M.Tree(gctx, v["partpos"], [0, 0, 0], [1, 1, 1], g["reduce_morton_set_level"][0],
               key_bits=64, morton_count=16)
    e = t.export()
    assert e["sort_index"].tolist() == v["index_map_obj_idx"]
    assert e["reduc"].tolist() == v["buf_reduc_index_map"]
    for k in ("lchild_id", "rchild_id", "lchild_flag", "rchild_flag", "endrange"):
        assert e[k].tolist() == v["expected_" + k], k
    assert np.array_equal(e["aabb_min"], np.array(v["aabb_min"], float))
    assert np.array_equal(e["aabb_max"], np.array(v["aabb_max"], float))


def test_golden_karras_topology(gctx, M, golden):
    """KarrasRadixTreeTests.cpp:19-77: the 12 hand-built codes, through the GPU tree by
    building on positions whose u64 codes are exactly those codes (grid centres)."""
    v = golden("karras_radix_tree.json")["tests"]["shamtree/KarrasRadixTree"]["vectors"]
    codes = np.array(v["test_morton_codes"], dtype=np.uint64)
    # decode each code to its grid cell and place the particle at the cell centre
    def decode(c):
        xyz = [0, 0, 0]
        for b in range(21):
            for a in range(3):
                xyz[a] |= int((int(c) >> (3 * b + (2 - a))) & 1) << b
        return xyz
    cells = np.array([decode(c) for c in codes], float)
    pos = (cells + 0.5) / 2097152.0
    t = M.Tree(gctx, pos, [0, 0, 0], [1, 1, 1], 0, key_bits=64)
    e = t.export()
    assert e["reduced"].tolist() == [int(c) for c in codes]
    for k in ("lchild_id", "rchild_id", "lchild_flag", "rchild_flag", "endrange"):
        assert e[k].tolist() == v["expected_" + k], k


@pytest.mark.parametrize("test", ["shamtree/LCBVHObjectIterator", "shamtree/LCBVHObjectIterator(one-cell)"])
def test_golden_object_iterator(gctx, M, golden, test):
    g = golden("clbvh_object_iterator.json")["tests"][test]
    v = g["vectors"]
    t = M.Tree(gctx, v["partpos"], [0, 0, 0], [1, 1, 1], g["rebuild_from_positions_level"][0],
               key_bits=64)
    assert t.leaf_count - 1 == g["scalar_requires"]["bvh.structure.get_internal_cell_count()"]
    c0, n0 = t.query(0)
    n = len(v["partpos"])
    assert c0.tolist() == [n] * n
    c1, n1 = t.query(1, 0.15)
    assert c1.tolist() == v["expected_counts"]
    assert n1.tolist() == v["expected_neigh"]


# ----------------------------------------------------------------------------- random parity
def _clustered(n, seed):
    rng = np.random.default_rng(seed)
    a = rng.random((n // 2, 3))
    b = np.clip(rng.normal(0.5, 0.02, size=(n - n // 2, 3)), 0, 1)
    return np.concatenate([a, b])


@pytest.mark.parametrize("n,key_bits", [(1, 32), (7, 32), (1000, 32), (4096, 32), (70001, 32),
                                        (300000, 32), (5000, 64), (70001, 64)])
def test_morton_sort_vs_oracle(gctx, M, n, key_bits):
    pos = _clustered(n, n)
    bmin, bmax = pos.min(0) - 1e-9, pos.max(0) + 1e-9
    P = 1 << int(np.ceil(np.log2(max(n, 1))))
    k_gpu = M.morton_codes(gctx, pos, bmin, bmax, P, key_bits)
    k_orc = O.morton_codes(pos, bmin, bmax, P, key_bits)
    assert np.array_equal(M.unsigned(k_gpu, key_bits), k_orc)
    sk, perm = M.sort_by_key(gctx, k_gpu, key_bits=key_bits)
    ok, operm = O.bitonic_sort(k_orc)
    assert np.array_equal(M.unsigned(sk, key_bits), ok)
    assert np.array_equal(perm.cpu().numpy().view(np.uint32), operm)


@pytest.mark.parametrize("n,key_bits,span", [(1 << 12, 32, 5), (1 << 13, 32, 7), (1 << 17, 32, 50),
                                             (1 << 16, 64, 30), (1 << 20, 32, 1000)])
def test_sort_ties_vs_oracle(gctx, M, n, key_bits, span):
    """Keys drawn from a few values: which of equal keys goes first is fixed by the
    bitonic network's compare-exchanges, so the permutation must be the oracle's."""
    import torch

    rng = np.random.default_rng(n + span)
    k = rng.integers(0, span, n)
    dt = torch.int32 if key_bits == 32 else torch.int64
    keys = torch.as_tensor(k.astype(np.int32 if key_bits == 32 else np.int64), dtype=dt, device="cuda")
    sk, perm = M.sort_by_key(gctx, keys, key_bits=key_bits)
    ok, operm = O.bitonic_sort(k.astype(np.uint32 if key_bits == 32 else np.uint64))
    assert np.array_equal(M.unsigned(sk, key_bits), ok)
    assert np.array_equal(perm.cpu().numpy().view(np.uint32), operm)


@pytest.mark.parametrize("n,level", [(2, 3), (100, 0), (5000, 1), (5000, 3), (120000, 3), (120001, 2)])
def test_tree_vs_oracle(gctx, M, n, level):
    rng = np.random.default_rng(n + level)
    pos = _clustered(n, n + 1)
    h = 0.01 + 0.02 * rng.random(n)
    bmin, bmax = pos.min(0), pos.max(0)
    t = M.Tree(gctx, pos, bmin, bmax, level, h=h, htol=1.1)
    e = t.export()
    o = O.Tree(pos, bmin, bmax, level, h=h, htol=1.1)
    assert t.leaf_count == o.leaf_count
    assert np.array_equal(e["sorted_keys"], o.sorted_keys.astype(np.uint32))
    assert np.array_equal(e["sort_index"], o.sort_index)
    assert np.array_equal(e["reduc"], o.reduc)
    for k in ("lchild_id", "rchild_id", "lchild_flag", "rchild_flag", "endrange"):
        assert np.array_equal(e[k], getattr(o, k)), k
    assert np.array_equal(e["aabb_min"], o.aabb_min)
    assert np.array_equal(e["aabb_max"], o.aabb_max)
    assert np.array_equal(e["rint"], o.rint)


def _lattice(n_cells, jitter, seed):
    from shamrock_gb300 import setups

    return setups.sedov_taylor(n_cells, jitter=jitter, seed=seed)


@pytest.mark.parametrize("n_cells,jitter", [(6, 0.0), (8, 0.05), (12, 0.1)])
def test_periodic_ghosts_vs_oracle(gctx, M, n_cells, jitter):
    s = _lattice(n_cells, jitter, 3)
    g = M.periodic_ghosts(gctx, s["pos"], s["h"], [0, 0, 0], [1, 1, 1], 1.1)
    src, off = O.periodic_ghosts(s["pos"], s["h"], [0, 0, 0], [1, 1, 1], 1.1)
    assert np.array_equal(g["src"], src)
    n = len(s["h"])
    assert np.array_equal(g["merged_pos"][:n], s["pos"])
    assert np.array_equal(g["merged_pos"][n:], s["pos"][src] + off)
    assert np.array_equal(g["merged_h"][n:], s["h"][src])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("n_cells,jitter,level", [(6, 0.0, 3), (8, 0.05, 3), (10, 0.2, 1), (12, 0.05, 3)])
def test_neighbour_cache_vs_oracle(gctx, M, n_cells, jitter, level, precision):
    """Bit-exact CSR; the mixed build pre-tests pairs in FP32 and must give the same cache
    (the unjittered lattice puts many pairs exactly on the threshold)."""
    s = _lattice(n_cells, jitter, 5)
    n = len(s["h"])
    g = M.periodic_ghosts(gctx, s["pos"], s["h"], [0, 0, 0], [1, 1, 1], 1.1)
    mpos, mh = g["merged_pos"], g["merged_h"]
    lo = np.nextafter(mpos.min(0), -np.inf)
    hi = np.nextafter(mpos.max(0), np.inf)
    t = M.Tree(gctx, mpos, lo, hi, level, h=mh, htol=1.1)
    csr = M.neighbour_cache(gctx, n, 1.1, precision)
    o = O.Tree(mpos, lo, hi, level, h=mh, htol=1.1)
    oc = o.neigh_cache(mpos, mh, n, 1.1)
    assert np.array_equal(csr["cnt"].cpu().numpy().view(np.uint32), oc["cnt"])
    assert np.array_equal(csr["scanned"].cpu().numpy().view(np.uint32), oc["scanned"])
    assert np.array_equal(csr["entries"].cpu().numpy().view(np.uint32), oc["entries"])


@pytest.mark.parametrize("budget", [1 << 10, None])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_neighbour_cache_slot_paths(gctx, M, budget, precision):
    """h three times the lattice estimate puts ~27x the usual neighbours in every row,
    overflowing the initial one-pass slots (256 leaves, 192 entries): with the default
    budget the builds rerun in one pass with grown slots, with a 1 KiB budget the exact
    two-pass builds run.  Both give the oracle's cache bit for bit."""
    s = _lattice(10, 0.05, 9)
    n = len(s["h"])
    h = s["h"] * 3.0
    g = M.periodic_ghosts(gctx, s["pos"], h, [0, 0, 0], [1, 1, 1], 1.1)
    mpos, mh = g["merged_pos"], g["merged_h"]
    lo = np.nextafter(mpos.min(0), -np.inf)
    hi = np.nextafter(mpos.max(0), np.inf)
    gctx.call("gbsph_set_cache_budget", 0 if budget is None else budget)
    try:
        t = M.Tree(gctx, mpos, lo, hi, 3, h=mh, htol=1.1)
        csr = M.neighbour_cache(gctx, n, 1.1, precision)
    finally:
        gctx.call("gbsph_set_cache_budget", 0)
    o = O.Tree(mpos, lo, hi, 3, h=mh, htol=1.1)
    oc = o.neigh_cache(mpos, mh, n, 1.1)
    assert oc["cnt"].max() > 192
    assert np.array_equal(csr["cnt"].cpu().numpy().view(np.uint32), oc["cnt"])
    assert np.array_equal(csr["scanned"].cpu().numpy().view(np.uint32), oc["scanned"])
    assert np.array_equal(csr["entries"].cpu().numpy().view(np.uint32), oc["entries"])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_neighbour_cache_varying_h_vs_oracle(gctx, M, precision):
    """Smoothing lengths spread over a factor 3 plus a dense clump with small h, free
    boundary.  Stage 1 drops, per owner leaf, the leaves that none of its rows can pair
    with (by the largest threshold of the rows it owns) and skips leaves that own no row;
    the cache must still be the oracle's bit for bit."""
    rng = np.random.default_rng(21)
    s = _lattice(12, 0.1, 21)
    n0 = len(s["h"])
    clump = 0.5 + 0.03 * rng.standard_normal((2000, 3))
    pos = np.concatenate([s["pos"], clump])
    h = np.concatenate([s["h"] * rng.uniform(0.6, 1.8, n0),
                        0.15 * s["h"][0] * rng.uniform(0.5, 2.0, 2000)])
    n = len(h)
    lo = np.nextafter(pos.min(0), -np.inf)
    hi = np.nextafter(pos.max(0), np.inf)
    t = M.Tree(gctx, pos, lo, hi, 3, h=h, htol=1.1)
    csr = M.neighbour_cache(gctx, n, 1.1, precision)
    o = O.Tree(pos, lo, hi, 3, h=h, htol=1.1)
    oc = o.neigh_cache(pos, h, n, 1.1)
    assert np.array_equal(csr["cnt"].cpu().numpy().view(np.uint32), oc["cnt"])
    assert np.array_equal(csr["scanned"].cpu().numpy().view(np.uint32), oc["scanned"])
    assert np.array_equal(csr["entries"].cpu().numpy().view(np.uint32), oc["entries"])


def test_sort_properties_large(gctx, M):
    """Size-independent properties at 2^24 keys: sorted output, permutation, stable pairing."""
    n = 1 << 24
    rng = np.random.default_rng(7)
    keys = rng.integers(0, 1 << 20, size=n, dtype=np.uint32)  # many equal keys
    import torch

    kt = torch.as_tensor(keys.view(np.int32), device="cuda")
    sk, perm = M.sort_by_key(gctx, kt, key_bits=32)
    s = M.unsigned(sk, 32)
    p = perm.cpu().numpy().view(np.uint32)
    assert np.all(s[1:] >= s[:-1])
    assert np.array_equal(np.sort(p), np.arange(n, dtype=np.uint32))
    assert np.array_equal(keys[p], s)
