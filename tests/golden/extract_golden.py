"""Extract the reference's own golden vectors for the SPH hot path into JSON fixtures.

Reads the Shamrock unit-test sources as text (they are C++ and cannot be built
here) and writes one JSON fixture per test file into this directory.  The
fixtures are committed; this script only needs to be re-run if the reference
tests change.  Usage::

    python tests/golden/extract_golden.py /path/to/shamrock/checkout

Fixtures produced (source files inside the Shamrock tree):

- morton_code_set.json       src/tests/shamtree/MortonCodeSetTests.cpp
- morton_reduced_set.json    src/tests/shamtree/MortonReducedSetTests.cpp
- karras_radix_tree.json     src/tests/shamtree/KarrasRadixTreeTests.cpp
- karras_radix_tree_aabb.json src/tests/shamtree/KarrasRadixTreeAABBTests.cpp
- clbvh_object_iterator.json src/tests/shamtree/CLBVHObjectIteratorTests.cpp
- h_iteration.json           src/tests/shammodels/sph/modules/IterateSmoothingLengthDensityTests.cpp
- sedov_taylor_table.json    src/shamphys/src/sedov_soluce_arrays.hpp (every 15th point of the
                             reference's tabulated Sedov-Taylor solution, plus the points
                             either side of the shock)
"""

import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def _strip_comments(src):
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return re.sub(r"//[^\n]*", "", src)


def _split_tests(src):
    """Return [(test_name, body)] for every NEW_TEST block."""
    out = []
    heads = list(re.finditer(r'NEW_TEST\(\s*\w+\s*,\s*"([^"]+)"\s*,\s*\d+\s*\)\s*\{', src))
    for k, m in enumerate(heads):
        end = heads[k + 1].start() if k + 1 < len(heads) else len(src)
        out.append((m.group(1), src[m.end():end]))
    return out


def _parse_number(tok):
    tok = tok.strip()
    tok = re.sub(r"_u64$|_u32$", "", tok)
    tok = tok.rstrip("uUlL") if re.match(r"^(0b[01]+|\d+)[uUlL]*$", tok) else tok
    if tok.startswith("0b"):
        return int(tok[2:], 2)
    if re.match(r"^-?\d+$", tok):
        return int(tok)
    return float(tok)


def _parse_values(body):
    """Parse an initializer list body into a flat list of numbers or of 3-tuples."""
    body = body.strip()
    vecs = re.findall(r"(?:Tvec\s*\(|\{)\s*([^{}()]+?)\s*(?:\)|\})", body)
    if vecs and ("Tvec" in body or body.lstrip().startswith("{")):
        return [[_parse_number(x) for x in v.split(",")] for v in vecs]
    toks = [t for t in body.replace("\n", " ").split(",") if t.strip()]
    return [_parse_number(t) for t in toks]


def _vectors(test_body):
    res = {}
    pat = re.compile(r"std::vector<([\w:]+)>\s+(\w+)\s*(?:=\s*)?\{", re.S)
    for m in pat.finditer(test_body):
        start = m.end()
        depth, i = 1, start
        while depth:
            if test_body[i] == "{":
                depth += 1
            elif test_body[i] == "}":
                depth -= 1
            i += 1
        res[m.group(2)] = _parse_values(test_body[start:i - 1])
    return res


def _calls(test_body, fname):
    """Last numeric argument of every call to `fname` in the body."""
    vals = []
    for m in re.finditer(re.escape(fname) + r"\((.*?)\);", test_body, flags=re.S):
        last = m.group(1).split(",")[-1].strip()
        try:
            vals.append(_parse_number(last))
        except ValueError:
            pass
    return vals


def _scalar_requires(test_body):
    res = {}
    for m in re.finditer(r"REQUIRE_EQUAL\(\s*([\w\.\(\)]+?)\s*,\s*(\d+)\s*\)", test_body):
        res[m.group(1)] = int(m.group(2))
    return res


def extract(ref_root):
    tests_root = os.path.join(ref_root, "src", "tests")
    files = {
        "morton_code_set.json": "shamtree/MortonCodeSetTests.cpp",
        "morton_reduced_set.json": "shamtree/MortonReducedSetTests.cpp",
        "karras_radix_tree.json": "shamtree/KarrasRadixTreeTests.cpp",
        "karras_radix_tree_aabb.json": "shamtree/KarrasRadixTreeAABBTests.cpp",
        "clbvh_object_iterator.json": "shamtree/CLBVHObjectIteratorTests.cpp",
        "h_iteration.json": "shammodels/sph/modules/IterateSmoothingLengthDensityTests.cpp",
    }
    for out_name, rel in files.items():
        with open(os.path.join(tests_root, rel)) as f:
            src = _strip_comments(f.read())
        fixture = {"source": "src/tests/" + rel, "file_level": _vectors(src.split("NEW_TEST")[0]),
                   "tests": {}}
        # the h-iteration test builds its inputs in a helper; keep its constants too
        for name, body in _split_tests(src):
            fixture["tests"][name] = {
                "vectors": _vectors(body),
                "reduce_morton_set_level": _calls(body, "reduce_morton_set"),
                "rebuild_from_positions_level": _calls(body, "rebuild_from_positions"),
                "scalar_requires": _scalar_requires(body),
                "constants": {m.group(1): _parse_number(m.group(2)) for m in re.finditer(
                    r"constexpr\s+Tscal\s+(\w+)\s*=\s*([-\d\.e]+)\s*;", body)},
            }
        with open(os.path.join(HERE, out_name), "w") as f:
            json.dump(fixture, f, indent=1)
        print("wrote", out_name, "tests:", list(fixture["tests"]))


def extract_sedov(ref_root):
    """Subsample of the reference's Sedov-Taylor table (gamma 5/3, E = 1, rho0 = 1, t = 0.1)."""
    path = os.path.join(ref_root, "src", "shamphys", "src", "sedov_soluce_arrays.hpp")
    with open(path) as f:
        src = _strip_comments(f.read())
    cols = {}
    for name in ("r_theo", "vr_theo", "rho_theo", "p_theo"):
        m = re.search(r"double\s+" + name + r"\[\]\s*=\s*\{(.*?)\};", src, re.S)
        cols[name] = [float(t) for t in m.group(1).replace("\n", " ").split(",") if t.strip()]
    n = len(cols["r_theo"])
    jump = max(range(1, n), key=lambda i: abs(cols["rho_theo"][i] - cols["rho_theo"][i - 1]))
    keep = sorted(set(range(0, n, 15)) | set(range(max(jump - 3, 0), min(jump + 3, n))) | {n - 1})
    fixture = {"source": "src/shamphys/src/sedov_soluce_arrays.hpp", "count_in_source": n,
               "case": {"gamma": 5.0 / 3.0, "e_blast": 1.0, "rho0": 1.0, "t": 0.1},
               "index": keep}
    for name, vals in cols.items():
        fixture[name] = [vals[i] for i in keep]
    with open(os.path.join(HERE, "sedov_taylor_table.json"), "w") as f:
        json.dump(fixture, f, indent=0)
    print("wrote sedov_taylor_table.json points:", len(keep))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python extract_golden.py <path of the Shamrock source checkout>")
    root = sys.argv[1]
    extract(root)
    extract_sedov(root)
