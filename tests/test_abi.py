"""The C-ABI library builds for sm_103a, loads, and exports every entry point that
include/gbsph.h declares (no GPU needed: nothing is called)."""

import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _header_functions():
    src = open(os.path.join(ROOT, "include", "gbsph.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gbsph_\w+)\s*\(", src)))


@pytest.fixture(scope="module")
def libpath():
    from shamrock_gb300 import build

    return build.build()


def test_header_declares_entry_points():
    fns = _header_functions()
    for must in ("gbsph_create", "gbsph_build_tree", "gbsph_neighbour_cache", "gbsph_h_iterate",
                 "gbsph_omega", "gbsph_eos_adiabatic", "gbsph_derivs_constAV",
                 "gbsph_periodic_ghosts", "gbsph_evolve_once"):
        assert must in fns


def test_library_exports_every_declared_symbol(libpath):
    lib = ctypes.CDLL(libpath)
    missing = [f for f in _header_functions() if not hasattr(lib, f)]
    assert not missing, missing


def test_binding_table_matches_header():
    from shamrock_gb300 import _lib

    assert set(_lib.exported_symbols()) <= set(_header_functions())


def test_build_targets_sm103a_only():
    from shamrock_gb300 import build

    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_header_compiles_as_c(tmp_path):
    src = tmp_path / "t.c"
    src.write_text('#include "gbsph.h"\nint main(void){gbsph_config c; (void)c; return 0;}\n')
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                        "-c", str(src), "-o", str(tmp_path / "t.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_struct_layouts_match_header(tmp_path):
    """Every ctypes mirror of a header struct has the C struct's size and the C offset of
    each of its fields (the drop-in boundary passes these structs by pointer)."""
    import ctypes as C

    from shamrock_gb300 import _lib

    pairs = [("gbsph_vec3", _lib.Vec3), ("gbsph_particles", _lib.Particles),
             ("gbsph_config", _lib.Config), ("gbsph_time_state", _lib.TimeState),
             ("gbsph_step_log", _lib.StepLog), ("gbsph_cotangents", _lib.Cotangents)]
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "gbsph.h"', "int main(void){"]
    expect = []
    for cname, py in pairs:
        lines.append(f'printf("%zu\\n", sizeof({cname}));')
        expect.append(C.sizeof(py))
        for fname, _ in py._fields_:
            lines.append(f'printf("%zu\\n", offsetof({cname}, {fname}));')
            expect.append(getattr(py, fname).offset)
    lines.append("return 0;}")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    r = subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()]
    assert got == expect
