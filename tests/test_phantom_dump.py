"""Phantom dump I/O (shamrock_gb300.phantom and the model's Phantom methods) on the CPU.

The reference's own test (src/tests/phantom_read_test.cpp) reads a Phantom dump, writes
it back and requires the two files to be byte-identical; its dumps (reference-files/
sedov_blast_phantom) are external, so here the file layout is pinned by bytes packed
independently with struct from the layout the reader follows (shambase/fortran_io.hpp,
PhantomDump.cpp:252-352), and the read-write identity is checked on dumps the model
writes."""

import math
import struct
import warnings

import numpy as np
import pytest

import shamrock_gb300 as sg
from shamrock_gb300 import phantom as P


def _rec(payload):
    m = struct.pack("<i", len(payload))
    return m + payload + m


def _tiny_dump():
    d = P.PhantomDump()
    d.override_magic_number()
    d.iversion = 1
    d.fileid = f"{'FT:test':100s}"
    d.table_header_fort_int.add("nparttot", 2)
    d.table_header_i8.add("flag", -3)
    d.table_header_i64.add("big", 2**40 + 5)
    d.table_header_fort_real.add("time", 0.25)
    d.table_header_fort_real.add("massoftype", 0.5)
    d.table_header_fort_real.add("massoftype", 0.0)
    d.table_header_f32.add("tolf", 1.5)
    b = P.PhantomDumpBlock(2)
    b.set_array("fort_real", "x", [1.0, -2.0])
    b.set_array("i8", "itype", [1, 2])
    b.set_array("f32", "h", [0.5, 0.25])
    d.blocks.append(b)
    return d


def _tiny_bytes():
    out = _rec(struct.pack("<idiii", 60769, 60878.0, 60878, 1, 690706))
    out += _rec(f"{'FT:test':100s}".encode())
    out += _rec(struct.pack("<i", 1)) + _rec(b"nparttot        ") + _rec(struct.pack("<i", 2))
    out += _rec(struct.pack("<i", 1)) + _rec(b"flag            ") + _rec(struct.pack("<b", -3))
    out += _rec(struct.pack("<i", 0))  # int16
    out += _rec(struct.pack("<i", 0))  # int32
    out += _rec(struct.pack("<i", 1)) + _rec(b"big             ") + _rec(struct.pack("<q", 2**40 + 5))
    out += (_rec(struct.pack("<i", 3)) + _rec(b"time            massoftype      massoftype      ")
            + _rec(struct.pack("<3d", 0.25, 0.5, 0.0)))
    out += _rec(struct.pack("<i", 1)) + _rec(b"tolf            ") + _rec(struct.pack("<f", 1.5))
    out += _rec(struct.pack("<i", 0))  # real*8
    out += _rec(struct.pack("<i", 1))  # nblocks
    out += _rec(struct.pack("<q8i", 2, 0, 1, 0, 0, 0, 1, 1, 0))
    out += _rec(b"itype           ") + _rec(struct.pack("<2b", 1, 2))
    out += _rec(b"x               ") + _rec(struct.pack("<2d", 1.0, -2.0))
    out += _rec(b"h               ") + _rec(struct.pack("<2f", 0.5, 0.25))
    return out


def test_layout_bytes():
    assert _tiny_dump().gen_file() == _tiny_bytes()


def test_read_write_identity(tmp_path):
    """phantom_read_test.cpp: load, write back, byte-identical."""
    raw = _tiny_bytes()
    f = tmp_path / "tiny"
    f.write_bytes(raw)
    d = sg.load_phantom_dump(str(f))
    out = tmp_path / "zout"
    d.save_dump(str(out))
    assert out.read_bytes() == raw
    assert d.read_header_int("nparttot") == 2
    assert d.read_header_ints("big") == [2**40 + 5]
    assert d.read_header_float("time") == 0.25
    assert d.read_header_floats("massoftype") == [0.5, 0.0]
    assert d.read_header_float("tolf") == 1.5
    assert d.has_header_entry("flag") and not d.has_header_entry("nope")
    assert np.array_equal(d.blocks[0].fill_vec("h"), [0.5, 0.25])
    with pytest.raises(KeyError):
        d.read_header_float("nope")


def test_reader_rejects_damage():
    raw = bytearray(_tiny_bytes())
    bad = bytes(raw[:4]) + struct.pack("<i", 1) + bytes(raw[8:])  # wrong i1
    with pytest.raises(P.FortranIOError):
        P.PhantomDump.from_bytes(bad)
    cut = bytes(raw[:-3])
    with pytest.raises(P.FortranIOError):
        P.PhantomDump.from_bytes(cut)
    wrong_mark = bytearray(raw)
    wrong_mark[-4:] = struct.pack("<i", 7)
    with pytest.raises(P.FortranIOError):
        P.PhantomDump.from_bytes(bytes(wrong_mark))
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        P.PhantomDump.from_bytes(bytes(raw) + b"\0" * 8)
    assert any("some data was not read" in str(x.message) for x in w)


def test_print_state_and_compare(capsys):
    a, b = _tiny_dump(), _tiny_dump()
    a.print_state()
    assert "table_header_fort_real len = 3" in capsys.readouterr().out
    assert sg.compare_phantom_dumps(a, b)
    b.table_header_fort_real.entries[0] = (f"{'time':16s}", 0.5)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        assert not sg.compare_phantom_dumps(a, b)
        c = _tiny_dump()
        c.table_header_f64.add("extra", 1.0)
        assert not sg.compare_phantom_dumps(a, c)


def _model(av="cd10", eos="adiabatic", periodic=True, n_cells=4, seed=2):
    from shamrock_gb300 import setups

    s = setups.sedov_taylor(n_cells, jitter=0.1, seed=seed)
    ctx = sg.Context()
    m = sg.get_Model_SPH(context=ctx, vector_type="f64_3", sph_kernel="M4")
    cfg = m.gen_default_config()
    if av == "cd10":
        cfg.set_artif_viscosity_VaryingCD10(alpha_min=0.0, alpha_max=1.0, sigma_decay=0.1,
                                            alpha_u=1.0, beta_AV=2.0)
    else:
        cfg.set_artif_viscosity_Constant(alpha_u=1.0, alpha_AV=1.0, beta_AV=2.0)
    if periodic:
        cfg.set_boundary_periodic()
    if eos == "adiabatic":
        cfg.set_eos_adiabatic(s["gamma"])
    else:
        cfg.set_eos_locally_isothermalLP07(cs0=0.3, q=0.25, r0=1.0)
    cfg.set_particle_mass(s["pmass"])
    cfg.set_cfl_cour(0.25)
    cfg.set_cfl_force(0.2)
    m.set_solver_config(cfg)
    m.resize_simulation_box(s["box_min"], s["box_max"])
    rng = np.random.default_rng(seed)
    n = len(s["h"])
    # h and alpha representable in real*4, as the dump stores them
    h = s["h"].astype(np.float32).astype(np.float64)
    alpha = rng.uniform(0, 1, n).astype(np.float32).astype(np.float64)
    m.set_particles(s["pos"], 0.1 * rng.standard_normal((n, 3)), h, s["u"], alpha=alpha)
    m.set_time(0.125)
    m.set_next_dt(1e-3)
    return m, s


@pytest.mark.parametrize("av,eos,periodic", [("cd10", "adiabatic", True),
                                              ("constant", "lp07", False)])
def test_model_dump_round_trip(tmp_path, av, eos, periodic):
    m, s = _model(av, eos, periodic)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")  # no unit system: SI defaults
        dump = m.make_phantom_dump()
    f = tmp_path / "dump_00000"
    dump.save_dump(str(f))
    back = sg.load_phantom_dump(str(f))
    assert back.gen_file() == f.read_bytes()
    assert sg.compare_phantom_dumps(dump, back)
    n = m.get_total_part_count()
    assert back.read_header_int("nparttot") == n
    # stored twice, in the default-int and the int64 tables
    assert back.read_header_ints("npartoftype") == ([n] + [0] * 7) * 2
    assert back.read_header_float("time") == 0.125
    assert back.read_header_float("dtmax") == 1e-3
    assert back.read_header_float("hfact") == 1.2
    assert back.read_header_int("ieos") == (2 if eos == "adiabatic" else 3)
    assert back.has_header_entry("xmin") == periodic
    blk = back.blocks[0]
    names = {k: [a.tag.strip() for a in blk.arrays[k]] for k, _ in P.TYPE_KINDS}
    assert names["fort_real"] == ["x", "y", "z", "vx", "vy", "vz", "u"]
    assert names["f32"] == (["h", "alpha", "divv"] if av == "cd10" else ["h"])

    cfg = m.gen_config_from_phantom_dump(back)
    assert cfg.gpart_mass == s["pmass"]
    assert (cfg.cfl_cour, cfg.cfl_force) == (0.25, 0.2)
    assert cfg.boundary == ("periodic" if periodic else "free")
    assert cfg.av["type"] == "cd10" and cfg.av["alpha_u"] == 1.0
    if eos == "adiabatic":
        assert cfg.eos == dict(type="adiabatic", gamma=s["gamma"])
    else:
        assert cfg.eos["type"] == "locally_isothermal_lp07"
        assert cfg.eos["cs0"] == pytest.approx(0.3, rel=1e-15) and cfg.eos["q"] == 0.25

    m2 = sg.get_Model_SPH(context=sg.Context(), vector_type="f64_3", sph_kernel="M4")
    m2.set_solver_config(cfg)
    m2.init_from_phantom_dump(back)
    a, b = m.collect_data(), m2.collect_data()
    for k in ("xyz", "vxyz", "hpart", "uint"):
        assert np.array_equal(a[k], b[k]), k
    if av == "cd10":
        assert np.array_equal(a["alpha_AV"], b["alpha_AV"])
    assert m2.get_time() == 0.125
    if periodic:
        assert np.array_equal(m2.box_min, m.box_min) and np.array_equal(m2.box_max, m.box_max)
    else:  # bounding box grown 1.2 times about its centre
        lo, hi = a["xyz"].min(0), a["xyz"].max(0)
        assert np.allclose(m2.box_max - m2.box_min, 1.2 * (hi - lo), rtol=1e-14)


def test_init_drops_dead_particles_and_scales_h():
    m, _ = _model("constant", "adiabatic", True)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        dump = m.make_phantom_dump()
    h = dump.blocks[0].get_ref("f32", "h")
    h.vals[:3] = -h.vals[:3]  # accreted / dead in Phantom's convention
    x = dump.blocks[0].get_ref("fort_real", "x")
    x.vals[5] = 1.0  # on the upper face: outside the half-open box
    m2 = sg.get_Model_SPH(context=sg.Context(), vector_type="f64_3", sph_kernel="M4")
    m2.set_solver_config(m.gen_config_from_phantom_dump(dump))
    m2.init_from_phantom_dump(dump, hpart_fact_load=2.0)
    a, b = m.collect_data(), m2.collect_data()
    keep = np.ones(len(a["hpart"]), bool)
    keep[:3] = False
    keep[5] = False
    assert m2.get_total_part_count() == keep.sum()
    assert np.array_equal(b["hpart"], 2.0 * a["hpart"][keep])
    assert np.array_equal(b["uint"], a["uint"][keep])


def test_units_and_eos_conversions():
    d = P.PhantomDump()
    u = sg.UnitSystem(unit_time=3.15e7, unit_length=1.496e11, unit_mass=1.989e30)
    P.write_units_in_dump(u, d)
    assert d.read_header_float("udist") == 1.496e11
    ucharge = math.sqrt(1.989e30 * 1.496e11 / (4 * math.pi))
    assert d.read_header_float("umagfd") == 1.989e30 / (3.15e7 * ucharge)
    cfg = sg.SolverConfig()
    cfg.set_units(u)
    assert cfg.constant_G == pytest.approx(6.6743015e-11 * 1.989e30 * 3.15e7**2 / 1.496e11**3)
    # LP07 with r0 != 1: Phantom's polyk holds cs0^2 / r0^2 and reads back with r0 = 1
    d2 = P.PhantomDump()
    P.write_eos_in_dump(dict(type="locally_isothermal_lp07", cs0=0.5, q=0.5, r0=2.0), d2)
    e = P.eos_config_from_dump(d2)
    assert e["cs0"] == pytest.approx(0.25, rel=1e-15) and e["r0"] == 1.0 and e["q"] == 0.5
    # EOS kinds off the path
    d3 = P.PhantomDump()
    P._write_headeropts_eos(d3, 1, polyk=0.04)
    with pytest.raises(NotImplementedError):
        P.eos_config_from_dump(d3)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        assert P.eos_config_from_dump(d3, bypass_error=True) is None
    with pytest.raises(ValueError):
        P._read_headeropts_eos(d3, 2)


def test_sink_block_is_refused():
    """Sink particles are not on the GB300 path: a dump holding any raises on loading
    (an empty sink block, as Phantom writes without sinks, is accepted)."""
    m, _ = _model("constant", "adiabatic", True)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        dump = m.make_phantom_dump()
    empty = P.PhantomDumpBlock(0)
    dump.blocks.append(empty)
    m2 = sg.get_Model_SPH(context=sg.Context(), vector_type="f64_3", sph_kernel="M4")
    m2.init_from_phantom_dump(dump)
    assert m2.get_total_part_count() == m.get_total_part_count()
    sinks = P.PhantomDumpBlock(1)
    for k in ("x", "y", "z", "m", "h", "vx", "vy", "vz"):
        sinks.set_array("fort_real", k, [0.5])
    dump.blocks[1] = sinks
    with pytest.raises(NotImplementedError):
        m2.init_from_phantom_dump(dump)
