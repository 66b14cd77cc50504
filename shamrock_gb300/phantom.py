"""Phantom dump files: read, write, compare, and the conversions to and from the model.

Mirrors the reference's Phantom I/O (shammodels/sph/io/PhantomDump.hpp and
src/io/PhantomDump.cpp, the Fortran record layer shambase/fortran_io.hpp, the EOS, AV,
unit and boundary conversions of src/io/Phantom2Shamrock.cpp and
src/io/PhantomDumpEOSUtils.cpp, and the Python names of src/pyPhantomDump.cpp):
``load_phantom_dump(fname)``, ``PhantomDump.save_dump / read_header_float /
read_header_int / print_state``, ``compare_phantom_dumps``.  The model side
(``gen_config_from_phantom_dump``, ``init_from_phantom_dump``, ``make_phantom_dump``,
shammodels/sph/src/Model.cpp:1203-1621) is in model.py on top of the helpers here.

File layout (sequential Fortran records: a 4-byte little-endian byte count, the
payload, the byte count again):
  1. i1 (int32), r1 (float64), i2, iversion, i3 (int32)        magic numbers
  2. fileid, 100 characters
  3. eight header tables, for the types int (Fortran default), int8, int16, int32,
     int64, real (float64), real4, real8: a record with the entry count n, then, when
     n > 0, a record of n 16-character tags and a record of n values
  4. nblocks (int32)
  5. per block: tot_count (int64) and the eight array counts (int32 each)
  6. per block, per type in the same order, per array: a 16-character tag record and
     a record of tot_count values.
Byte order is the host's in the reference (it streams raw values); this module writes
and reads little endian, the byte order of both x86-64 and AArch64 hosts.

A record longer than 2^31 - 1 bytes cannot be described by its 4-byte count; the
reference's writer would wrap the count, this one refuses such a file.
"""

from __future__ import annotations

import math
import struct
import sys
import warnings

import numpy as np

__all__ = ["PhantomDump", "PhantomDumpBlock", "PhantomDumpBlockArray", "PhantomDumpTableHeader",
           "load_phantom_dump", "compare_phantom_dumps", "TYPE_KINDS"]

# (name, numpy dtype) of the eight typed tables/arrays, in file order
TYPE_KINDS = (("fort_int", np.dtype("<i4")), ("i8", np.dtype("i1")), ("i16", np.dtype("<i2")),
              ("i32", np.dtype("<i4")), ("i64", np.dtype("<i8")), ("fort_real", np.dtype("<f8")),
              ("f32", np.dtype("<f4")), ("f64", np.dtype("<f8")))
_KIND_DTYPE = dict(TYPE_KINDS)
_INT_KINDS = ("fort_int", "i8", "i16", "i32", "i64")
_FLOAT_KINDS = ("fort_real", "f32", "f64")
MAGIC_I1, MAGIC_I2, MAGIC_I3 = 60769, 60878, 690706
_MAX_RECORD = 2**31 - 1


def _tag(s: str) -> str:
    """A tag as stored: the name left-justified in 16 characters (fmt "{:16s}")."""
    return f"{s:16s}"


class FortranIOError(RuntimeError):
    pass


class _Writer:
    """Sequential unformatted Fortran records (shambase/fortran_io.hpp FortranIOFile)."""

    def __init__(self):
        self.parts = []

    def record(self, payload):
        """payload: bytes or a byte view (arrays are kept as views until written)."""
        n = len(payload)
        if n > _MAX_RECORD:
            raise FortranIOError(f"a Fortran record of {n} bytes exceeds the 4-byte record length")
        mark = struct.pack("<i", n)
        self.parts += [mark, payload, mark]

    def values(self, fmt: str, *vals):
        self.record(struct.pack("<" + fmt, *vals))

    def string(self, s: str, length: int):
        b = s.encode("latin-1")
        if len(b) != length:
            raise FortranIOError(f"string of {len(b)} characters where {length} are stored")
        self.record(b)

    def array(self, vals: np.ndarray, dtype: np.dtype, count: int):
        a = np.ascontiguousarray(vals, dtype=dtype)
        if count > a.size:
            raise FortranIOError("val count is higher than vec size")
        self.record(memoryview(np.ascontiguousarray(a[:count])).cast("B"))

    def getvalue(self) -> bytes:
        return b"".join(self.parts)


class _Reader:
    def __init__(self, data: bytes):
        self.buf = memoryview(data)
        self.pos = 0

    def record(self, expect: int) -> memoryview:
        if self.pos + 4 > len(self.buf):
            raise FortranIOError("the byte count is not correct (end of file)")
        (n,) = struct.unpack_from("<i", self.buf, self.pos)
        if n != expect:
            raise FortranIOError(f"the byte count is not correct ({n} where {expect} expected)")
        start = self.pos + 4
        end = start + n
        if end + 4 > len(self.buf):
            raise FortranIOError("the byte count is not correct (truncated record)")
        (n2,) = struct.unpack_from("<i", self.buf, end)
        if n2 != n:
            raise FortranIOError("fortran 4 bytes invalid")
        self.pos = end + 4
        return self.buf[start:end]

    def values(self, fmt: str):
        return struct.unpack("<" + fmt, self.record(struct.calcsize("<" + fmt)))

    def string(self, length: int) -> str:
        return bytes(self.record(length)).decode("latin-1")

    def strings(self, length: int, count: int):
        raw = bytes(self.record(length * count)).decode("latin-1")
        return [raw[i * length:(i + 1) * length] for i in range(count)]

    def array(self, dtype: np.dtype, count: int) -> np.ndarray:
        return np.frombuffer(self.record(dtype.itemsize * count), dtype=dtype).copy()

    def finished(self) -> bool:
        return self.pos == len(self.buf)


class PhantomDumpTableHeader:
    """One typed header table: (tag, value) entries in file order; tags may repeat
    (npartoftype, massoftype)."""

    def __init__(self, kind: str):
        self.kind = kind
        self.entries: list[tuple[str, object]] = []

    def add(self, s: str, val):
        self.entries.append((_tag(s), val))

    def fetch(self, tag16: str):
        """Last value stored under the padded tag, or None."""
        ret = None
        for k, v in self.entries:
            if k == tag16:
                ret = v
        return ret

    def fetch_multiple(self, tag16: str):
        return [v for k, v in self.entries if k == tag16]

    def _write(self, w: _Writer):
        n = len(self.entries)
        w.values("i", n)
        if n == 0:
            return
        w.string("".join(k for k, _ in self.entries), 16 * n)
        w.array(np.array([v for _, v in self.entries]), _KIND_DTYPE[self.kind], n)

    @classmethod
    def _read(cls, r: _Reader, kind: str):
        t = cls(kind)
        (n,) = r.values("i")
        if n == 0:
            return t
        tags = r.strings(16, n)
        vals = r.array(_KIND_DTYPE[kind], n)
        t.entries = [(k, v.item()) for k, v in zip(tags, vals)]
        return t

    def print_state(self, out=None):
        for k, v in self.entries:
            print(k, v, file=out or sys.stdout)


class PhantomDumpBlockArray:
    def __init__(self, tag: str, kind: str, vals=None):
        self.tag = tag  # padded to 16 characters
        self.kind = kind
        self.vals = np.zeros(0, _KIND_DTYPE[kind]) if vals is None else np.asarray(
            vals, _KIND_DTYPE[kind])

    def print_state(self, out=None):
        print("tag =", self.tag, "size =", self.vals.size, file=out or sys.stdout)


class PhantomDumpBlock:
    """A block of per-particle arrays (block 0: gas particles, block 1: sink particles)."""

    def __init__(self, tot_count: int = 0):
        self.tot_count = int(tot_count)
        self.arrays = {kind: [] for kind, _ in TYPE_KINDS}

    def get_ref(self, kind: str, s: str) -> PhantomDumpBlockArray:
        """The array of this kind tagged s, appended empty if absent (get_ref_<kind>)."""
        tag = _tag(s)
        for a in self.arrays[kind]:
            if a.tag == tag:
                return a
        a = PhantomDumpBlockArray(tag, kind)
        self.arrays[kind].append(a)
        return a

    def set_array(self, kind: str, s: str, vals):
        self.get_ref(kind, s).vals = np.asarray(vals, _KIND_DTYPE[kind]).copy()

    def fill_vec(self, field_name: str) -> np.ndarray:
        """All values tagged field_name, across the eight kinds in file order, as float64
        (the reference appends each match to one vector of the caller's type)."""
        tag = _tag(field_name)
        parts = [a.vals.astype(np.float64) for kind, _ in TYPE_KINDS for a in self.arrays[kind]
                 if a.tag == tag]
        return np.concatenate(parts) if parts else np.zeros(0)

    def counts(self):
        return [len(self.arrays[kind]) for kind, _ in TYPE_KINDS]

    def print_state(self, out=None):
        out = out or sys.stdout
        for kind, _ in TYPE_KINDS:
            print(f"--blocks_{kind:9s}--", file=out)
            for a in self.arrays[kind]:
                a.print_state(out)


class PhantomDump:
    """In-memory Phantom dump (shammodels::sph::PhantomDump)."""

    def __init__(self):
        self.i1 = self.i2 = self.i3 = 0
        self.iversion = 0
        self.r1 = 0.0
        self.fileid = " " * 100
        self.tables = {kind: PhantomDumpTableHeader(kind) for kind, _ in TYPE_KINDS}
        self.blocks: list[PhantomDumpBlock] = []

    def override_magic_number(self):
        self.i1, self.i2, self.i3 = MAGIC_I1, MAGIC_I2, MAGIC_I3
        self.r1 = float(self.i2)

    def check_magic_numbers(self):
        if (self.i1 != MAGIC_I1 or self.i2 != MAGIC_I2 or self.i3 != MAGIC_I3
                or self.r1 != self.i2):
            raise FortranIOError("not a Phantom dump: the magic numbers do not match")

    # -- file I/O
    def gen_file(self) -> bytes:
        """The dump as the bytes of a Phantom file (PhantomDump::gen_file)."""
        return self._records().getvalue()

    def _records(self) -> _Writer:
        w = _Writer()
        w.values("idiii", self.i1, self.r1, self.i2, self.iversion, self.i3)
        w.string(self.fileid, 100)
        for kind, _ in TYPE_KINDS:
            self.tables[kind]._write(w)
        w.values("i", len(self.blocks))
        for b in self.blocks:
            w.values("q8i", b.tot_count, *b.counts())
        for b in self.blocks:
            for kind, dt in TYPE_KINDS:
                for a in b.arrays[kind]:
                    w.string(a.tag, 16)
                    w.array(a.vals, dt, b.tot_count)
        return w

    def save_dump(self, fname: str):
        """Writes the records one by one (no whole-file copy in memory)."""
        parts = self._records().parts
        with open(fname, "wb") as f:
            f.writelines(parts)

    @classmethod
    def from_bytes(cls, data: bytes) -> "PhantomDump":
        r = _Reader(data)
        d = cls()
        d.i1, d.r1, d.i2, d.iversion, d.i3 = r.values("idiii")
        d.check_magic_numbers()
        d.fileid = r.string(100)
        for kind, _ in TYPE_KINDS:
            d.tables[kind] = PhantomDumpTableHeader._read(r, kind)
        (nblocks,) = r.values("i")
        heads = [r.values("q8i") for _ in range(nblocks)]
        for h in heads:
            b = PhantomDumpBlock(h[0])
            for (kind, dt), cnt in zip(TYPE_KINDS, h[1:]):
                for _ in range(cnt):
                    tag = r.string(16)
                    b.arrays[kind].append(PhantomDumpBlockArray(tag, kind, r.array(dt, b.tot_count)))
            d.blocks.append(b)
        if not r.finished():
            warnings.warn("[PhantomReader] some data was not read")
        return d

    # -- header queries (names padded to 16 characters before the lookup)
    def has_header_entry(self, s: str) -> bool:
        tag = _tag(s)
        return any(t.fetch(tag) is not None for t in self.tables.values())

    def read_header_float(self, s: str) -> float:
        tag = _tag(s)
        for kind in _FLOAT_KINDS:
            v = self.tables[kind].fetch(tag)
            if v is not None:
                return float(v)
        raise KeyError("the entry cannot be found : " + tag)

    def read_header_floats(self, s: str):
        tag = _tag(s)
        return [float(v) for kind in _FLOAT_KINDS for v in self.tables[kind].fetch_multiple(tag)]

    def read_header_int(self, s: str) -> int:
        tag = _tag(s)
        for kind in _INT_KINDS:
            v = self.tables[kind].fetch(tag)
            if v is not None:
                return int(v)
        raise KeyError("the entry cannot be found")

    def read_header_ints(self, s: str):
        tag = _tag(s)
        return [int(v) for kind in _INT_KINDS for v in self.tables[kind].fetch_multiple(tag)]

    def print_state(self, out=None):
        out = out or sys.stdout
        print("--- dump state ---", file=out)
        for kind, _ in TYPE_KINDS:
            t = self.tables[kind]
            print(f"table_header_{kind} len =", len(t.entries), file=out)
            t.print_state(out)
        for i, b in enumerate(self.blocks):
            print("block ", i, ":", file=out)
            b.print_state(out)
        print("------------------", file=out)


# the typed tables under the reference's member names (table_header_fort_int, ...)
for _kind, _ in TYPE_KINDS:
    setattr(PhantomDump, "table_header_" + _kind,
            property(lambda self, k=_kind: self.tables[k], doc=f"the {_kind} header table"))
del _kind


def load_phantom_dump(fname: str) -> PhantomDump:
    """shamrock.load_phantom_dump (pyPhantomDump.cpp:40-43)."""
    with open(fname, "rb") as f:
        return PhantomDump.from_bytes(f.read())


def compare_phantom_dumps(dump_ref: PhantomDump, dump_comp: PhantomDump) -> bool:
    """True when both headers hold the same keys with the same values (every typed
    table folded into one map, the last value of a repeated key kept, as
    PhantomDump.cpp:391-463).  Each difference is reported as a warning."""

    def load(d):
        m = {}
        for kind, _ in TYPE_KINDS:
            for k, v in d.tables[kind].entries:
                m[k] = float(v)
        return m

    a, b = load(dump_ref), load(dump_comp)
    offenses = 0
    for k in sorted(set(a) - set(b)):
        warnings.warn(f"PhantomDump: the dump we are comparing against is missing the key {k}")
        offenses += 1
    for k in sorted(set(a) & set(b)):
        if a[k] != b[k] and not (math.isnan(a[k]) and math.isnan(b[k])):
            warnings.warn(f"PhantomDump: mismatch in the header key {k}, ref={a[k]}, comp={b[k]}")
            offenses += 1
    for k in sorted(set(b) - set(a)):
        warnings.warn(f"PhantomDump: the dump we are comparing against has the extra key {k}")
        offenses += 1
    return offenses == 0


# ---------------------------------------------------------------- EOS headers
# (src/io/PhantomDumpEOSUtils.cpp: the EOS options Phantom stores with each ieos)

def _write_headeropts_eos(dump: PhantomDump, ieos: int, gamma=1.0, polyk=0.0, qfacdisc=0.75):
    dump.table_header_i32.add("ieos", ieos)
    dump.table_header_i32.add("isink", 0)
    dump.table_header_fort_real.add("gamma", gamma)
    dump.table_header_fort_real.add("RK2", 1.5 * polyk)
    dump.table_header_fort_real.add("polyk2", 0.0)
    dump.table_header_fort_real.add("qfacdisc", qfacdisc)
    dump.table_header_fort_real.add("qfacdisc2", 0.75)


def _read_headeropts_eos(dump: PhantomDump, ieos: int):
    have = dump.read_header_int("ieos")
    if have != ieos:
        raise ValueError(f"You are querying phantom dump eos {ieos} parameters, even though "
                         f"ieos is {have}")
    return dict(gamma=dump.read_header_float("gamma"),
                polyk=2.0 / 3.0 * dump.read_header_float("RK2"),
                polyk2=dump.read_header_float("polyk2"),
                qfacdisc=dump.read_header_float("qfacdisc"),
                qfacdisc2=dump.read_header_float("qfacdisc2"),
                isink=dump.read_header_int("isink"))


def eos_config_from_dump(dump: PhantomDump, bypass_error: bool = False):
    """The model's EOS dict for the dump's ieos (Phantom2Shamrock.cpp:19-55): 2 adiabatic,
    3 locally isothermal (Lodato & Pringle 2007, r0 = 1 since Phantom's polyk already
    holds cs0^2/r0^2).  ieos 1, 13 and 14 (isothermal, Farris et al. 2014) are not on the
    GB300 path; like every other ieos they raise unless bypass_error, which warns and
    returns None."""
    ieos = dump.read_header_int("ieos")
    if ieos == 2:
        return dict(type="adiabatic", gamma=_read_headeropts_eos(dump, 2)["gamma"])
    if ieos == 3:
        o = _read_headeropts_eos(dump, 3)
        return dict(type="locally_isothermal_lp07", cs0=math.sqrt(o["polyk"]), q=o["qfacdisc"],
                    r0=1.0)
    msg = f"loading phantom ieos={ieos} is not implemented on the GB300 path"
    if bypass_error:
        warnings.warn(msg)
        return None
    raise NotImplementedError(msg)


def write_eos_in_dump(eos: dict, dump: PhantomDump, bypass_error: bool = False):
    """Phantom2Shamrock.cpp:57-106 for the EOS kinds of the GB300 path."""
    if eos is not None and eos["type"] == "adiabatic":
        _write_headeropts_eos(dump, 2, gamma=eos["gamma"])
    elif eos is not None and eos["type"] == "locally_isothermal_lp07":
        _write_headeropts_eos(dump, 3, polyk=eos["cs0"] ** 2 / eos["r0"] ** 2, qfacdisc=eos["q"])
    else:
        msg = "The current EOS is not implemented in phantom dump conversion"
        if not bypass_error:
            raise NotImplementedError(msg)
        warnings.warn(msg)


def write_units_in_dump(units, dump: PhantomDump):
    """Phantom2Shamrock.cpp:135-166: udist, umass, utime and the magnetic-field unit of
    the Gaussian system; 1, 1, 1, 3.54491 without a unit system."""
    if units is None:
        warnings.warn("no units are set, defaulting to SI")
        for k, v in (("udist", 1.0), ("umass", 1.0), ("utime", 1.0), ("umagfd", 3.54491)):
            dump.table_header_f64.add(k, v)
        return
    udist, umass, utime = units.unit_length, units.unit_mass, units.unit_time
    dump.table_header_f64.add("udist", udist)
    dump.table_header_f64.add("umass", umass)
    dump.table_header_f64.add("utime", utime)
    ucharge = math.sqrt(umass * udist / (4.0 * math.pi))
    dump.table_header_f64.add("umagfd", umass / (utime * ucharge))
