"""Particle files in the reference's FastASCII format.

A particles set of the reference names a file and the fields it holds
(``<Load format="FastASCII" file=... fields="r, normal, ..."/>``).  Each
non-comment line is one particle: the fields in that order, a ``vec`` field
as ``dims`` numbers in 2-D and 4 in 3-D (the reference's vec is float2 /
float4).  The parser is native (``aqua_read_fastascii`` of the library,
following InputOutput/FastASCII.cpp and the line rules of
InputOutput/ASCII.cpp); the writer follows ASCII::print_file
(InputOutput/ASCII.cpp:239-332): a banner with the time, then one line per
particle, fields separated by ',' and vector components by ' ', numbers with
16 significant digits (the precision the reference uses on devices with
64-bit addresses).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _lib
from .case import Case, Params

# the reference's types of the Variables a particles file may hold
# (basic.xml / cfd.xml Variable declarations)
VARIABLE_TYPES = {
    "r": "vec", "normal": "vec", "tangent": "vec", "binormal": "vec",
    "u": "vec", "dudt": "vec", "rho": "float", "drhodt": "float",
    "m": "float", "p": "float", "shepard": "float", "imove": "int",
    "iset": "unsigned int", "id": "unsigned int",
}
_COLUMN = {"vec": _lib.AQUA_COLUMN_FLOAT, "float": _lib.AQUA_COLUMN_FLOAT,
           "int": _lib.AQUA_COLUMN_INT, "unsigned int": _lib.AQUA_COLUMN_UINT}
_DTYPE = {"vec": np.float32, "float": np.float32, "int": np.int32,
          "unsigned int": np.uint32}


class ParticlesFileError(RuntimeError):
    pass


def _parse_fields(fields) -> list:
    if isinstance(fields, str):
        fields = fields.split(",")
    return [f.strip() for f in fields if f.strip()]


def _ncomp(kind: str, dims: int) -> int:
    return (4 if dims == 3 else 2) if kind == "vec" else 1


def count_particles(path: str) -> int:
    """Particle lines of a file (ASCII::readNParticles)."""
    lib = _lib.load()
    n = C.c_uint64(0)
    st = lib.aqua_read_fastascii(os.fsencode(path), 0, None, None, 0,
                                 C.byref(n), None)
    if st == _lib.AQUA_ERR_IO:
        raise ParticlesFileError(f"Failure reading the file \"{path}\".")
    _lib.check("aqua_read_fastascii", st)
    return int(n.value)


def load_fastascii(path: str, fields, dims: int, n: int = None,
                   types: dict = None) -> dict:
    """Reads a FastASCII file: returns {field: array} with vec fields shaped
    (n, 2|4).  ``n`` (the set's declared particle count) must match the
    file when given; ``types`` declares extra Variables ({name: "vec" |
    "float" | "int" | "unsigned int"}), as a case's XML may.  Errors as the
    reference's loader raises them: no fields, "r" missing, an undeclared
    field, a count mismatch, a malformed line (with its number)."""
    known = dict(VARIABLE_TYPES, **(types or {}))
    fields = _parse_fields(fields)
    if not fields:
        raise ParticlesFileError("0 fields were set to be read from the file.")
    if "r" not in fields:
        raise ParticlesFileError('"r" field was not set to be read from the file.')
    for f in fields:
        if f not in known:
            raise ParticlesFileError(f'Undeclared variable "{f}" set to be read.')
    kinds = [known[f] for f in fields]
    cols = []
    for k in kinds:
        cols += [_COLUMN[k]] * _ncomp(k, dims)
    found = count_particles(path)
    if n is not None and n != found:
        raise ParticlesFileError(
            f"Expected {n} particles, but the file contains just {found} ones.")
    lib = _lib.load()
    col_types = np.asarray(cols, np.int32)
    words = np.zeros((found, len(cols)), np.uint32)
    rows = C.c_uint64(0)
    bad = C.c_uint64(0)
    st = lib.aqua_read_fastascii(
        os.fsencode(path), len(cols), col_types.ctypes.data_as(_lib._I),
        words.ctypes.data_as(C.c_void_p), found, C.byref(rows), C.byref(bad))
    if st == _lib.AQUA_ERR_FORMAT:
        raise ParticlesFileError(
            f"Line {bad.value} of \"{path}\" does not hold {len(cols)} valid "
            f"numbers for the fields {', '.join(fields)}.")
    if st == _lib.AQUA_ERR_IO:
        raise ParticlesFileError(f"Failure reading the file \"{path}\".")
    _lib.check("aqua_read_fastascii", st)
    out = {}
    c = 0
    for f, k in zip(fields, kinds):
        nc = _ncomp(k, dims)
        block = np.ascontiguousarray(words[:, c:c + nc]).view(_DTYPE[k])
        out[f] = block if k == "vec" else block[:, 0].copy()
        c += nc
    return out


def _fmt(v, kind: str) -> str:
    if kind in ("int", "unsigned int"):
        return str(int(v))
    return format(float(v), ".16g")


def _fmt_t(t) -> str:
    return format(float(np.float32(t)), "g")


BANNER = """#########################################################
#                                                       #
#    #    ##   #  #   #                           #     #
#   # #  #  #  #  #  # #                          #     #
#  ##### #  #  #  # #####  ##  ###  #  #  ## ###  ###   #
#  #   # #  #  #  # #   # #  # #  # #  # #   #  # #  #  #
#  #   # #  #  #  # #   # #  # #  # #  #   # #  # #  #  #
#  #   #  ## #  ##  #   #  ### ###   ### ##  ###  #  #  #
#                            # #             #          #
#                          ##  #             #          #
#                                                       #
#########################################################
"""


def write_fastascii(path: str, arrays: dict, fields, dims: int, t: float = 0.0):
    """Writes particles as ASCII::print_file does: the banner with the time,
    an empty line, then per particle the fields separated by ',' and the
    components of a vec by ' '."""
    fields = _parse_fields(fields)
    kinds = [VARIABLE_TYPES[f] for f in fields]
    cols = []
    for f, k in zip(fields, kinds):
        a = np.asarray(arrays[f])
        if k == "vec":
            a = a.reshape(len(a), -1)[:, :_ncomp(k, dims)]
        cols.append((a, k))
    n = len(cols[0][0])
    with open(path, "w") as fh:
        fh.write(BANNER)
        fh.write("#\n#    File autogenerated by AQUAgpusph\n")
        fh.write(f"#    t = {_fmt_t(t)} s\n#\n")
        fh.write("#########################################################\n\n")
        for i in range(n):
            parts = []
            for a, k in cols:
                if k == "vec":
                    parts.append(" ".join(_fmt(v, k) for v in a[i]))
                else:
                    parts.append(_fmt(a[i], k))
            fh.write(",".join(parts) + "\n")


def case_from_files(params: Params, sets) -> Case:
    """A :class:`Case` from particle sets, each ``(path, fields, n)`` (n may
    be None): set k's particles get iset = k and consecutive ids, as the
    reference's loaders do (InputOutput/Particles.cpp:122-190, loadDefault);
    fields a file does not hold keep their defaults (zero, imove = 1)."""
    loaded = []
    for path, fields, n in sets:
        loaded.append(load_fastascii(path, fields, params.dims, n))
    total = sum(len(d["r"]) for d in loaded)
    c = Case(params, total)
    o = 0
    for k, d in enumerate(loaded):
        m = len(d["r"])
        c.iset[o:o + m] = k
        for f, a in d.items():
            if f in ("id", "iset"):
                continue
            getattr(c, f)[o:o + m] = a
        o += m
    return c
