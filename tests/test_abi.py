"""The C ABI library builds for sm_103a, loads, and exports every function
include/aqua_gb300.h declares (no GPU needed: nothing is called)."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "aqua_gb300.h")
LEARNED_HEADER = os.path.join(ROOT, "include", "aqua_learned.h")


def declared_functions(header=HEADER):
    text = open(header).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[\w*]+\s+\**(aqua_\w+)\s*\(",
                                 text, flags=re.M)))


@pytest.fixture(scope="module")
def lib_path():
    from aquagpusph_gb300 import build
    return build.build()


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("aqua_create", "aqua_destroy", "aqua_set_state",
                 "aqua_get_state", "aqua_step", "aqua_linklist",
                 "aqua_radix_sort", "aqua_check"):
        assert must in names


def test_library_exports_every_declared_symbol(lib_path):
    lib = ctypes.CDLL(lib_path)
    for name in declared_functions():
        assert hasattr(lib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", lib_path],
                         capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (aqua_\w+)", out))
    assert set(declared_functions()) <= exported


def test_binding_covers_header(lib_path):
    from aquagpusph_gb300 import _lib
    bound = {name for name, _, _ in _lib.SIGNATURES}
    assert bound == set(declared_functions())


def test_structs_match_between_oracle_and_library():
    import oracle as O
    from aquagpusph_gb300 import _lib
    # the library's aqua_params is the leading part of the oracle's aq_params
    # (the oracle adds the per-case roll fields that the library keeps in
    # aqua_case)
    lib_fields = [f[0] for f in _lib.AquaParams._fields_]
    assert [f[0] for f in O.AqParams._fields_][: len(lib_fields)] == lib_fields
    for name in lib_fields:
        assert getattr(O.AqParams, name).offset == getattr(_lib.AquaParams, name).offset


def test_learned_header_exported_and_bound(lib_path):
    from aquagpusph_gb300 import learned
    names = declared_functions(LEARNED_HEADER)
    assert len(names) >= 20
    lib = ctypes.CDLL(lib_path)
    for name in names:
        assert hasattr(lib, name), name
    assert set(learned.SIGNATURES) == set(names)
