"""The host runtime (libaqua_host.so) and the installable step tool
(libaqua_cuda_tool.so) on the CPU: both libraries build and export their
entry points, the loader reports the failures the reference's CalcServer
reports when it loads an installable tool (CalcServer.cpp:375-398: library
not found, no create_object symbol), and the tool's setup stops on a missing
or short Variable before any device call."""
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "aqua_host.h")


def declared(header=HEADER):
    text = re.sub(r"/\*.*?\*/", "", open(header).read(), flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[\w*]+\s+\**(aqua_\w+)\s*\(",
                                 text, flags=re.M)))


def exported(path):
    out = subprocess.run(["nm", "-D", "--defined-only", path],
                         capture_output=True, text=True).stdout
    return set(re.findall(r" T (\w+)", out))


@pytest.fixture(scope="module")
def rt():
    from aquagpusph_gb300 import build, host
    build.build()
    r = host.HostRuntime()
    r.clear()
    yield r
    r.clear()


def test_libraries_export_their_entry_points(rt):
    from aquagpusph_gb300 import host
    names = declared()
    assert "aqua_host_add_installable" in names
    assert set(names) <= exported(host.HOST_LIB)
    assert "create_object" in exported(host.TOOL_LIB)


def test_binding_covers_header():
    from aquagpusph_gb300 import host
    assert {n for n, _, _ in host._SIGS} == set(declared())


def test_missing_library_is_reported(rt):
    from aquagpusph_gb300 import host
    with pytest.raises(host.HostError, match="failed loading"):
        rt.add_installable("nothing", os.path.join(ROOT, "no_such_tool.so"))
    assert rt.tool_count() == 0


def test_library_without_factory_is_reported(rt):
    from aquagpusph_gb300 import host
    with pytest.raises(host.HostError, match="create_object"):
        rt.add_installable("not a tool", host.HOST_LIB)
    assert rt.tool_count() == 0


def small_case():
    from aquagpusph_gb300 import case as cases
    return cases.dam_break_2d(dx=0.05)


def test_setup_needs_every_variable(rt):
    from aquagpusph_gb300 import host
    rt.clear()
    rt.add_installable("aqua cuda step")
    assert rt.tool_count() == 1
    with pytest.raises(host.HostError, match="unregistered Variable"):
        rt.setup()
    # a whole case but one Definition
    rt.clear()
    rt.set_case(small_case())
    full = rt.variables()
    rt.clear()
    rt.add_installable("aqua cuda step")
    for name, (vt, a) in full.items():
        if name != "__DR_FACTOR__":
            rt.set_variable(name, vt, a)
    with pytest.raises(host.HostError, match="__DR_FACTOR__"):
        rt.setup()
    rt.clear()


def test_setup_rejects_a_short_variable(rt):
    from aquagpusph_gb300 import host
    rt.clear()
    rt.set_case(small_case())
    rt.set_variable("g", "vec", np.zeros(1, np.float32))  # 4 bytes: too few
    rt.add_installable("aqua cuda step")
    with pytest.raises(host.HostError, match="\"g\" holds 4 bytes"):
        rt.setup()
    rt.clear()


def test_link_list_tool_is_built_by_name(rt):
    """create_object("link-list...") builds the link-list tool: it needs r_in
    and its outputs, not the step's Variables."""
    from aquagpusph_gb300 import host
    rt.clear()
    rt.add_installable("link-list")
    assert rt.tool_count() == 1
    with pytest.raises(host.HostError, match="unregistered Variable"):
        rt.setup()
    rt.clear()
