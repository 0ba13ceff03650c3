"""Particle files (FastASCII reader and ASCII writer) and report formats, on
the CPU: the native reader of the library (no GPU call), the writers, the
reports' output rule, and the oracle's free-surface restatement."""
import os

import numpy as np
import pytest

import oracle as O
from aquagpusph_gb300 import particles_io as P
from aquagpusph_gb300 import reports as R

REF = O.reference_dir()


@pytest.fixture(scope="module")
def lib():
    from aquagpusph_gb300 import build
    build.build()
    from aquagpusph_gb300 import _lib
    return _lib.load()


@pytest.mark.skipif(REF is None or not os.path.isdir(os.path.join(REF, "tests")),
                    reason="reference tree not given (AQUA_REFERENCE_DIR)")
def test_reads_reference_fixtures_like_the_golden_inputs(lib):
    # the link-list and radix-sort tests' particles.dat (FastASCII), against
    # the arrays the golden fixtures were generated from
    for dims in (2, 3):
        a = P.load_fastascii(os.path.join(REF, f"tests/{dims}D/LinkList/cMake/"
                                               "particles.dat"), "r", dims)["r"]
        g = np.load(os.path.join(os.path.dirname(__file__), "golden",
                                 f"linklist_{dims}d.npz"))["r"]
        assert np.array_equal(a[:, :dims], g[: len(a), :dims])
    k = P.load_fastascii(os.path.join(REF, "tests/3D/RadixSort/cMake/particles.dat"),
                         "r, f", 3, types={"f": "unsigned int"})["f"]
    g = np.load(os.path.join(os.path.dirname(__file__), "golden",
                             "radixsort_3d.npz"))["keys"]
    assert np.array_equal(k, g)


@pytest.mark.parametrize("dims", [2, 3])
def test_write_then_read_is_exact(lib, tmp_path, dims):
    rng = np.random.default_rng(dims)
    n, vs = 257, (4 if dims == 3 else 2)
    arrays = {
        "r": rng.normal(size=(n, vs)).astype(np.float32) * 10,
        "normal": rng.normal(size=(n, vs)).astype(np.float32),
        "u": (rng.normal(size=(n, vs)) * 1e-7).astype(np.float32),
        "rho": rng.uniform(990, 1010, n).astype(np.float32),
        "m": rng.uniform(0, 1e-3, n).astype(np.float32),
        "imove": rng.integers(-3, 2, n).astype(np.int32),
        "iset": rng.integers(0, 5, n).astype(np.uint32),
    }
    fields = ["r", "normal", "u", "rho", "m", "imove", "iset"]
    path = str(tmp_path / "set.dat")
    P.write_fastascii(path, arrays, fields, dims, t=0.125)
    text = open(path).read()
    assert "#    t = 0.125 s" in text
    back = P.load_fastascii(path, ", ".join(fields), dims, n=n)
    for f in fields:
        assert back[f].dtype == arrays[f].dtype
        assert np.array_equal(back[f], arrays[f]), f


def test_line_rules(lib, tmp_path):
    path = tmp_path / "rules.dat"
    path.write_text(
        "# header comment\n"
        "\n"
        "  (1.5, 2.5)  ; [ -3 ]  {7}\t# trailing comment\n"
        ",,0.25 0.5,,,1,,2,\n"
        "   \t  \n"
        "1e-3,2E+1 -1 4294967295   \r\n")
    d = P.load_fastascii(str(path), "r, imove, iset", 2,
                         types=None)
    assert np.array_equal(d["r"], np.array([[1.5, 2.5], [0.25, 0.5],
                                            [1e-3, 20.0]], np.float32))
    assert np.array_equal(d["imove"], np.array([-3, 1, -1], np.int32))
    assert np.array_equal(d["iset"], np.array([7, 2, 4294967295], np.uint32))
    assert P.count_particles(str(path)) == 3


def test_number_prefix_and_unsigned_wrap(lib, tmp_path):
    # each column is parsed as a number prefix (std::sto* semantics): the
    # rest of the field is skipped; "-1" for an unsigned field wraps
    path = tmp_path / "prefix.dat"
    path.write_text("1.5x 2 3.9 -1\n")
    d = P.load_fastascii(str(path), "r, imove, iset", 2)
    assert np.array_equal(d["r"], np.array([[1.5, 2.0]], np.float32))
    assert d["imove"][0] == 3 and d["iset"][0] == 0xFFFFFFFF


@pytest.mark.parametrize("text,line", [
    ("1 2 1\n1 2\n", 2),            # too few fields
    ("1 2 1\n\n1 2 3 4\n", 3),      # too many
    ("1 abc 1\n", 1),               # no number
    ("1 1e39 1\n", 1),              # float out of range
    ("1 2 3000000000\n", 1),        # int out of range
])
def test_malformed_lines_name_the_line(lib, tmp_path, text, line):
    path = tmp_path / "bad.dat"
    path.write_text(text)
    with pytest.raises(P.ParticlesFileError, match=f"Line {line} "):
        P.load_fastascii(str(path), "r, imove", 2)


def test_loader_argument_errors(lib, tmp_path):
    path = tmp_path / "ok.dat"
    path.write_text("1 2\n3 4\n")
    with pytest.raises(P.ParticlesFileError, match="Expected 3 particles"):
        P.load_fastascii(str(path), "r", 2, n=3)
    with pytest.raises(P.ParticlesFileError, match='"r" field'):
        P.load_fastascii(str(path), "u", 2)
    with pytest.raises(P.ParticlesFileError, match="Undeclared"):
        P.load_fastascii(str(path), "r, foo", 2)
    with pytest.raises(P.ParticlesFileError, match="0 fields"):
        P.load_fastascii(str(path), "", 2)
    with pytest.raises(P.ParticlesFileError, match="Failure reading"):
        P.load_fastascii(str(tmp_path / "missing.dat"), "r", 2)


def test_case_from_files(lib, tmp_path):
    from aquagpusph_gb300 import case as cases
    c = cases.dam_break_2d(dx=0.05)
    fl = c.imove == cases.FLUID
    a = {k: getattr(c, k)[fl] for k in ("r", "normal", "u", "rho", "m", "imove")}
    b = {k: getattr(c, k)[~fl] for k in ("r", "normal", "u", "rho", "m", "imove")}
    fields = "r, normal, u, rho, m, imove"
    P.write_fastascii(str(tmp_path / "a.dat"), a, fields, 2)
    P.write_fastascii(str(tmp_path / "b.dat"), b, fields, 2)
    d = P.case_from_files(c.params, [(str(tmp_path / "a.dat"), fields, int(fl.sum())),
                                     (str(tmp_path / "b.dat"), fields, None)])
    assert d.N == c.N
    assert np.array_equal(d.id, np.arange(c.N))
    assert np.array_equal(d.iset, np.r_[np.zeros(fl.sum()), np.ones((~fl).sum())])
    assert np.array_equal(d.r, np.r_[a["r"], b["r"]])
    assert np.array_equal(d.imove, np.r_[a["imove"], b["imove"]])


def test_set_tab_file_format(tmp_path):
    path = str(tmp_path / "sensors.out")
    rep = R.SetTabFile(path, "p, shepard", first=7200, n=2, ipf=1)
    rep.write(np.float32(4.4444444e-05), {
        "p": np.array([1234.5, 0.0], np.float32),
        "shepard": np.array([0.5, 1.0], np.float32)})
    rep.close()
    lines = open(path).read().splitlines()
    assert lines[0] == "# Time p_7200 shepard_7200 p_7201 shepard_7201 "
    assert lines[1] == "4.44444e-05 1234.5 0.5 0 1 "
    t, cols = R.read_set_tab_file(path)
    assert cols["p_7200"][0] == 1234.5 and cols["shepard_7201"][0] == 1.0
    rep = R.SetTabFile(path, "u", first=0, n=1, ipf=1)
    rep.write(0.5, {"u": np.array([[0.1, -2.0]], np.float32)})
    rep.close()
    assert open(path).read().splitlines()[1] == \
        "0.5 (0.1000000014901161,-2) "


def test_tab_file_format(tmp_path):
    path = str(tmp_path / "h.out")
    rep = R.TabFile(path, "t, H1, H2")
    rep.write({"t": 0.001, "H1": 0.55, "H2": 0.0})
    rep.close()
    assert open(path).read() == "# t H1 H2 \n0.001 0.55 0 \n"


def test_report_output_rule():
    r = R.Report(ipf=3)
    fired = [it for it in range(1, 11) if r.must_update(it * 0.1, it)]
    assert fired == [1, 4, 7, 10]
    r = R.Report(fps=10.0)
    ts = np.float32(0.03) * np.arange(1, 20, dtype=np.float32)
    fired = [i for i, t in enumerate(ts, 1) if r.must_update(t, i)]
    # first output at once (last output time 0), then every >= 0.1 s
    assert fired[0] == 1
    gaps = np.diff([ts[i - 1] for i in fired])
    assert np.all(gaps >= np.float32(0.1) - 1e-7) and np.all(gaps < 0.13)


def test_oracle_free_surface_restatement():
    class St(dict):
        pass
    st = St()
    st["r"] = np.array([[0.0, 0.3], [0.015, 0.5], [0.05, 0.9], [0.0, 2.0],
                        [0.0, -1.0]], np.float32)
    st["imove"] = np.array([1, 1, 1, -3, 1], np.int32)
    h = O.free_surface(st, [0.0, 0.05, 10.0], dr=0.01, dims=2)
    # sensor 0: particles 0, 1 and 4 within 2 dr; 1 is highest
    assert h[0] == np.float32(0.5) + np.float32(0.5) * np.float32(0.01)
    # sensor 1: only particle 2 (x = 0.05)
    assert h[1] == np.float32(0.9) + np.float32(0.005)
    # sensor 2: nothing near -> every particle contributes 0
    assert h[2] == 0.0
