"""Case set-up: compiled Definitions and the synthetic workloads."""
import numpy as np

from aquagpusph_gb300 import case as cases


def test_define_float_is_six_significant_digits():
    # CalcServer.cpp:247-257 formats evaluated Definitions with "%#G"
    assert cases.define_float(0.01) == np.float32(0.01)
    assert cases.define_float(1.0 / 0.02 ** 2) == np.float32(2500.0)
    assert cases.define_float(1.0 / 0.01 ** 5) == np.float32(1.0e10)
    assert cases.define_float(1.0 / 3.0) == np.float32(0.333333)
    assert cases.define_float(3) == np.float32(3.0)


def test_dam_break_2d_counts():
    c = cases.dam_break_2d()
    assert c.n_fluid == 7200
    assert int((c.imove == cases.SENSOR).sum()) == 1
    assert int((c.imove == cases.WALL).sum()) == 2 * 322 + 2 * 180
    # hydrostatic density through the linear EOS
    fl = c.imove == 1
    p = c.params.cs ** 2 * (c.rho[fl] - 998.0)
    assert np.allclose(p, c.p[fl], rtol=1e-3, atol=5.0)


def test_dam_break_3d_counts():
    c = cases.dam_break_3d(dx=0.02, tank=(0.5, 0.24, 0.4), block=(0.2, 0.24, 0.16),
                           probes_z=(0.02,))
    assert c.n_fluid == 10 * 12 * 8
    w = c.imove == cases.WALL
    assert np.allclose(np.linalg.norm(c.normal[w, :3], axis=1), 1.0)
    assert np.all(c.m[w] == np.float32(0.02 ** 2))


def test_config1_size():
    """The benchmark workload: 246x200x110 fluid + 466,400 wall elements
    + 4 probes."""
    nx, ny, nz = (int(round(v / 0.005)) for v in (1.228, 1.0, 0.55))
    NX, NY, NZ = (int(round(v / 0.005)) for v in (3.22, 1.0, 1.0))
    walls = NX * NY + 2 * NY * NZ + 2 * NX * NZ
    assert nx * ny * nz == 5_412_000 and walls == 466_400


def test_fixed_time_step():
    c = cases.dam_break_2d()
    assert np.isclose(c.params.dt_fixed, 0.1 * 0.02 / 45.0, rtol=1e-6)
