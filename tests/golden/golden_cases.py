"""Small cases shared by the golden-fixture generator and the tests."""
import numpy as np

from aquagpusph_gb300 import case as cases


def perturbed(c, seed):
    """Random velocities, rates and position jitter on the fluid, one NaN
    and one out-of-domain particle, and dt = the fixed time step: a state
    that reaches the Domain, elastic-bounce and PST branches."""
    rng = np.random.default_rng(seed)
    c = c.copy()
    d = c.dims
    fl = np.flatnonzero(c.imove == 1)
    dx = c.params.h / 2
    c.u[fl, :d] = rng.normal(0, 2.0, (len(fl), d))
    c.r[fl, :d] += (rng.uniform(-0.2, 0.2, (len(fl), d)) * dx).astype(np.float32)
    c.dudt[fl, :d] = rng.normal(0, 5.0, (len(fl), d))
    c.drhodt[fl] = rng.normal(0, 50.0, len(fl))
    c.r[fl[0], 0] = np.nan
    c.r[fl[1], 0] = c.params.domain_max[0] + 1.0
    c.dt = np.float32(c.params.dt_fixed)
    return c


def small_case(dims):
    """A dam break of a few hundred (2-D) or a few thousand (3-D) particles."""
    if dims == 2:
        return cases.dam_break_2d(dx=0.02, tank=(1.0, 0.6), column=(0.4, 0.3),
                                  probe_y=0.1)
    return cases.dam_break_3d(dx=0.02, tank=(0.5, 0.24, 0.4),
                              block=(0.2, 0.24, 0.16), probes_z=(0.02, 0.06))
