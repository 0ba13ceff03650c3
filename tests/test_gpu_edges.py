"""Edge cases of the step on the GPU against the CPU oracle, with the
default launch shape (the direct sweep) and a queued one:

* tiny cases -- one fluid particle; two fluid particles within the support;
  a fluid particle with a boundary element and a probe;
* every particle outside the domain (Domain.cl parks them all at
  domain_max as buffer particles, and the step goes on with no fluid);
* a cell holding more particles than the 16-bit queue entries of the
  queued sweep can address (11-bit offsets): the direct sweep steps it like
  the oracle, the queued variant reports AQUA_ERR_CAPACITY instead of
  reading past the cell.

The exact build is bit-exact with the oracle here but for the positions,
which pass through powf in the BIe PST (within 1e-6)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import oracle as O
from aquagpusph_gb300 import case as cases
from test_gpu_parity import compare_state

QUEUED = (1, 8)   # 64 threads, 128 queued 16-bit entries, 8 blocks per SM


@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    torch.cuda.set_device(0)
    return torch


def base_params(dims):
    if dims == 2:
        return cases.dam_break_2d(dx=0.05).params
    return cases.dam_break_3d(dx=0.05, tank=(0.6, 0.3, 0.4),
                              block=(0.2, 0.3, 0.2)).params


def build_case(dims, r, imove, normal=None, u=None):
    p = base_params(dims)
    n = len(r)
    c = cases.Case(p, n)
    vs = c.vs
    c.r[:, :dims] = np.asarray(r, np.float32)
    c.imove[:] = imove
    dx = p.h / 2.0
    for i in range(n):
        c.rho[i] = p.refd[0]
        if imove[i] == cases.WALL:
            c.m[i] = dx ** (dims - 1)
        elif imove[i] == 1:
            c.m[i] = dx ** dims * p.refd[0]
    if normal is not None:
        c.normal[:, :dims] = np.asarray(normal, np.float32)
    if u is not None:
        c.u[:, :dims] = np.asarray(u, np.float32)
    del vs
    c.dt = p.dt_fixed
    return c


def run_both(c, tuning, steps=3):
    from aquagpusph_gb300.solver import Solver
    sv = Solver(c.params, capacity=c.N)
    if tuning is not None:
        sv.set_tuning(*tuning)
    sv.set_case(c)
    st = O.OracleState(c)
    orc = O.load_oracle()
    for k in range(steps):
        sv.step(1, graph=False)
        sv.check()
        orc.step(st)
        compare_state(sv.get_case(), st, exact_floats=(k == 0))
    sv.close()


@pytest.mark.parametrize("tuning", [None, QUEUED])
@pytest.mark.parametrize("dims", [2, 3])
def test_tiny_cases_match_oracle(gpu, dims, tuning):
    mid = [0.3, 0.15, 0.1][:dims]
    h = base_params(dims).h
    one = build_case(dims, [mid], [1])
    run_both(one, tuning)
    two = build_case(dims, [mid, [mid[0] + 0.7 * h] + mid[1:]], [1, 1],
                     u=[[0.1] + [0.0] * (dims - 1), [-0.2] + [0.0] * (dims - 1)])
    run_both(two, tuning)
    # a fluid particle above a boundary element (outward normal -z / -y) and
    # a probe between them
    up = dims - 1
    wall = list(mid)
    wall[up] = mid[up] - 0.5 * h
    probe = list(mid)
    probe[up] = mid[up] - 0.25 * h
    nrm = [0.0] * dims
    nrm[up] = -1.0
    mixed = build_case(dims, [mid, wall, probe], [1, cases.WALL, 0],
                       normal=[[0.0] * dims, nrm, [0.0] * dims],
                       u=[[0.0] * (dims - 1) + [-0.5], [0.0] * dims,
                          [0.0] * dims])
    run_both(mixed, tuning)


@pytest.mark.parametrize("dims", [2, 3])
def test_all_particles_outside_the_domain(gpu, dims):
    p = base_params(dims)
    far = [p.domain_max[k] + 1.0 for k in range(dims)]
    c = build_case(dims, [far, far, far], [1, 1, cases.WALL])
    run_both(c, None, steps=2)


def crowded_case():
    """2,200 fluid particles packed inside one cell of a 2-D tank."""
    p = base_params(2)
    h = p.h
    side = 47                     # 47 x 47 = 2,209 particles
    s = 1.5 * h / side            # all inside a cell of edge 2h
    xs = 0.3 + s * np.arange(side)
    ys = 0.2 + s * np.arange(side)
    r = np.array([[x, y] for y in ys for x in xs], np.float32)
    c = build_case(2, r, np.ones(len(r), np.int32))
    c.m[:] = np.float32(s * s * p.refd[0])
    return c


def test_crowded_cell_direct_sweep_matches_oracle(gpu):
    run_both(crowded_case(), None, steps=1)


def test_crowded_cell_queued_sweep_reports_capacity(gpu):
    from aquagpusph_gb300 import _lib
    from aquagpusph_gb300.solver import Solver
    c = crowded_case()
    sv = Solver(c.params, capacity=c.N)
    sv.set_tuning(*QUEUED)
    sv.set_case(c)
    sv.step(1, graph=False)
    with pytest.raises(_lib.AquaError) as e:
        sv.check()
    assert e.value.status == _lib.AQUA_ERR_CAPACITY
    sv.close()
