"""Launch shapes of the sweep (threads per block, queue depth, the direct
sweep without a queue, persistent blocks per SM) change only the schedule:
each particle's neighbours are still summed in the link-list order, so every
shape gives bit-identical state, with the exact and with the fast build.  The tuner picks one of them and the solver
keeps stepping correctly."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import oracle as O
from aquagpusph_gb300 import _lib
from aquagpusph_gb300 import case as cases


@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    torch.cuda.set_device(0)
    return torch


def three_d_case():
    from golden_cases import perturbed
    c = perturbed(cases.dam_break_3d(dx=0.01, tank=(0.6, 0.3, 0.4),
                                     block=(0.2, 0.3, 0.2), probes_z=(0.02,)), 43)
    c.dt = c.params.dt_fixed
    return c


def run(c, variant, blocks, steps=3, fast=False):
    from aquagpusph_gb300.solver import Solver
    sv = Solver(c.params, capacity=c.N)
    sv.set_precision(fast)
    sv.set_tuning(variant, blocks)
    sv.set_case(c)
    sv.step(steps, graph=True)
    sv.check()
    g = sv.get_case()
    sv.close()
    return g


SHAPES = [(0, 2), (0, 5), (1, 10), (2, 4), (3, 8), (4, 12), (5, 10), (5, 3),
          (6, 6), (7, 12), (7, 2), (8, 6), (9, 14), (10, 7), (11, 16),
          (12, 8), (13, 18), (14, 9)]


# the clustered sweep of the fast 3-D build: its own summation order, the
# same for every one of its shapes
SHAPES_CL = [(15, 2), (15, 1), (16, 3), (16, 1), (17, 2), (17, 1), (16, 7)]


@pytest.mark.parametrize("fast", [False, True])
def test_every_launch_shape_gives_identical_state(gpu, fast):
    c = three_d_case()
    groups = [SHAPES] + ([SHAPES_CL] if fast else [])
    for shapes in groups:
        base = run(c, *shapes[0], fast=fast)
        for v, b in shapes[1:]:
            g = run(c, v, b, fast=fast)
            for name, a in base.state_arrays().items():
                assert np.array_equal(getattr(g, name), a), (v, b, name)


def test_clustered_choice_falls_back_where_it_does_not_apply(gpu):
    """A clustered variant with the exact build runs the direct sweep: the
    state equals that of the direct sweep's default shape."""
    c = three_d_case()
    a = run(c, 16, 3, fast=False)
    b = run(c, 9, 14, fast=False)
    for name, x in b.state_arrays().items():
        assert np.array_equal(getattr(a, name), x), name


def test_tuned_shape_matches_oracle(gpu):
    from aquagpusph_gb300 import autotune
    from aquagpusph_gb300.solver import Solver
    c = three_d_case()
    sv = Solver(c.params, capacity=c.N)
    sv.set_precision(False)
    sv.set_case(c)
    choice = autotune.autotune(sv, fast=False, steps=1, use_cache=False)
    assert (choice["variant"], choice["blocks_per_sm"]) in set(autotune.candidates())
    assert len(choice["candidates"]) == len(list(autotune.candidates()))
    # the tuner advanced the state; restart from the case and compare one step
    sv.set_case(c)
    sv.step(1, graph=True)
    sv.check()
    g = sv.get_case()
    sv.close()
    st = O.OracleState(c)
    O.load_oracle().step(st)
    fl = st["imove"] == 1
    for name in ("dudt", "drhodt", "rho", "p"):
        assert np.array_equal(getattr(g, name)[fl], st[name][fl]), name


def test_invalid_tuning_is_rejected(gpu):
    from aquagpusph_gb300.solver import Solver
    c = three_d_case()
    sv = Solver(c.params, capacity=c.N)
    with pytest.raises(_lib.AquaError):
        sv.set_tuning(99, 4)
    with pytest.raises(_lib.AquaError):
        sv.set_tuning(18, 2)
    with pytest.raises(_lib.AquaError):
        sv.set_tuning(0, 0)
    sv.close()
