"""Generates the golden fixtures of tests/golden/ (run where the reference
tree is mounted; the fixtures are committed so that hosts without it, the
GPU host included, can check against them).

    python tests/golden/make_golden.py [/path/to/reference]

* linklist_{2d,3d}.npz -- the reference's LinkList test input
  (tests/{2D,3D}/LinkList/cMake/particles.dat, loaded twice as two particle
  sets of 500, h = 0.1, support = 2, as tests/*/LinkList/cMake/main.xml
  does) and the link-list the reference's own iCell/iHoc/linkList kernels
  give on it (oracle/_ref harness): icell, id_sorted, id_unsorted, ihoc,
  n_cells, r_min, r_max.
* radixsort_3d.npz -- the keys of tests/3D/RadixSort/cMake/particles.dat
  (5th column) and their stable sort: sorted keys, perm, inv_perm.
* step_{2d,3d}.npz -- a small perturbed dam break (every particle type, a
  NaN and an out-of-domain particle, random velocities and rates) and the
  Variables after one (out1_*) and two (out2_*) canonical steps of the
  reference-kernel harness.
* step_bi_{2d,3d}.npz -- the same kind of case with BI walls (cfd/BI.xml in
  place of cfd/BIe.xml) and the Variables after one, two and five steps
  (out1_*, out2_*, out5_*) of the harness.
* step_ie_{2d,3d}.npz -- BI walls with the improved Euler scheme
  (basic/time_scheme/improved_euler.xml in place of the midpoint scheme, as
  in the reference's BI examples), after one, two and five steps.
* history_3d.npz -- the probe-pressure history of the CPU oracle (the
  restatement the reference kernels pin) over a small 3-D dam break (0.6 x
  0.2 x 0.4 m tank, 0.2 m water cube, dx = 0.01 m, 15,602 particles) from
  rest through the impact on the far wall, to t = 0.3 s (6,001 steps):
  the oracle takes minutes for it, so the GPU test reads it from here.

    python tests/golden/make_golden.py [/path/to/reference] [bi|ie|history]

regenerates everything, or only the BI, improved-Euler or history fixtures.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from aquagpusph_gb300 import case as cases  # noqa: E402
import oracle as O  # noqa: E402
sys.path.insert(0, HERE)
from golden_cases import perturbed, small_case  # noqa: E402

STATE_KEYS = ("id", "iset", "imove", "r", "normal", "tangent", "binormal",
              "u", "dudt", "rho", "drhodt", "m", "p")


def read_columns(path):
    rows = []
    with open(path) as f:
        for line in f:
            line = line.replace(",", " ").strip()
            if line:
                rows.append([float(x) for x in line.split()])
    return np.array(rows)


def linklist_case(dims, pos):
    vs = 4 if dims == 3 else 2
    p = cases.Params(dims=dims, h=0.1, cs=1.0, g=(0, 0, 0, 0),
                     refd=(1.0, 1.0), visc_dyn=(0.0, 0.0), delta=(0.0, 0.0),
                     domain_min=(-10, -10, -10, 0), domain_max=(10, 10, 10, 0))
    n = 2 * len(pos)
    c = cases.Case(p, n)
    c.r[:, :] = 0
    c.r[: len(pos), :dims] = pos[:, :dims]
    c.r[len(pos):, :dims] = pos[:, :dims]
    c.iset[len(pos):] = 1
    return c


def make_linklist(ref_root):
    out = {}
    for dims in (2, 3):
        pos = read_columns(os.path.join(ref_root, "tests", f"{dims}D", "LinkList",
                                        "cMake", "particles.dat"))
        c = linklist_case(dims, pos.astype(np.float32))
        lib = O.load_ref(dims)
        st = O.OracleState(c, ihoc_capacity=1 << 16)
        st.arrays["r_in"][...] = c.r
        lib.linklist(st)
        out[dims] = dict(r=c.r, h=np.float32(0.1), support=np.float32(2.0),
                         icell=st["icell"], id_sorted=st["id_sorted"],
                         id_unsorted=st["id_unsorted"], ihoc=st["ihoc"],
                         n_cells=st["n_cells"], r_min=st["r_min"],
                         r_max=st["r_max"])
        np.savez_compressed(os.path.join(HERE, f"linklist_{dims}d.npz"),
                            **out[dims])
    return out


def make_radixsort(ref_root):
    data = read_columns(os.path.join(ref_root, "tests", "3D", "RadixSort",
                                     "cMake", "particles.dat"))
    keys = data[:, 4].astype(np.uint32)
    k, perm, inv = O.load_ref(3).sort(keys)
    np.savez_compressed(os.path.join(HERE, "radixsort_3d.npz"), keys=keys,
                        sorted=k, perm=perm, inv_perm=inv)


def make_steps():
    for dims in (2, 3):
        c = perturbed(small_case(dims), 11 + dims)
        st = O.OracleState(c)
        data = {"in_" + k: getattr(c, k) for k in STATE_KEYS}
        data.update({"in_t": np.float32(c.t), "in_dt": np.float32(c.dt),
                     "in_iter": np.uint32(c.iter)})
        lib = O.load_ref(dims)
        for step in (1, 2):
            lib.step(st)
            for k, a in st.arrays.items():
                data[f"out{step}_" + k] = (st[k] if k == "ihoc" else a).copy()
            for k in ("n_cells", "r_min", "r_max", "t", "dt", "iter"):
                data[f"out{step}_" + k] = np.asarray(st[k])
        np.savez_compressed(os.path.join(HERE, f"step_{dims}d.npz"), **data)


def make_steps_bi(scheme=0):
    import dataclasses
    for dims in (2, 3):
        c = perturbed(small_case(dims), (31 if scheme else 21) + dims)
        c.params = dataclasses.replace(c.params, boundary=1, scheme=scheme)
        c.u[c.imove == 1] *= 0.25   # gentler flow near the walls
        st = O.OracleState(c)
        data = {"in_" + k: getattr(c, k) for k in STATE_KEYS}
        data.update({"in_t": np.float32(c.t), "in_dt": np.float32(c.dt),
                     "in_iter": np.uint32(c.iter)})
        lib = O.load_ref(dims)
        for step in (1, 2, 3, 4, 5):
            lib.step(st)
            if step not in (1, 2, 5):
                continue
            for k, a in st.arrays.items():
                data[f"out{step}_" + k] = (st[k] if k == "ihoc" else a).copy()
            for k in ("n_cells", "r_min", "r_max", "t", "dt", "iter"):
                data[f"out{step}_" + k] = np.asarray(st[k])
        name = "step_ie" if scheme else "step_bi"
        np.savez_compressed(os.path.join(HERE, f"{name}_{dims}d.npz"), **data)


def history_case_3d():
    c = cases.dam_break_3d(dx=0.01, tank=(0.6, 0.2, 0.4), block=(0.2, 0.2, 0.2),
                           probes_z=(0.02, 0.06))
    c.dt = c.params.dt_fixed
    return c


HISTORY_T_END = 0.3


def make_history_3d():
    c = history_case_3d()
    first = c.N - 2
    orc = O.load_oracle()
    st = O.OracleState(c)
    ts, ps = [], []
    while st["t"] < HISTORY_T_END:
        orc.step(st)
        ts.append(st["t"])
        ps.append(O.probe_values(st, "p", first, 2))
    np.savez_compressed(os.path.join(HERE, "history_3d.npz"),
                        t=np.array(ts, np.float64), p=np.array(ps, np.float32),
                        n=np.int64(c.N), first=np.int64(first))


def main():
    ref_root = sys.argv[1] if len(sys.argv) > 1 else O.reference_dir()
    if not ref_root:
        sys.exit("usage: make_golden.py REFERENCE_TREE (or set AQUA_REFERENCE_DIR)")
    os.environ["AQUA_REFERENCE_DIR"] = ref_root
    O.build_oracle(ref=True)
    if len(sys.argv) > 2 and sys.argv[2] in ("bi", "ie"):
        make_steps_bi(1 if sys.argv[2] == "ie" else 0)
        return
    if len(sys.argv) > 2 and sys.argv[2] == "history":
        make_history_3d()
        return
    make_linklist(ref_root)
    make_radixsort(ref_root)
    make_steps()
    make_steps_bi()
    make_steps_bi(scheme=1)
    make_history_3d()
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
