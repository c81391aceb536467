"""Runs the oracle on the full 500x500x5 convertible NEWTON workload for its
first stress period (10 steps of TSMULT 1.2 over 10 d; BiCGSTAB + ILU0 and
DBD under-relaxation, modflow6_gb300/workloads.py C3_*), and records per
time step the outer and inner iteration counts and the model budget's
percent discrepancy, and at the end of the period the heads on a fixed
sample of cells: every WEL cell and 100,000 cells drawn without replacement
(numpy default_rng(2025)), stored with their node numbers so the test does
not depend on numpy's sampler.

Output: tests/golden/c3_oracle_period1.json and c3_oracle_period1_heads.npz.
Usage: python tests/golden/make_c3_reference.py [--seed 0]
"""
import argparse
import json
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

import oracle  # noqa: E402
from modflow6_gb300.dis import make_config  # noqa: E402
from modflow6_gb300.workloads import C3_IMS, C3_OUTER, C3_PERIOD, step_lengths  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--scale", type=float, default=1.0)
    a = ap.parse_args()
    m = make_config("c3", seed=a.seed, scale=a.scale)
    g = oracle.Gwf(m, oracle.settings(**C3_IMS))
    steps = []
    t_all = time.perf_counter()
    for kstp, delt in enumerate(step_lengths(C3_PERIOD["perlen"], C3_PERIOD["nstp"],
                                             C3_PERIOD["tsmult"]), start=1):
        hold = g.x.copy()
        t0 = time.perf_counter()
        st = g.timestep(kper=1, kstp=kstp, delt=delt, transient=True, **C3_OUTER)
        dt = time.perf_counter() - t0
        _, bud = g.budget(g.x, hold=hold, delt=delt, transient=True)
        steps.append(dict(kstp=kstp, delt=delt, outer=st["outer"], inner=st["inner_total"],
                          converged=st["converged"], seconds=dt,
                          percent_discrepancy=bud["percent_discrepancy"]))
        print(json.dumps(steps[-1]), flush=True)
    rnd = np.random.default_rng(2025).choice(m.nodes, size=min(100_000, m.nodes), replace=False)
    cells = np.unique(np.concatenate([m.wel_node, rnd])).astype(np.int32)
    out = dict(workload=f"c3 seed={a.seed} scale={a.scale}, stress period 1", nodes=m.nodes,
               ims=C3_IMS, outer=C3_OUTER, period=C3_PERIOD, steps=steps,
               oracle_seconds=time.perf_counter() - t_all, head_checksum=float(g.x.sum()),
               head_min=float(g.x.min()), head_max=float(g.x.max()))
    suffix = "" if a.scale == 1.0 else f"_scale{a.scale}"
    here = Path(__file__).parent
    (here / f"c3_oracle_period1{suffix}.json").write_text(json.dumps(out, indent=1))
    np.savez_compressed(here / f"c3_oracle_period1_heads{suffix}.npz", cells=cells, heads=g.x[cells])


if __name__ == "__main__":
    main()
