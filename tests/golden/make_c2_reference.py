"""Runs the CPU oracle's IMS (PCG + ILU0, FP64) on the full 1000x1000x10
steady-state workload to closure and records, per outer iteration, the inner
iteration count and the oracle's wall time, plus the oracle's time per inner
iteration.  Output: tests/golden/c2_oracle_reference.json, and the oracle's
converged heads on a fixed sample of cells in
tests/golden/c2_oracle_heads_sample.npz:

  * every WEL cell (the pumped cells carry the largest gradients);
  * every cell next to a CHD face (columns 2 and ncol-1 of every row and
    layer);
  * 100,000 further cells drawn without replacement (numpy default_rng(2024)).

`cells` (int32, sorted, 0-based node numbers) and `heads` (float64) are
stored side by side, so the test does not depend on numpy's sampler.

Usage: python tests/golden/make_c2_reference.py [--scale 1.0] [--seed 0]
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
from modflow6_gb300.workloads import C2_IMS, C2_OUTER  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--scale", type=float, default=1.0)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", default=str(Path(__file__).with_name("c2_oracle_reference.json")))
    a = ap.parse_args()
    t0 = time.perf_counter()
    m = make_config("c2", seed=a.seed, scale=a.scale)
    g = oracle.Gwf(m, oracle.settings(**C2_IMS))
    t_setup = time.perf_counter() - t0
    t1 = time.perf_counter()
    st = g.timestep(kper=1, kstp=1, delt=1.0, transient=False, **C2_OUTER)
    t_solve = time.perf_counter() - t1
    out = dict(workload=f"c2 scale={a.scale} seed={a.seed}", nodes=m.nodes, ims=C2_IMS,
               outer=C2_OUTER, stats=st, oracle_seconds=t_solve, setup_seconds=t_setup,
               head_checksum=float(np.sum(g.x)), head_min=float(g.x.min()), head_max=float(g.x.max()))
    Path(a.out).write_text(json.dumps(out, indent=1))
    nrc = m.nrow * m.ncol
    k, i = np.meshgrid(np.arange(m.nlay), np.arange(m.nrow), indexing="ij")
    beside_chd = np.concatenate([(k * nrc + i * m.ncol + 1).ravel(),
                                 (k * nrc + i * m.ncol + m.ncol - 2).ravel()])
    rnd = np.random.default_rng(2024).choice(m.nodes, size=min(100_000, m.nodes), replace=False)
    cells = np.unique(np.concatenate([m.wel_node, beside_chd, rnd])).astype(np.int32)
    np.savez_compressed(Path(a.out).with_name("c2_oracle_heads_sample.npz"), cells=cells,
                        heads=g.x[cells].astype(np.float64))
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
