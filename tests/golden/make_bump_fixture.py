"""Writes tests/golden/ex_gwf_bump.npz from the reference's committed files.

The reference's autotest/test_gwf_newton_under_relaxation.py (lines 8-35,
106-119) checks MODFLOW 6 against a head file that MODFLOW 6 itself wrote,
autotest/data/ex-gwf-bump/results.hds.cmp, for a 51x51x1 convertible NEWTON
UNDER_RELAXATION model whose cell bottoms are autotest/data/ex-gwf-bump/
bottom.txt.  This script copies those two arrays, as they are, into one small
fixture (the reference tree is not present where the GPU tests run):

    bottom  (51, 51) float64   from bottom.txt
    heads   (51, 51) float64   the HEAD record of results.hds.cmp
    header  the record's kstp, kper, pertim, totim, ncol, nrow, ilay

Run from the repository root:  python tests/golden/make_bump_fixture.py
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from modflow6_gb300.mf6io import read_dependent_variable  # noqa: E402

DATA = Path("/root/reference/autotest/data/ex-gwf-bump")


def main():
    recs = read_dependent_variable(DATA / "results.hds.cmp")
    assert len(recs) == 1 and recs[0].text == "HEAD", recs
    r = recs[0]
    bottom = np.loadtxt(DATA / "bottom.txt").reshape(r.nrow, r.ncol)
    np.savez_compressed(Path(__file__).with_name("ex_gwf_bump.npz"), bottom=bottom, heads=r.data,
                        header=np.array([r.kstp, r.kper, r.pertim, r.totim, r.ncol, r.nrow, r.ilay]))
    # the raw head file too, so the reader is tested on MODFLOW 6's own bytes
    Path(__file__).with_name("ex_gwf_bump_results.hds").write_bytes(
        (DATA / "results.hds.cmp").read_bytes())


if __name__ == "__main__":
    main()
