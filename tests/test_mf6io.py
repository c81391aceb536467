"""The binary head-file reader and writer (modflow6_gb300.mf6io) on a file
that MODFLOW 6 wrote: autotest/data/ex-gwf-bump/results.hds.cmp, committed as
tests/golden/ex_gwf_bump_results.hds (tests/golden/make_bump_fixture.py)."""
from pathlib import Path

import numpy as np
import pytest

from modflow6_gb300 import mf6io

GOLDEN = Path(__file__).resolve().parent / "golden"


def test_read_mf6_head_file():
    recs = mf6io.read_dependent_variable(GOLDEN / "ex_gwf_bump_results.hds")
    assert len(recs) == 1
    r = recs[0]
    assert (r.kstp, r.kper, r.pertim, r.totim, r.text, r.ncol, r.nrow, r.ilay) == \
        (1, 1, 1.0, 1.0, "HEAD", 51, 51, 1)
    f = np.load(GOLDEN / "ex_gwf_bump.npz")
    np.testing.assert_array_equal(r.data, f["heads"])
    hd = mf6io.read_heads(GOLDEN / "ex_gwf_bump_results.hds")
    assert list(hd) == [(1, 1)] and hd[(1, 1)].shape == (1, 51, 51)


def test_write_reproduces_mf6_bytes(tmp_path):
    """Writing the same record gives MODFLOW 6's bytes exactly."""
    f = np.load(GOLDEN / "ex_gwf_bump.npz")
    out = tmp_path / "h.hds"
    mf6io.write_dependent_variable(out, f["heads"], 1, 51, 51, kstp=1, kper=1, pertim=1.0, totim=1.0)
    assert out.read_bytes() == (GOLDEN / "ex_gwf_bump_results.hds").read_bytes()


def test_multi_layer_multi_step_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    nlay, nrow, ncol = 3, 4, 5
    out = tmp_path / "m.hds"
    steps = {}
    for i, (kper, kstp) in enumerate([(1, 1), (1, 2), (2, 1)]):
        h = rng.standard_normal(nlay * nrow * ncol)
        steps[(kper, kstp)] = h
        mf6io.write_dependent_variable(out, h, nlay, nrow, ncol, kstp=kstp, kper=kper,
                                       pertim=0.5 * (i + 1), totim=float(i + 1), append=i > 0)
    hd = mf6io.read_heads(out)
    assert list(hd) == list(steps)
    for k, h in steps.items():
        np.testing.assert_array_equal(hd[k].ravel(), h)
    recs = mf6io.read_dependent_variable(out)
    assert [r.ilay for r in recs] == [1, 2, 3] * 3


def test_truncated_file_is_rejected():
    b = (GOLDEN / "ex_gwf_bump_results.hds").read_bytes()
    with pytest.raises(ValueError):
        mf6io.read_dependent_variable(b[:-8])
    with pytest.raises(ValueError):
        mf6io.read_dependent_variable(b[:30])
