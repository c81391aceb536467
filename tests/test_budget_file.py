"""MODFLOW 6 budget files (OC BUDGET FILEOUT): the record layout of
ubdsv1/ubdsv06/ubdsvd (src/Utilities/InputOutput.f90:945-1072) checked byte
for byte on a hand-built record, the reader against the writer, and, on the
GPU, a time step's budget file against the device's flows and budget."""
import struct

import numpy as np
import pytest

from modflow6_gb300.mf6io import BudgetRecord, gwf_budget_records, read_budget, write_budget


def test_budget_record_bytes(tmp_path):
    """imeth 1: the 36-byte identification (kstp, kper, text, ncol, nrow,
    -nlay), the 28-byte imeth/delt/pertim/totim record, the values; imeth 6:
    the same, four 16-byte names, naux+1, nlist and (node, node2, q)."""
    r1 = BudgetRecord(2, 3, "FLOW-JA-FACE", 2, 1, 1, 1, 0.5, 1.5, 4.5, data=np.array([1.25, -2.0]))
    r6 = BudgetRecord(2, 3, "WEL", 5, 4, 3, 6, 0.5, 1.5, 4.5, names=("GWF", "GWF", "GWF", "WEL"),
                      node=np.array([17]), node2=np.array([1]), q=np.array([-3.0]))
    p = tmp_path / "t.cbc"
    write_budget(p, [r1, r6])
    want = (struct.pack("<ii16siii", 2, 3, b"    FLOW-JA-FACE", 2, 1, -1)
            + struct.pack("<iddd", 1, 0.5, 1.5, 4.5) + struct.pack("<dd", 1.25, -2.0)
            + struct.pack("<ii16siii", 2, 3, b"             WEL", 5, 4, -3)
            + struct.pack("<iddd", 6, 0.5, 1.5, 4.5)
            + b"GWF".ljust(16) * 3 + b"WEL".ljust(16)
            + struct.pack("<ii", 1, 1) + struct.pack("<iid", 17, 1, -3.0))
    assert p.read_bytes() == want


def test_budget_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    recs = [BudgetRecord(1, 1, "STO-SS", 4, 3, 2, 1, 1.0, 1.0, 1.0, data=rng.random(24)),
            BudgetRecord(1, 1, "FLOW-JA-FACE", 60, 1, 1, 1, 1.0, 1.0, 1.0, data=rng.random(60)),
            BudgetRecord(1, 1, "RCH", 4, 3, 2, 6, 1.0, 1.0, 1.0, names=("M", "M", "M", "RCH"),
                         auxnames=("CONC",), node=np.arange(1, 5), node2=np.arange(1, 5),
                         q=rng.random(4), aux=rng.random((4, 1)))]
    p = tmp_path / "r.cbc"
    write_budget(p, recs)
    back = read_budget(p)
    assert [r.text for r in back] == ["STO-SS", "FLOW-JA-FACE", "RCH"]
    for a, b in zip(recs, back):
        assert (a.kstp, a.kper, a.ndim1, a.ndim2, a.ndim3, a.imeth) == \
               (b.kstp, b.kper, b.ndim1, b.ndim2, b.ndim3, b.imeth)
        if a.imeth == 1:
            np.testing.assert_array_equal(a.data, b.data)
        else:
            assert b.names == a.names and b.auxnames == a.auxnames
            np.testing.assert_array_equal(a.q, b.q)
            np.testing.assert_array_equal(a.aux, b.aux)


@pytest.mark.gpu
@pytest.mark.parametrize("name,scale", [("c3", 0.04), ("c5", 0.1)])
def test_gpu_budget_file_matches_the_device_budget(gblib, tmp_path, name, scale):
    """One transient time step saved as a budget file: FLOW-JA-FACE is the
    device's, the per-cell and per-entry rates add up to the model budget's
    entries, and each CHD entry's rate is minus its cell's face flows."""
    from modflow6_gb300.dis import make_config
    from modflow6_gb300.ims import ImsLinearSettings
    from modflow6_gb300.solution import GwfSolution, Nonlinear
    m = make_config(name, seed=4, scale=scale)
    sol = GwfSolution(m, ImsLinearSettings(dvclose=1e-8, rclose=1e-6, iter1=2000, ilinmeth=2),
                      Nonlinear(dvclose=1e-6, mxiter=60))
    st = sol.timestep(1, 1, 2.0)
    assert st["converged"] == 1
    path = tmp_path / "m.cbc"
    sol.save_budget(path, name="gwf", delt=2.0, pertim=2.0, totim=2.0)
    recs = {r.text: r for r in read_budget(path)}
    want = ["STO-SS"] + (["STO-SY"] if (m.icelltype != 0).any() else []) + ["FLOW-JA-FACE"]
    want += [k for k, v in (("CHD", m.chd_node), ("WEL", m.wel_node), ("RCH", m.rch_node)) if len(v)]
    assert list(recs) == want
    fj, bud = sol.budget(flowja=True)
    np.testing.assert_array_equal(recs["FLOW-JA-FACE"].data, fj)
    entries = {"STO-SS": recs["STO-SS"].data}
    if "STO-SY" in recs:
        entries["STO-SY"] = recs["STO-SY"].data
    for k in ("CHD", "WEL", "RCH"):
        if k in recs:
            entries[k] = recs[k].q
    for i, k in enumerate(sol.BUDGET_ENTRIES):
        if k not in entries:
            continue
        v = entries[k]
        scale_k = max(1.0, float(np.abs(v).sum()))
        assert abs(v[v > 0].sum() - bud["rate_in"][i]) <= 1e-11 * scale_k, k
        assert abs(-v[v < 0].sum() - bud["rate_out"][i]) <= 1e-11 * scale_k, k
    if "CHD" in recs:
        chd = recs["CHD"]
        ia = m.connections()["ia"]
        rows = chd.node - 1
        face = np.array([fj[ia[r] + 1:ia[r + 1]].sum() for r in rows])
        np.testing.assert_allclose(chd.q, -face, rtol=1e-12, atol=1e-12 * np.abs(face).max())
        assert (chd.node2 == np.arange(1, len(chd.q) + 1)).all()
    assert recs["WEL"].names == ("GWF", "GWF", "GWF", "WEL")
