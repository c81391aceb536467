"""The MODFLOW 6 input writer (modflow6_gb300.mf6input): every keyword it
writes is one the reference's input definition files accept in that block
(tests/golden/mf6_dfn_index.json, from doc/mf6io/mf6ivar/dfn/*.dfn by
tests/golden/make_mf6_dfn_index.py), and the arrays and boundary lists read
back bit for bit."""
import json
from pathlib import Path

import numpy as np
import pytest

from modflow6_gb300.dis import make_config
from modflow6_gb300.ims import ImsLinearSettings
from modflow6_gb300.mf6input import read_array, read_blocks, write_simulation
from modflow6_gb300.solution import Nonlinear
from test_oracle_known_answers import bump_model

INDEX = json.loads((Path(__file__).parent / "golden" / "mf6_dfn_index.json").read_text())
DFN_OF = {"sim": "sim-nam", "tdis": "sim-tdis", "ims": "sln-ims", "nam": "gwf-nam",
          "dis": "gwf-dis", "ic": "gwf-ic", "npf": "gwf-npf", "sto": "gwf-sto", "chd": "gwf-chd",
          "wel": "gwf-wel", "rch": "gwf-rch", "oc": "gwf-oc"}
# blocks whose lines start with a keyword of the block (the others hold data rows)
KEYWORD_BLOCKS = {"options", "nonlinear", "linear", "dimensions", "griddata", "timing"}


def check_keywords(files):
    for key, path in files.items():
        idx = INDEX[DFN_OF[key]]
        for block, _, lines in read_blocks(path):
            assert block in idx, (key, block)
            if block not in KEYWORD_BLOCKS:
                continue
            for line in lines:
                w = line.split()[0].lower()
                if w in ("internal", "constant") or not w[0].isalpha():
                    continue  # array control records and values
                assert w in idx[block], (key, block, w)
        if key == "ims":
            lin = dict((b, ls) for b, _, ls in read_blocks(path))["linear"]
            assert any(l.upper().startswith("INNER_RCLOSE") for l in lin)


def test_bump_model_files(tmp_path):
    m, _ = bump_model()
    ims = ImsLinearSettings(dvclose=1e-9, rclose=1e-3, iter1=100, ilinmeth=2)
    nl = Nonlinear(dvclose=1e-8, mxiter=75, nonmeth=0, iallowptc=0)
    files = write_simulation(tmp_path, m, ims, nl, name="nr_ur01")
    check_keywords(files)
    blocks = {b: ls for b, _, ls in read_blocks(files["dis"])}
    np.testing.assert_array_equal(read_array(blocks["griddata"], "DELR"), m.delr)
    np.testing.assert_array_equal(read_array(blocks["griddata"], "BOTM"), m.botm)
    np.testing.assert_array_equal(read_array(blocks["griddata"], "TOP"), m.top)
    npf = {b: ls for b, _, ls in read_blocks(files["npf"])}
    np.testing.assert_array_equal(read_array(npf["griddata"], "K"), m.k11)
    np.testing.assert_array_equal(read_array(npf["griddata"], "ICELLTYPE"), m.icelltype)
    nam = {b: ls for b, _, ls in read_blocks(files["nam"])}
    assert nam["options"] == ["NEWTON UNDER_RELAXATION"]
    ims_b = {b: ls for b, _, ls in read_blocks(files["ims"])}
    assert "NO_PTC ALL" in ims_b["options"]
    assert "LINEAR_ACCELERATION BICGSTAB" in ims_b["linear"]
    # CHD rows: 1-based (layer, row, column) and the head, in the model's order
    rows = [b for b in read_blocks(files["chd"]) if b[0] == "period"][0][2]
    assert len(rows) == m.chd_node.size
    for line, node, hd in zip(rows, m.chd_node, m.chd_head):
        k, i, j, h = line.split()
        assert (int(k) - 1) * m.nrow * m.ncol + (int(i) - 1) * m.ncol + int(j) - 1 == node
        assert float(h) == hd


@pytest.mark.parametrize("name", ["c1", "c3"])
def test_workload_files(tmp_path, name):
    m = make_config(name, seed=3, scale=0.05 if name == "c3" else 1.0)
    m.icellavg, m.ivarcv, m.idewatcv = (2, 1, 1) if name == "c3" else (0, 0, 0)
    ims = ImsLinearSettings.preset_config("COMPLEX", icnvgopt=3, iscl=2, iord=1)
    nl = Nonlinear.preset("COMPLEX")
    periods = [(10.0, 10, 1.2, False)] * 3 if name == "c3" else [(1.0, 1, 1.0, True)]
    files = write_simulation(tmp_path, m, ims, nl, periods=periods)
    check_keywords(files)
    if name == "c3":
        sto = read_blocks(files["sto"])
        assert [b[1] for b in sto if b[0] == "period"] == ["1", "2", "3"]
        npf = {b: ls for b, _, ls in read_blocks(files["npf"])}
        assert "ALTERNATIVE_CELL_AVERAGING AMT-LMK" in npf["options"]
        assert "VARIABLECV DEWATERED" in npf["options"]
        ic = {b: ls for b, _, ls in read_blocks(files["ic"])}
        np.testing.assert_array_equal(read_array(ic["griddata"], "STRT"), m.strt)
    ims_b = {b: ls for b, _, ls in read_blocks(files["ims"])}
    assert any(l.endswith("RELATIVE_RCLOSE") for l in ims_b["linear"])
    assert "REORDERING_METHOD RCM" in ims_b["linear"] and "SCALING_METHOD L2NORM" in ims_b["linear"]
    assert "UNDER_RELAXATION DBD" in ims_b["nonlinear"]


def test_unbalanced_block_is_rejected(tmp_path):
    p = tmp_path / "bad.ims"
    p.write_text("BEGIN options\n  NO_PTC ALL\nEND linear\n")
    with pytest.raises(ValueError):
        read_blocks(p)
