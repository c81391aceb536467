"""Writes tests/golden/mf6_dfn_index.json: for the input files that
modflow6_gb300.mf6input writes, the variable names MODFLOW 6 accepts in each
block, read from the reference's input definition files
(doc/mf6io/mf6ivar/dfn/<component>.dfn: "block <name>" / "name <variable>"
records).  The writer's test checks every keyword it writes against this
index.

Run from the repository root:  python tests/golden/make_mf6_dfn_index.py
"""
import json
from pathlib import Path

DFN = Path("/root/reference/doc/mf6io/mf6ivar/dfn")
FILES = ["sim-nam", "sim-tdis", "sln-ims", "gwf-nam", "gwf-dis", "gwf-ic", "gwf-npf", "gwf-sto",
         "gwf-chd", "gwf-wel", "gwf-rch", "gwf-oc"]


def parse(path):
    blocks = {}
    block = None
    for line in path.read_text().splitlines():
        w = line.split()
        if len(w) >= 2 and w[0] == "block":
            block = w[1]
        elif len(w) >= 2 and w[0] == "name" and block:
            blocks.setdefault(block, []).append(w[1])
    return {b: sorted(set(v)) for b, v in blocks.items()}


def main():
    out = {f: parse(DFN / f"{f}.dfn") for f in FILES}
    Path(__file__).with_name("mf6_dfn_index.json").write_text(json.dumps(out, indent=1, sort_keys=True))


if __name__ == "__main__":
    main()
