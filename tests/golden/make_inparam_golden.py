"""Regenerate tests/golden/inparam_template.json from the reference's own template parfiles.

Reads template/input/inparam.{model,nu,time_src_recv,advanced} of the reference checkout
and keeps their parameter entries (KEY followed by its values, in file order; comments
and blank lines dropped).  Run in a checkout that has the reference next to it:

    python tests/golden/make_inparam_golden.py /path/to/AxiSEM3D
"""
import json
import sys
from pathlib import Path

if len(sys.argv) != 2:
    sys.exit("usage: make_inparam_golden.py <path of the AxiSEM3D checkout>")
ref = Path(sys.argv[1]) / "template" / "input"
out = {"source": "template/input/inparam.* of the reference (parameter entries only)"}
for name in ("inparam.model", "inparam.nu", "inparam.time_src_recv", "inparam.advanced"):
    entries = []
    for line in (ref / name).read_text().splitlines():
        strs = line.strip().split()
        if strs and not strs[0].startswith("#"):
            entries.append([strs[0], strs[1:]])
    out[name] = entries
dst = Path(__file__).with_name("inparam_template.json")
dst.write_text(json.dumps(out, indent=0))
print(dst)
