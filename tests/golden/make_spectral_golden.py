"""Regenerate tests/golden/spectral_npol4.json from the reference's own table.

Reads the nPol = 4 arrays (pgll_4, pglj_4, wgll_4, wglj_4, Ggll_4, Gglj_4) out of the
reference source text SOLVER/src/preloop/spectral/SpectralConstants.cpp and writes
them as JSON.  Run in a checkout that has the reference next to it:

    python tests/golden/make_spectral_golden.py /path/to/AxiSEM3D
"""
import json
import re
import sys
from pathlib import Path

if len(sys.argv) != 2:
    sys.exit("usage: make_spectral_golden.py <path of the AxiSEM3D checkout>")
ref = Path(sys.argv[1])
src = (ref / "SOLVER/src/preloop/spectral/SpectralConstants.cpp").read_text()
out = {}
for name in ("pgll_4", "pglj_4", "wgll_4", "wglj_4", "Ggll_4", "Gglj_4"):
    m = re.search(r"double\s+%s\[\]\s*=\s*\{([^}]*)\}" % name, src)
    out[name] = [float(v) for v in m.group(1).split(",")]
out["source"] = "SOLVER/src/preloop/spectral/SpectralConstants.cpp:40-46 (row-major Map<RDMatPP>)"
dst = Path(__file__).with_name("spectral_npol4.json")
dst.write_text(json.dumps(out, indent=1))
print(dst)
