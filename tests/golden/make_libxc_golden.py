"""Extracts libxc 6.2.2's own golden vectors for the two functionals on the
hot path (LDA_X, id 1, and LDA_C_PW, id 12; energy "zk" and potential
"vrho") from the reference tree's vendored testsuite:
  ExLib/libxc/libxc-6.2.2/testsuite/input/{H,Li,BrOH,BrOH+}
  ExLib/libxc/libxc-6.2.2/testsuite/regression/{lda_x,lda_c}/*.{unpol,pol}.{0,1}.bz2
Unpolarised densities are rhoa + rhob, as testsuite/xc-regression.c:258-262;
polarised ones keep (rhoa, rhob) and vrho has one column per spin.
Writes tests/golden/libxc_lda_unpol.json and libxc_lda_pol.json:
  python tests/golden/make_libxc_golden.py <DEReK tree>   (or DEREK_REFERENCE=...)
"""
import bz2
import json
import os
import sys

ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("DEREK_REFERENCE")
if not ref or not os.path.isdir(os.path.join(ref, "ExLib/libxc/libxc-6.2.2/testsuite")):
    sys.exit("usage: make_libxc_golden.py <DEReK tree> (or set DEREK_REFERENCE); "
             f"no libxc 6.2.2 testsuite under {ref!r}")
base = os.path.join(ref, "ExLib/libxc/libxc-6.2.2/testsuite")
for spin in ("unpol", "pol"):
    out = {"source": "libxc 6.2.2 testsuite (vendored in the DEReK tree, ExLib/libxc)", "systems": {}}
    for sysname in ("H", "Li", "BrOH", "BrOH+"):
        with open(os.path.join(base, "input", sysname)) as f:
            lines = f.read().split("\n")
        n = int(lines[0])
        rows = [[float(x) for x in line.split()] for line in lines[1:n + 1]]
        if spin == "unpol":
            entry = {"rho": [c[0] + c[1] for c in rows]}
        else:
            entry = {"rhoa": [c[0] for c in rows], "rhob": [c[1] for c in rows]}
        for fam, func, key in (("lda_x", "lda_x", "x"), ("lda_c", "lda_c_pw", "c")):
            for order, name in ((0, "zk"), (1, "vrho")):
                path = os.path.join(base, "regression", fam, f"{func}.{sysname}.{spin}.{order}.bz2")
                with bz2.open(path, "rt") as f:
                    txt = f.read().split("\n")
                vals = [[float(x) for x in line.split()] for line in txt[2:] if line.strip()]
                if spin == "unpol" or order == 0:
                    entry[f"{name}_{key}"] = [v[0] for v in vals]
                else:
                    entry[f"{name}_{key}"] = vals
        out["systems"][sysname] = entry
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), f"libxc_lda_{spin}.json")
    with open(dst, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", dst)
