"""Extracts libxc 6.2.2's own golden vectors for the two functionals on the
hot path (LDA_X, id 1, and LDA_C_PW, id 12; spin-unpolarised; energy "zk"
and potential "vrho") from the reference tree's vendored testsuite:
  ExLib/libxc/libxc-6.2.2/testsuite/input/{H,Li,BrOH,BrOH+}
  ExLib/libxc/libxc-6.2.2/testsuite/regression/{lda_x,lda_c}/*.unpol.{0,1}.bz2
Unpolarised densities are rhoa + rhob, as testsuite/xc-regression.c:258-262.
Writes tests/golden/libxc_lda_unpol.json.  Run in a tree where the reference
is mounted: python tests/golden/make_libxc_golden.py [reference_root]
"""
import bz2
import json
import os
import sys

ref = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
base = os.path.join(ref, "ExLib/libxc/libxc-6.2.2/testsuite")
out = {"source": "libxc 6.2.2 testsuite (vendored in the DEReK tree, ExLib/libxc)", "systems": {}}
for sysname in ("H", "Li", "BrOH", "BrOH+"):
    with open(os.path.join(base, "input", sysname)) as f:
        lines = f.read().split("\n")
    n = int(lines[0])
    rho = []
    for line in lines[1:n + 1]:
        cols = [float(x) for x in line.split()]
        rho.append(cols[0] + cols[1])
    entry = {"rho": rho}
    for fam, func, key in (("lda_x", "lda_x", "x"), ("lda_c", "lda_c_pw", "c")):
        for order, name in ((0, "zk"), (1, "vrho")):
            path = os.path.join(base, "regression", fam, f"{func}.{sysname}.unpol.{order}.bz2")
            with bz2.open(path, "rt") as f:
                txt = f.read().split("\n")
            vals = [float(x) for x in txt[2:] if x.strip()]
            entry[f"{name}_{key}"] = vals
    out["systems"][sysname] = entry
dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libxc_lda_unpol.json")
with open(dst, "w") as f:
    json.dump(out, f, indent=1)
print("wrote", dst)
