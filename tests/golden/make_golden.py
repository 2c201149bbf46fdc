"""Generate the golden fixtures in this directory from the HelFEM reference
tree (run once in a container that has the reference checked out):

    python tests/golden/make_golden.py /path/to/HelFEM

Writes
  ci_energies.json  converged atomic SCF energies recorded by the reference's
                    own test harness (tests/refs/ci.json) together with the
                    run arguments (tests/cases.json) and the Ne anchor from
                    tests/README.md;
  gaunt.json        Gaunt and modified-Gaunt values hard-coded in
                    src/general/gaunt_test.cpp.
Only numbers and run arguments are extracted; no reference source is copied.
"""
from __future__ import annotations

import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))

# atomic cases whose physics the oracle/product implement (HF, LDA VWN5,
# PBE; restricted and unrestricted; per-m fixed occupations)
KEEP = {
    "atomic-He-hf-r", "atomic-He-hf-u", "atomic-He-lda-r", "atomic-He-lda-u",
    "atomic-He-gga-r", "atomic-He-gga-u", "atomic-Be-hf-r", "atomic-Be-hf-u",
    "atomic-Be-lda-r", "atomic-Be-lda-u", "atomic-H-hf-u", "atomic-Be-nop-l0",
    "atomic-O-3P-p0-hf", "atomic-O-3P-pplus-hf", "atomic-O-3P-pminus-hf",
}


def parse_args(args):
    out = {}
    for a in args:
        k, v = a.lstrip("-").split("=", 1)
        out[k] = v
    return out


def main(ref_root: str):
    refs = json.load(open(os.path.join(ref_root, "tests/refs/ci.json")))["cases"]
    cases = {c["name"]: c for c in json.load(open(os.path.join(ref_root, "tests/cases.json")))["cases"]}
    out = []
    for name in sorted(KEEP):
        r, c = refs[name], cases[name]
        ent = {
            "name": name,
            "args": parse_args(c["args"]),
            "occs": c.get("input_files", {}).get("occs.dat"),
            "total": r["total"],
            "components": {k: r[k] for k in ("kinetic", "nuclear", "Coulomb", "Exx", "XC")},
            "source": "tests/refs/ci.json",
        }
        out.append(ent)
    readme = open(os.path.join(ref_root, "tests/README.md")).read()
    m = re.search(r"Ne\s+(-128\.\d+)", readme)
    out.append({
        "name": "atomic-Ne-hf-r",
        "args": parse_args(cases["atomic-Ne-hf-r"]["args"]),
        "occs": None,
        "total": float(m.group(1)),
        "components": None,
        "source": "tests/README.md",
    })
    json.dump(out, open(os.path.join(HERE, "ci_energies.json"), "w"), indent=1)

    src = open(os.path.join(ref_root, "src/general/gaunt_test.cpp")).read()
    pat = re.compile(r"val=helfem::gaunt::(gaunt_coefficient|modified_gaunt_coefficient)\(([-\d,]+)\);\s*ref=([-+.\deE]+);")
    g = [{"fn": "coeff" if f == "gaunt_coefficient" else "mod_coeff",
          "args": [int(x) for x in a.split(",")], "ref": float(v)} for f, a, v in pat.findall(src)]
    json.dump(g, open(os.path.join(HERE, "gaunt.json"), "w"))
    print(f"{len(out)} energies, {len(g)} Gaunt values")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {os.path.basename(__file__)} <path of the HelFEM source tree>")
    main(sys.argv[1])
