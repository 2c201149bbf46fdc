"""Generate the diatomic golden fixtures in this directory from the HelFEM
reference tree (run once in a container that has the reference checked out):

    python tests/golden/make_diatomic_golden.py /path/to/HelFEM

Writes diatomic.json with
  legendre   Maple reference values of P_l^m(x) and Q_l^m(x) for x > 1 (the
             prolate spheroidal range), l <= 12 and l in {16,20,26,32,40},
             m <= 8, read from
             src/legendre/legendre_reference_data.h;
  scf        converged diatomic HF and DFT (pure-m XC grid) energies recorded
             by the reference's own test harness (tests/refs/ci.json) with
             the run arguments (tests/cases.json).
Only numbers and run arguments are extracted; no reference source is copied.
"""
from __future__ import annotations

import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
KEEP = {"diatomic-H2-hf-r", "diatomic-H2-hf-u", "diatomic-He-dummy-hf", "diatomic-Ne-dummy-hf",
        "diatomic-H2-purem-on", "diatomic-Ne-dummy-lda", "diatomic-Ne-dummy-gga", "diatomic-NH-lda-u",
        "diatomic-NH-lda-absm"}


def find(obj, key):
    if isinstance(obj, dict):
        if key in obj:
            return obj[key]
        for v in obj.values():
            r = find(v, key)
            if r is not None:
                return r
    return None


def main(root):
    leg = []
    pat = re.compile(r'\{\s*(\d+),\s*(\d+),\s*"([^"]+)",\s*"([^"]+)",\s*"([^"]+)"\}')
    with open(os.path.join(root, "src", "legendre", "legendre_reference_data.h")) as f:
        for line in f:
            m = pat.search(line)
            if not m:
                continue
            l, mm, x, P, Q = int(m.group(1)), int(m.group(2)), m.group(3), m.group(4), m.group(5)
            if float(x) > 1.0 and (l <= 12 or l in (16, 20, 26, 32, 40)) and mm <= 8:
                leg.append({"l": l, "m": mm, "x": x, "P": P, "Q": Q})
    cases = json.load(open(os.path.join(root, "tests", "cases.json")))["cases"]
    refs = json.load(open(os.path.join(root, "tests", "refs", "ci.json")))
    scf = []
    for c in cases:
        if c["name"] not in KEEP:
            continue
        r = find(refs, c["name"])
        args = {}
        for a in c["args"]:
            k, v = a.lstrip("-").split("=", 1)
            args[k] = v
        scf.append({"name": c["name"], "args": args,
                    "ref": {k: r[k] for k in ("total", "kinetic", "nuclear", "Coulomb", "Exx", "XC", "Enucr") if k in r}})
    out = {"legendre": leg, "scf": scf}
    with open(os.path.join(HERE, "diatomic.json"), "w") as f:
        json.dump(out, f, indent=0)
    print(len(leg), "legendre values,", len(scf), "scf cases")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {os.path.basename(__file__)} <path of the HelFEM source tree>")
    main(sys.argv[1])
