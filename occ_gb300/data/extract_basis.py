"""Extract the basis sets this package's workloads use into occ_gb300/data/basis.

Basis-set data are inputs to the XC build (OCC passes an AOBasis in); the
values are the Basis Set Exchange data that OCC ships as share/basis/*.json.
Only the elements the workloads need (H, C, N, O) are kept, in the same
schema (electron_shells -> angular_momentum, exponents, coefficients, with
numbers left as the original decimal strings so that parsing them gives the
same doubles).

usage: python extract_basis.py <dir with BSE json files>
"""
import json
import os
import sys

NAMES = ["sto-3g", "3-21g", "6-31g", "6-31g(d,p)", "def2-svp", "def2-tzvp"]
ELEMENTS = ["1", "6", "7", "8"]


def main(src):
    out_dir = os.path.join(os.path.dirname(os.path.abspath(__file__)), "basis")
    os.makedirs(out_dir, exist_ok=True)
    for name in NAMES:
        with open(os.path.join(src, name + ".json")) as f:
            d = json.load(f)
        elems = {}
        for z in ELEMENTS:
            if z not in d["elements"]:
                continue
            shells = []
            for s in d["elements"][z]["electron_shells"]:
                shells.append({"angular_momentum": s["angular_momentum"],
                               "exponents": s["exponents"],
                               "coefficients": s["coefficients"]})
            elems[z] = {"electron_shells": shells}
        with open(os.path.join(out_dir, name + ".json"), "w") as f:
            json.dump({"name": d.get("name", name), "elements": elems}, f, separators=(",", ":"))


if __name__ == "__main__":
    main(sys.argv[1])
