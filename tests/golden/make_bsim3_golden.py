#!/usr/bin/env python3
"""Writes tests/golden/bsim3_dc.json from the reference's own BSIM3 golden
data (run from the repository root; the argument is a checkout of the
Spicier sources):

    python tests/golden/make_bsim3_golden.py <path to spicier>

The source is crates/spicier-parser/tests/golden_data/dc_bsim3.json
(ngspice-45 operating points of five BSIM3v3.3 netlists, with the tolerances
the reference's golden tests apply).  The netlists, results, device
quantities and tolerances are copied unchanged; nothing is computed here.
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: make_bsim3_golden.py <path to the Spicier sources>")
    path = os.path.join(sys.argv[1], "crates/spicier-parser/tests/golden_data/dc_bsim3.json")
    with open(path) as f:
        data = json.load(f)
    out = {"source": "crates/spicier-parser/tests/golden_data/dc_bsim3.json",
           "generator": data.get("generator"), "circuits": []}
    for c in data["circuits"]:
        a = c["analysis"]
        out["circuits"].append({"name": c["name"], "netlist": c["netlist"], "results": a.get("results", {}),
                                "reference": a.get("reference", {}), "tolerances": a.get("tolerances", {})})
    with open(os.path.join(HERE, "bsim3_dc.json"), "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")


if __name__ == "__main__":
    main()
