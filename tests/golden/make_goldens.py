"""Generate the golden fixtures used by the parity tests.

Reads (as text; nothing is executed) the reference's golden tables in
testing/testing.py:69-153 and examples/test_examples.py:63-153 of a
VALENCE checkout, and copies the matching input files next to this script,
so that the tests never need the reference tree at run time.

usage: python tests/golden/make_goldens.py /path/to/VALENCE
"""
import json
import os
import re
import shutil
import sys

PAT = re.compile(
    r"vsvb_output\(\s*([-0-9.eE+]+)\s*,\s*([-0-9.eE+]+)\s*,\s*(True|False)\s*,\s*([-0-9.eE+]+)\s*,\s*\"([^\"]+)\"\s*\)",
    re.S)


def parse(path):
    text = open(path).read()
    out = []
    for m in PAT.finditer(text):
        out.append(dict(nuclear_repulsion=float(m.group(1)), guess_energy=float(m.group(2)),
                        converged=m.group(3) == "True", total_energy=float(m.group(4)),
                        name=m.group(5)))
    return out


def main(ref):
    here = os.path.dirname(os.path.abspath(__file__))
    cases = []
    for suite, table, indir in (("testing", "testing/testing.py", "testing/test_cases"),
                                ("examples", "examples/test_examples.py", "examples")):
        dst = os.path.join(here, "cases", suite)
        os.makedirs(dst, exist_ok=True)
        for g in parse(os.path.join(ref, table)):
            src = os.path.join(ref, indir, g["name"])
            if not os.path.exists(src):
                continue
            shutil.copyfile(src, os.path.join(dst, g["name"]))
            g["suite"] = suite
            g["input"] = f"cases/{suite}/{g['name']}"
            g["source"] = f"{table} ({indir}/{g['name']})"
            cases.append(g)
    with open(os.path.join(here, "reference_goldens.json"), "w") as f:
        json.dump({"tolerances": {"nuclear_repulsion": 1e-10, "guess_energy": 1e-8,
                                  "total_energy": 1e-6,
                                  "source": "testing/testing.py:22-24"},
                   "cases": cases}, f, indent=1)
    print(f"{len(cases)} golden cases")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_goldens.py <path of the VALENCE source tree>")
    main(sys.argv[1])
