"""Extract the reference's golden vectors into golden_byte.json.

Reads the GOLDEN table and the CASES list from the reference's
tests/golden.rs (lines 68-74 and 141-147) as text and writes them as JSON.
Run where a checkout of the reference is present, giving its golden.rs:

    python tests/golden/extract_golden.py <reference checkout>/tests/golden.rs
"""
import json
import os
import re
import sys


def main(path):
    src = open(path).read()
    cases = []
    for m in re.finditer(
            r'Case \{ name: "([^"]+)",\s*w: (\d+), h: (\d+),\s*rest: (true|false),\s*inlet: (\d+),'
            r' plate: (true|false),\s*threads: (\d+), steps: (\d+) \}', src):
        cases.append(dict(name=m.group(1), w=int(m.group(2)), h=int(m.group(3)),
                          rest=m.group(4) == "true", inlet=int(m.group(5)),
                          plate=m.group(6) == "true", threads=int(m.group(7)),
                          steps=int(m.group(8))))
    golden = {}
    for m in re.finditer(r'\("([^"]+)", (0x[0-9a-f]+), (0x[0-9a-f]+), (-?\d+), (-?\d+), (-?\d+),'
                         r' (-?[0-9.]+), (-?[0-9.]+)\)', src):
        golden[m.group(1)] = dict(cells=m.group(2), field=m.group(3), mass=int(m.group(4)),
                                  px=int(m.group(5)), py=int(m.group(6)),
                                  ux=float(m.group(7)), uy=float(m.group(8)))
    consts = {}
    for name in ("DENSITY", "SPEED", "SEED", "BLOCK"):
        m = re.search(r'const %s: \w+ = ([0-9A-Fa-fx.]+);' % name, src)
        consts[name] = m.group(1)
    out = dict(source="tests/golden.rs:49-52,68-74,141-147 of daleobrien/lattice-gas",
               constants=consts, cases=cases, golden=golden)
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden_byte.json")
    with open(dst, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", dst, len(cases), "cases")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: extract_golden.py <path to the reference's tests/golden.rs>")
    main(sys.argv[1])
