"""Writes the golden vectors of tests/golden/ from the reference's own test
sources, read as text (nothing of the reference is run):

- cubic_equation_kats.json: rs/src/no/uib/cipr/rs/util/test/CubicEquationTest.java,
  each `new CubicEquation(a0, a1, a2)` with the expected largest and smallest
  roots and the tolerance of its assertEquals calls.

Usage: python tests/golden/make_golden.py <reference checkout>
"""
import json
import os
import re
import sys


def cubic_kats(ref):
    path = os.path.join(ref, "rs/src/no/uib/cipr/rs/util/test/CubicEquationTest.java")
    text = open(path).read()
    kats = []
    for body in re.findall(r"public void test\w+\(\)\s*\{(.*?)\n    \}", text, re.S):
        coeffs = re.search(r"new CubicEquation\(([^)]*)\)", body)
        largest = re.search(r"assertEquals\(([^,]+),\s*eqn\.getLargestRoot\(\),\s*([^)]+)\)", body)
        smallest = re.search(r"assertEquals\(([^,]+),\s*eqn\.getSmallestRoot\(\),\s*([^)]+)\)", body)
        if not (coeffs and largest and smallest):
            continue
        kats.append({
            "coefficients": [float(v) for v in coeffs.group(1).split(",")],
            "largest": float(largest.group(1)), "smallest": float(smallest.group(1)),
            "tolerance": float(largest.group(2)),
        })
    return {"source": "rs/src/no/uib/cipr/rs/util/test/CubicEquationTest.java", "kats": kats}


def main():
    ref = sys.argv[1]
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "cubic_equation_kats.json"), "w") as f:
        json.dump(cubic_kats(ref), f, indent=1)
        f.write("\n")


if __name__ == "__main__":
    main()
