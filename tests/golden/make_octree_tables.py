"""Extracts the octree neighbour lookup tables of the reference (pbosler/lpmKokkos,
src/LpmOctreeLUT.hpp:70-137: ParentLUT and ChildLUT, 8 x 27 each) into
octree_tables.json, the known answer the oracle's and the product's generated tables are
checked against.  Reads the reference source tree, so it runs where that tree is present.

Run:  python tests/golden/make_octree_tables.py <path-to-lpmKokkos-checkout>
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def table(text, name):
    m = re.search(r"struct\s+" + name + r"\s*\{.*?entries\[\d+\]\s*=\s*\{([^}]*)\}", text, re.S)
    vals = [int(v) for v in re.findall(r"-?\d+", m.group(1))]
    assert len(vals) == 216, (name, len(vals))
    return [vals[27 * i:27 * (i + 1)] for i in range(8)]


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: make_octree_tables.py <path-to-lpmKokkos-checkout>")
    ref = sys.argv[1]
    with open(os.path.join(ref, "src", "LpmOctreeLUT.hpp")) as f:
        text = f.read()
    out = {"source": "src/LpmOctreeLUT.hpp", "ParentLUT": table(text, "ParentLUT"), "ChildLUT": table(text, "ChildLUT")}
    with open(os.path.join(HERE, "octree_tables.json"), "w") as f:
        json.dump(out, f)
    print("wrote octree_tables.json")


if __name__ == "__main__":
    main()
