"""Extract the reference's Morton byte tables (pkg/pt/morton.go:23-129, kept
there as a comment) into tests/golden/morton256.json.

These 3 x 256 entries are the only known-answer vectors the reference ships
for the LBVH path: morton256_x[b] is splitBy3(b), _y is that shifted by 1,
_z by 2.  Usage: python make_morton_tables.py <path to pkg/pt/morton.go of the
reference>; the committed JSON is what the tests read.
"""
import json
import os
import re
import sys

if len(sys.argv) != 2:
    sys.exit("usage: python make_morton_tables.py <path to the reference's pkg/pt/morton.go>")
SRC = sys.argv[1]
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "morton256.json")

text = open(SRC).read()
tables = {}
for axis in "xyz":
    m = re.search(r"morton256_%s\s*=\s*\[256\]uint64\{(.*?)\}" % axis, text, re.S)
    vals = [int(v, 16) for v in re.findall(r"0x[0-9a-fA-F]+", m.group(1))]
    assert len(vals) == 256, (axis, len(vals))
    tables[axis] = vals
json.dump({"source": "pkg/pt/morton.go:23-129", "tables": tables}, open(OUT, "w"))
print("wrote", OUT)
