"""Regenerates reference_vectors.json from the reference's own test files, read as text.

The reference (kshitijl/micrographia) is Rust and cannot be built or run here; its known-answer
vectors live in its sources. This script pulls them out verbatim:
  - Random123 Threefry-2x32 known answers (crates/gpu-prims/src/threefry.rs:53-63),
  - GOLDEN_INT_HASH and its setup (crates/md/src/checks.rs:155-167),
  - the separation/min-image test values of crates/md-core/src/fixed.rs:78-98.
Usage: python tests/golden/extract.py /path/to/reference
"""

import json
import os
import re
import sys


def main(ref):
    out = {}
    src = open(os.path.join(ref, "crates/gpu-prims/src/threefry.rs")).read()
    kat = []
    for m in re.finditer(r"\((\d+), \[(0x[0-9a-f]+), (0x[0-9a-f]+)\], \[(0x[0-9a-f]+), (0x[0-9a-f]+)\], \[(0x[0-9a-f]+), (0x[0-9a-f]+)\]\)", src):
        r, c0, c1, k0, k1, w0, w1 = m.groups()
        kat.append({"rounds": int(r), "ctr": [int(c0, 16), int(c1, 16)], "key": [int(k0, 16), int(k1, 16)], "want": [int(w0, 16), int(w1, 16)]})
    out["threefry_kat"] = kat
    chk = open(os.path.join(ref, "crates/md/src/checks.rs")).read()
    h = re.search(r"GOLDEN_INT_HASH: u64 = (0x[0-9a-f_]+);", chk).group(1).replace("_", "")
    out["golden_int_hash"] = h
    setup = re.search(r"pub fn golden_int_setup\(\)[^{]*\{(.*?)\n\}", chk, re.S).group(1)
    out["golden_int_setup_source"] = " ".join(setup.split())
    fx = open(os.path.join(ref, "crates/md-core/src/fixed.rs")).read()
    vals = re.search(r"for &d in &\[(.*?)\]", fx).group(1)
    out["sep_antisymmetry_values"] = [v.strip() for v in vals.split(",")]
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_vectors.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print(path)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/extract.py /path/to/reference")
    main(sys.argv[1])
