"""Generates tests/golden/cube_example.json from the reference's only example
mesh (examples/cube_example.stl of ceschmiedel/CFD_, 12 triangles).

The file is a binary STL whose triangle count sits at byte 79 instead of 80
(a 79-byte header), which the reference's size rule 84 + 50 n accepts with a
one-byte shift.  Run with the reference checked out next to the repo:
    python tests/golden/make_cube.py /path/to/reference
"""
import json
import os
import struct
import sys


def main(ref_root):
    data = open(os.path.join(ref_root, "examples", "cube_example.stl"), "rb").read()
    for hdr in (80, 79):
        n = struct.unpack_from("<I", data, hdr)[0]
        if hdr + 4 + 50 * n == len(data) and n > 0:
            break
    else:
        raise SystemExit("not a binary STL")
    verts, idx = [], []
    for t in range(n):
        off = hdr + 4 + 50 * t + 12          # skip the facet normal
        for k in range(3):
            verts.append(list(struct.unpack_from("<3f", data, off + 12 * k)))
        idx.append([3 * t, 3 * t + 1, 3 * t + 2])
    out = {"source": "examples/cube_example.stl", "header_bytes": hdr, "n_triangles": n,
           "positions": verts, "indices": idx}
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "cube_example.json")
    with open(dst, "w") as f:
        json.dump(out, f)
    print("wrote", dst, n, "triangles")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} REFERENCE_CHECKOUT")
    main(sys.argv[1])
