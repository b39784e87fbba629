"""Regenerate the golden fixtures under tests/golden/ from the reference tree.

Runs only where the reference checkout exists (it is read, never copied):

    python tests/golden/make_golden.py /path/to/reference

Fixtures written:
  icosphere_off.json  -- sha256, byte length, header and a few sampled lines of
                         icosasphere3.off and icosasphere4.off, the only data
                         fixtures the reference ships; the mesh generator of the
                         library must reproduce these files byte for byte.
"""
import hashlib
import json
import os
import sys


def main(ref):
    out = {}
    for level in (3, 4):
        path = os.path.join(ref, "icosasphere%d.off" % level)
        data = open(path, "rb").read()
        lines = data.decode().splitlines()
        nv, nf, _ = (int(x) for x in lines[1].split())
        out[str(level)] = {
            "sha256": hashlib.sha256(data).hexdigest(),
            "bytes": len(data),
            "n_nodes": nv,
            "n_faces": nf,
            # a handful of lines, for a readable diff when the hash differs
            "samples": {str(i): lines[i] for i in (2, 13, 2 + nv - 1, 2 + nv, 2 + nv + nf - 1)},
        }
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "icosphere_off.json")
    with open(dst, "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print("wrote", dst)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <reference checkout>")
    main(sys.argv[1])
