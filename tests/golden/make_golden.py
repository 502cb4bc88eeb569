"""Regenerate tests/golden/hk_bases.json from the reference's basis files.

Reads the EOM-IMSRG inputs sp_inputs/hk<e>.sps (label n l 2j 2tz e) and the
"8 8" (16O) row of sp_inputs/hole_scheme_hk, and stores them as a small JSON
fixture so that the tests never need the reference tree at run time.
Usage:  python tests/golden/make_golden.py <path-to-EOM-IMSRG-checkout>
"""
import json
import os
import sys


def main(ref):
    sp = os.path.join(ref, "sp_inputs")
    out = {}
    for e in range(3, 15):
        rows = []
        with open(os.path.join(sp, f"hk{e}.sps")) as f:
            for line in f:
                p = line.split()
                if len(p) < 6:
                    continue
                rows.append([int(p[1]), int(p[2]), int(p[3]), int(p[4]), float(p[5])])
        out[f"hk{e}"] = rows
    with open(os.path.join(sp, "hole_scheme_hk")) as f:
        for line in f:
            p = line.split()
            if len(p) >= 2 and p[0] == "8" and p[1] == "8":
                out["hole_scheme_8_8"] = [int(x) for x in p[2:32]]
                break
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "hk_bases.json"), "w") as f:
        json.dump(out, f, separators=(",", ":"))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
