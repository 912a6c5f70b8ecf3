"""Build the ex2 known-answer fixture from the reference's shipped example.

ex2 (Ti hcp, mode 3, 14 c/a values at V = 238 bohr^3) has a recorded SKOUT that
ends after the first structure's k-mesh header: SKIN is read with
blank='zero' (static.f:682), so the mesh line "12   12   12" under (5I5) gives
12000 divisions per axis, and kptgen.f stops when the full-zone mesh passes its
array bound (kptgen.f:141-145); SKENG is empty.  What SKOUT does record for
structure 1 -- the lattice from the (V, c/a) form, the Cartesian positions, the
minimum pair distance, the pair count, the secular size, the electron count,
the reciprocal vectors and metric, and the mesh divisions as read -- is the
fixture.  This script copies the inputs unchanged into tests/golden/ex2/ and
writes tests/golden/ex2_golden.json.

Run once, in a checkout that has the reference mounted:
    python tests/golden/make_ex2_fixture.py /path/to/reference/NRLtb/ex2
"""
import json
import os
import re
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def _floats(line):
    return [float(x.replace("D", "E")) for x in line.split()]


def main(src):
    dst = os.path.join(HERE, "ex2")
    os.makedirs(dst, exist_ok=True)
    for name in ["SKIN", "ti_par", "spcgp1.hcp"]:
        shutil.copyfile(os.path.join(src, name), os.path.join(dst, name))
    lines = open(os.path.join(src, "SKOUT")).read().splitlines()
    text = "\n".join(lines)
    plv = [_floats(re.search(r"PRIMITIVE LATTICE VECTOR NO\. %d(.*)" % i, text).group(1)) for i in (1, 2, 3)]
    i = next(j for j, ln in enumerate(lines) if "FINAL ATOMIC COORDINATES" in ln)
    cart = [_floats(lines[i + 1 + a])[3:6] for a in range(2)]
    frac = [_floats(lines[i + 1 + a])[0:3] for a in range(2)]
    i = next(j for j, ln in enumerate(lines) if "PRIMITIVE VECTORS OF THE RECIPROCAL LATTICE" in ln)
    recip = [_floats(lines[i + 2 + r]) for r in range(3)]
    i = next(j for j, ln in enumerate(lines) if "RECIPROCAL SPACE METRIC" in ln)
    metric = [_floats(lines[i + 2 + r]) for r in range(3)]
    kdiv = re.search(r"KDIV1,KDIV2,KDIV3=(.{15})", text).group(1)
    gold = {
        "source": "reference NRLtb/ex2 SKOUT, structure 1 (static v1.33, mode 3, Ti hcp, V=238, c/a=1.30)",
        "plv": plv,                                       # 6 decimals
        "volume": float(re.search(r"Volume=\s+(\S+)", text).group(1)),
        "cartesian": cart,                                # 7 decimals
        "fractional": frac,
        "dismin": float(re.search(r"Minimum distance this configuration =\s+(\S+)", text).group(1)),
        "npairs": int(re.search(r"Number of pairs =\s+(\d+)", text).group(1)),
        "nv": int(re.search(r"Secular equation size =\s+(\d+)", text).group(1)),
        "electrons": float(re.search(r"(\S+)\s+electrons in the calculation", text).group(1)),
        "recip": recip,                                   # 6 decimals
        "metric": metric,                                 # 8 significant digits
        "kdiv_as_read": [int(kdiv[5 * j:5 * j + 5]) for j in range(3)],
    }
    with open(os.path.join(HERE, "ex2_golden.json"), "w") as f:
        json.dump(gold, f, indent=1)
    print("wrote", dst, "and ex2_golden.json")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference/NRLtb/ex2")
