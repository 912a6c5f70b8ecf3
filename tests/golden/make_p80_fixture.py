"""Build the P80 known-answer fixture from the reference's shipped example.

P80 (carbon, 24-atom bcc cell, new-style overlap parameters, mode 9 with a
999 k path) has a recorded SKOUT that stops where the first atom line is
read: the SKIN file has a comment line there, "(Position of atom in Lattice
coordinates)", which list-directed input cannot read as an integer; SKENG
and QLMT are empty.  What SKOUT does record -- the mode, temperature and
cut-off, the parameter file as read (basis kind, spin state, overlap form,
cut-offs, all 97 parameters), the bcc lattice, the volume and the basis size
-- is the fixture.  This script copies the inputs unchanged into
tests/golden/P80/ and writes tests/golden/p80_golden.json.

Run once, in a checkout that has the reference mounted:
    python tests/golden/make_p80_fixture.py /path/to/reference/NRLtb/P80
"""
import json
import os
import re
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def main(src):
    dst = os.path.join(HERE, "P80")
    os.makedirs(dst, exist_ok=True)
    for name in ["SKIN", "C_par", "spcgrp.bcc"]:
        shutil.copyfile(os.path.join(src, name), os.path.join(dst, name))
    text = open(os.path.join(src, "SKOUT")).read()
    params = [float(v) for i, v in re.findall(r"^\s+(\d+)\s+(\S+E[+-]\d+)\s*$", text, re.M)]
    cut = re.search(r"Cutoff parameters:\s*\n\s*1\s+(\S+)\s+(\S+)", text)
    gold = {
        "source": "reference NRLtb/P80 SKOUT (static v1.33, mode 9, C 24-atom bcc)",
        "mode": int(re.search(r"mode=\s+(\d+)", text).group(1)),
        "tkb": float(re.search(r"temp\. broad\. \(ryd\):\s+(\S+)", text).group(1)),
        "eigcut": float(re.search(r"eigenvalue cutoff =\s+(\S+)", text).group(1)),
        "non_orthogonal": "Non-Orthogonal Basis Functions" in text,
        "spin_restricted": "Spin-restricted calculation" in text,
        "new_overlap": "Using S(l,lp,R) -> delta(l,lp) for like atoms" in text,
        "dnn": float(cut.group(1)),
        "screenl": float(cut.group(2)),
        "params": params,
        "plv": [[float(x) for x in re.search(r"PRIMITIVE LATTICE VECTOR NO\. %d(.*)" % i, text).group(1).split()]
                for i in (1, 2, 3)],
        "volume": float(re.search(r"Volume=\s+(\S+)", text).group(1)),
        "natoms": int(re.search(r"(\d+) TOTAL ATOMS", text).group(1)),
        "kbas": int(re.search(r"(\d+) BASIS FUNCTIONS ON ATOM KIND 1", text).group(1)),
    }
    assert len(params) == 97
    with open(os.path.join(HERE, "p80_golden.json"), "w") as f:
        json.dump(gold, f, indent=1)
    print("wrote", dst, "and p80_golden.json")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference/NRLtb/P80")
