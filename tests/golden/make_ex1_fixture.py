"""Build the ex1 known-answer fixture from the reference's shipped example run.

The reference's only recorded outputs for this path are the ex1 Pd run: its
inputs (SKIN, the pd_par parameter file, the fcc.08 / bcc.08 k lists and the
space-group files SKIN names) and its outputs SKENG (9 decimals) and SKOUT (full
precision).  This script copies the inputs unchanged into tests/golden/ex1/ and
extracts the golden numbers into tests/golden/ex1_golden.json.

Run once, in a checkout that has the reference mounted:
    python tests/golden/make_ex1_fixture.py /path/to/reference/NRLtb/ex1
"""
import json
import os
import re
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def main(src):
    dst = os.path.join(HERE, "ex1")
    os.makedirs(dst, exist_ok=True)
    for name in ["SKIN", "pd_par", "fcc.08", "bcc.08", "spcgrp.fcc", "spcgrp.bcc"]:
        shutil.copyfile(os.path.join(src, name), os.path.join(dst, name))
    skout = open(os.path.join(src, "SKOUT")).read()
    grab = lambda pat, conv=float: [conv(x) for x in re.findall(pat, skout)]
    rows = [line.split() for line in open(os.path.join(src, "SKENG")) if line.strip()]
    gold = {
        "source": "reference NRLtb/ex1 SKENG and SKOUT (static v1.33, mode 4, kT=0.005, eigcut=0.5)",
        "labels": [" ".join(r[:2]) for r in rows],
        "skeng": [[float(x) for x in r[2:6]] for r in rows],   # volume, E_F, E(T), P(T)
        "efermi": grab(r"EFermi =\s+(\S+)"),
        "e_total": grab(r"E\(T\) =\s+(\S+)"),
        "fermi_shift": grab(r"Fermi level shift:\s+(\S+)"),
        "pressure": grab(r"P\(T\) =\s+(\S+)"),
        "npairs": grab(r"Number of pairs =\s+(\d+)", int),
        "dismin": grab(r"Minimum distance this configuration =\s+(\S+)"),
    }
    assert len(gold["efermi"]) == len(rows) == 18
    with open(os.path.join(HERE, "ex1_golden.json"), "w") as f:
        json.dump(gold, f, indent=1)
    print("wrote", dst, "and ex1_golden.json")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference/NRLtb/ex1")
