"""The SKIN reader's generated k-point meshes (kptin.f's NKV <= 0 branch with
kptgen.f, rdspgp.f): the C reader against the numpy restatement in
oracle/kptgen.py (same points in the same order, same weights), and the bcc
mesh against the reference's own ex1/bcc.08 (its 55 points and weights, each
point up to a symmetry-equivalent representative)."""
import os
import shutil

import numpy as np
import pytest

import kptgen as okpt
from nrltb import read_skin, synth

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ex1")


def _write(dirname, latline, plv_or_none, lattic, sgname, ilat, mesh_lines):
    par = synth.make_params([9], [10.0], seed=1)
    os.makedirs(dirname, exist_ok=True)
    synth.write_params(os.path.join(dirname, "par"), par)
    shutil.copy(os.path.join(GOLD, sgname), os.path.join(dirname, sgname))
    with open(os.path.join(dirname, "SKIN"), "w") as f:
        f.write("Mode=3\n0.005 1000\npar\n")
        f.write("mesh test\ns0\n0\n")
        for line in latline:
            f.write(line + "\n")
        f.write("0\n1\n1 1 1\nF\n-1 0 0 0 0 0 0\n")
        f.write("NEWSYM=T\nLATTIC=%d\n%s\nILAT=%s\n" % (lattic, sgname, "T" if ilat else "F"))
        for line in mesh_lines:
            f.write(line + "\n")


def _read(dirname):
    sk = read_skin(os.path.join(dirname, "SKIN"))
    st, km = sk.structures[0][2], sk.structures[0][3]
    return np.array(st.plv, float), np.array(km.k), np.array(km.w)


def _kfile(path):
    lines = open(path).read().splitlines()
    n = int(lines[0][:5])
    q = np.array([[float(x) for x in ln.split()[:3]] for ln in lines[1:1 + n]])
    w = np.array([float(ln.split()[3]) for ln in lines[1:1 + n]])
    return q, w


def test_bcc_mesh_reproduces_ex1(tmp_path):
    d = str(tmp_path / "bcc")
    _write(d, ["2", "5.80"], None, 2, "spcgrp.bcc", False, ["    0", "LSPEC=F LINFOK=F", "   16   16   16    0    0"])
    plv, q, w = _read(d)
    qo, wo, rspct = okpt.kptin_mesh(plv, 2, os.path.join(d, "spcgrp.bcc"), False, (16, 16, 16))
    assert q.shape == qo.shape and np.array_equal(q, qo) and np.array_equal(w, wo)
    assert len(q) == 55 and w.sum() == pytest.approx(1.0, abs=1e-15)
    # every point of the reference's bcc.08 is one of ours up to a rotation, a
    # reciprocal lattice vector and time reversal, with the same weight
    qg, wg = _kfile(os.path.join(GOLD, "bcc.08"))
    rs = [np.array(r) for r in rspct]
    used = set()
    for p, wp in zip(qg, wg):
        hit = None
        for i, u in enumerate(q):
            if i in used:
                continue
            for r in rs:
                v = r @ u
                if any(np.abs(sg * v - p - np.round(sg * v - p)).sum() < 1e-6 for sg in (1, -1)):
                    hit = i
                    break
            if hit is not None:
                break
        assert hit is not None, p
        used.add(hit)
        assert w[hit] == wp, (p, w[hit], wp)


@pytest.mark.parametrize("lspec", [False, True])
def test_fcc_mesh_matches_restatement(tmp_path, lspec):
    d = str(tmp_path / ("fcc%d" % lspec))
    flag = "T" if lspec else "F"
    _write(d, ["1", "7.37"], None, 1, "spcgrp.fcc", False,
           ["    0", "LSPEC=%s LINFOK=F" % flag, "    6    6    6    0    0"])
    plv, q, w = _read(d)
    qo, wo, _ = okpt.kptin_mesh(plv, 1, os.path.join(d, "spcgrp.fcc"), False, (6, 6, 6), lspec=lspec)
    assert np.array_equal(q, qo) and np.array_equal(w, wo)
    assert w.sum() == pytest.approx(1.0, abs=1e-14)


def test_selection_and_information_points(tmp_path):
    d = str(tmp_path / "sel")
    # two information-only points (NKV = -2, LINFOK), then points 3..10 kept and renormalised
    _write(d, ["2", "5.80"], None, 2, "spcgrp.bcc", False,
           ["   -2", "LSPEC=F LINFOK=T", "    8    8    8    3   10", "0.1 0.2 0.3", "0.0 0.0 0.25"])
    plv, q, w = _read(d)
    qo, wo, _ = okpt.kptin_mesh(plv, 2, os.path.join(d, "spcgrp.bcc"), False, (8, 8, 8), kpst=3, kpend=10,
                                info=[(0.1, 0.2, 0.3), (0.0, 0.0, 0.25)])
    assert np.array_equal(q, qo) and np.array_equal(w, wo)
    assert len(q) == 8 and w.sum() == pytest.approx(1.0, abs=1e-15)
