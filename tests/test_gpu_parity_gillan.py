"""Modes 1 and 2 (Gillan's T -> 0 extrapolation, bande.f:1100-1476) on the GPU
path against the oracle, in both precision forms.

Tolerances: E_F 1e-9 Ry; E(T), A(T) = E - kT S and E(0) 1e-8 Ry/atom (so kT S
too); P(T), the entropy shift and P(0) 1e-3 kbar.  Modes 1 and 2 give E_F, E(T),
P(T) and the Fermi-level shift bit for bit as modes 3 and 4 do on the same
context.  The host driver's SKENG line in mode 2 carries E_F, E(0) and P(0).
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle
from conftest import GOLDEN
from nrltb import Opts, abi, build, read_skin

pytestmark = pytest.mark.gpu

KBAR = 1.0 / 147105.08
P_TOL = 1e-3 * KBAR


def _skin(dirname, mode, tkb, alats):
    os.makedirs(dirname, exist_ok=True)
    for f in ("pd_par", "spcgrp.fcc", "fcc.08"):
        shutil.copy(os.path.join(GOLDEN, "ex1", f), os.path.join(dirname, f))
    with open(os.path.join(dirname, "SKIN"), "w") as f:
        f.write("Mode=%d\n%.17g 0.5\npd_par\n" % (mode, tkb))
        for j, a in enumerate(alats):
            f.write("Pd fcc\n fcc %.4f\n 0.00\n 1\n %.17g\n 0\n 1\n 4 4 4\nF\n 1 0 0 0 0 0 0\n" % (a, a))
            f.write("NEWSYM=T\nLATTIC=1\nspcgrp.fcc\nILAT=F\n-1313\nfcc.08\n" if j == 0 else "NEWSYM=F\n")
    return read_skin(os.path.join(dirname, "SKIN"))


@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_MIXED])
@pytest.mark.parametrize("mode", [1, 2])
@pytest.mark.parametrize("idx,tkb", [(0, 0.005), (9, 0.005), (4, 0.02)])
def test_gillan_against_oracle(ctx, ex1, mode, precision, idx, tkb):
    _, _, st, km = ex1.structures[idx]
    opts = Opts(mode=mode, precision=precision, tkb=tkb, eigcut=ex1.eigcut, fermi_tol=1e-11)
    g = ctx.bande(st, ex1.params, km, opts)
    o = oracle.bande(st, ex1.params, km, Opts(mode=mode, tkb=tkb, eigcut=ex1.eigcut, fermi_tol=1e-11))
    na = st.natoms
    assert abs(g.efermi - o.efermi) <= 1e-9
    assert abs(g.e_total - o.e_total) / na <= 1e-8
    assert o.entropy > 0
    assert abs(tkb * (g.entropy - o.entropy)) / na <= 1e-8
    assert abs(g.free_energy - o.free_energy) / na <= 1e-8
    assert abs(g.earg1 - o.earg1) / na <= 1e-8
    if mode == 1:
        assert g.earg2 == g.e_total and g.entropy_shift == 0
    else:
        assert abs(g.pressure - o.pressure) <= P_TOL
        assert abs(g.entropy_shift - o.entropy_shift) <= P_TOL
        assert abs(g.earg2 - o.earg2) <= P_TOL


@pytest.mark.parametrize("gillan,plain", [(1, 3), (2, 4)])
def test_gillan_modes_keep_the_plain_outputs(ctx, ex1, gillan, plain):
    _, _, st, km = ex1.structures[13]
    g = ctx.bande(st, ex1.params, km, Opts(mode=gillan, tkb=ex1.tkb, eigcut=ex1.eigcut))
    p = ctx.bande(st, ex1.params, km, Opts(mode=plain, tkb=ex1.tkb, eigcut=ex1.eigcut))
    assert (g.efermi, g.e_total, g.pressure, g.fermi_shift) == (p.efermi, p.e_total, p.pressure, p.fermi_shift)
    assert np.array_equal(g.eig, p.eig)
    assert p.entropy == 0 and p.earg1 == p.e_total and p.earg2 == (p.pressure if plain == 4 else 0.0)


def test_host_driver_mode2_skeng(tmp_path):
    tkb = 0.01
    sk = _skin(str(tmp_path), 2, tkb, [7.0, 7.3])
    r = subprocess.run([build.DRIVER, "SKIN"], cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    lines = (tmp_path / "SKENG").read_text().splitlines()
    assert len(lines) == 2
    for line, (_, _, st, km) in zip(lines, sk.structures):
        o = oracle.bande(st, sk.params, km, Opts(mode=2, tkb=tkb, eigcut=sk.eigcut))
        vals = [float(x) for x in line[20:].split()]
        assert len(vals) == 4
        assert abs(vals[0] - st.volume) <= 5e-7
        for v, ref in zip(vals[1:], (o.efermi, o.earg1, o.earg2)):
            assert abs(v - ref) <= 1.01e-9
    out = (tmp_path / "SKOUT").read_text()
    assert out.count("P(0) =") == 2 and out.count("S(T) =") == 2
