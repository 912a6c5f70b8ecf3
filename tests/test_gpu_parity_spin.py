"""Collinear spin-polarized sets (jspins = 2) and spin flips on the GPU path
against the oracle, in both precision forms, on a CsCl cell of one spd species
(two atoms, 4^3 k points, 20 electrons over 18 bands per spin).

Tolerances: eigenvalues of both spin channels 1e-10 Ry (FP64) / 1e-9 Ry
(mixed), E_F 1e-9 Ry, E(T) 1e-8 Ry/atom, P 1e-3 kbar, moment 1e-8 electrons.
"""
import os
import subprocess
from dataclasses import replace

import numpy as np
import pytest

import oracle
from nrltb import Opts, Structure, abi, build, synth

pytestmark = pytest.mark.gpu

KBAR = 1.0 / 147105.08
P_TOL = 1e-3 * KBAR
A, TKB = 5.6, 0.01


def _cscl(flip=None):
    plv = np.eye(3) * A
    return Structure([1, 1], [[0, 0, 0], [A / 2, A / 2, A / 2]], plv, synth.search_box(plv, 16.5), A ** 3,
                     flip=None if flip is None else np.array(flip))


@pytest.fixture(scope="module")
def mag():
    return synth.make_magnetic_params([9], [10.0], 7, split=0.08)


@pytest.fixture(scope="module")
def km():
    return synth.mp_mesh(4)


@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_MIXED])
@pytest.mark.parametrize("mode", [4, 2])
@pytest.mark.parametrize("flip", [None, [0, 1]])
def test_spin_against_oracle(ctx, mag, km, precision, mode, flip):
    st = _cscl(flip)
    g = ctx.bande(st, mag, km, Opts(mode=mode, precision=precision, tkb=TKB, eigcut=1e3, fermi_tol=1e-11))
    o = oracle.bande(st, mag, km, Opts(mode=mode, tkb=TKB, eigcut=1e3, fermi_tol=1e-11))
    etol = 1e-10 if precision == abi.PREC_FP64 else 1e-9
    assert g.eig.shape == (2 * km.nk, o.nv) and (g.k_status == 0).all()
    assert np.abs(g.eig - o.eig).max() <= etol
    assert abs(g.efermi - o.efermi) <= 1e-9
    assert abs(g.e_total - o.e_total) / st.natoms <= 1e-8
    assert abs(g.pressure - o.pressure) <= P_TOL
    assert abs(g.smag - o.smag) <= 1e-8
    assert abs(g.earg1 - o.earg1) / st.natoms <= 1e-8
    if mode == 2:
        assert abs(g.earg2 - o.earg2) <= P_TOL
    if flip is None:
        assert g.smag > 1.0
    else:
        assert abs(g.smag) <= 1e-10


def test_identical_sets_match_spin_restricted(ctx, km):
    p1 = synth.make_params([9], [10.0], 7)
    p2 = replace(p1, param=np.concatenate([p1.param, p1.param]), jspins=2)
    st = _cscl()
    r1 = ctx.bande(st, p1, km, Opts(mode=4, tkb=TKB, eigcut=1e3, fermi_tol=1e-12))
    r2 = ctx.bande(st, p2, km, Opts(mode=4, tkb=TKB, eigcut=1e3, fermi_tol=1e-12))
    assert np.array_equal(r2.eig[:km.nk], r1.eig) and np.array_equal(r2.eig[km.nk:], r1.eig)
    assert abs(r2.efermi - r1.efermi) <= 1e-11
    assert abs(r2.e_total - r1.e_total) <= 1e-11
    assert abs(r2.pressure - r1.pressure) <= 1e-12
    assert r2.smag == 0.0


def test_host_driver_spin_skeng(tmp_path, mag, km):
    st = _cscl([0, 1])
    synth.write_skin(str(tmp_path), [(st, km), (_cscl(), km)], mag, mode=4, tkb=TKB)
    r = subprocess.run([build.DRIVER, "SKIN"], cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    lines = (tmp_path / "SKENG").read_text().splitlines()
    assert len(lines) == 2
    for line, s in zip(lines, (st, _cscl())):
        o = oracle.bande(s, mag, km, Opts(mode=4, tkb=TKB, eigcut=1e3))
        vals = [float(x) for x in line[20:].split()]
        assert len(vals) == 5   # volume, E_F, E(T), P(T), moment (a20,f12.6,3f15.9,f10.6)
        for v, ref in zip(vals[1:4], (o.efermi, o.earg1, o.earg2)):
            assert abs(v - ref) <= 1.01e-9
        assert abs(vals[4] - o.smag) <= 5.01e-7
    assert "magnetization" in (tmp_path / "SKOUT").read_text()
