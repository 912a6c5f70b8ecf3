"""Orthogonal parameter sets (S = I, diag.f:368-412) and the reference's ex2
structure (Ti hcp, two atoms, generated 12^3 mesh) on the GPU path against the
oracle, in both precision forms.

Tolerances as for the other parity tests: eigenvalues 1e-10 Ry (FP64) / 1e-9
Ry (mixed), E_F 1e-9 Ry, E(T) 1e-8 Ry/atom, P 1e-3 kbar.
"""
import os
import shutil
from dataclasses import replace

import numpy as np
import pytest

import oracle
from conftest import GOLDEN
from nrltb import KMesh, Opts, abi, read_skin, synth

pytestmark = pytest.mark.gpu

KBAR = 1.0 / 147105.08
P_TOL = 1e-3 * KBAR


def _check(ctx, st, par, km, tkb, mode, precision):
    opts = Opts(mode=mode, precision=precision, tkb=tkb, eigcut=1e3, fermi_tol=1e-11)
    g = ctx.bande(st, par, km, opts)
    o = oracle.bande(st, par, km, Opts(mode=mode, tkb=tkb, eigcut=1e3, fermi_tol=1e-11))
    etol = 1e-10 if precision == abi.PREC_FP64 else 1e-9
    assert (g.k_status == 0).all() and g.npairs == o.npairs
    assert np.abs(g.eig - o.eig).max() <= etol
    assert abs(g.efermi - o.efermi) <= 1e-9
    assert abs(g.e_total - o.e_total) / st.natoms <= 1e-8
    if mode in (2, 4):
        assert abs(g.pressure - o.pressure) <= P_TOL
    if mode in (1, 2):
        assert abs(g.earg1 - o.earg1) / st.natoms <= 1e-8
        assert abs(g.earg2 - o.earg2) <= (P_TOL if mode == 2 else 1e-8 * st.natoms)
    return g, o


@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_MIXED])
def test_orthogonal_fcc1(ctx, precision):
    st, par, km, o = synth.fcc1()
    idx = np.arange(0, km.nk, 37)
    km = KMesh(km.k[idx], km.w[idx] / km.w[idx].sum())
    _check(ctx, st, replace(par, jsover=0), km, o["tkb"], 4, precision)


@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_MIXED])
def test_orthogonal_bcc32_mode2(ctx, precision):
    st, par, km, o = synth.bcc32()
    idx = np.array([0, 21, 42, 63])
    km = KMesh(km.k[idx], km.w[idx] / km.w[idx].sum())
    _check(ctx, st, replace(par, jsover=0), km, o["tkb"], 2, precision)


@pytest.fixture(scope="module")
def ex2(tmp_path_factory):
    d = str(tmp_path_factory.mktemp("ex2"))
    for f in ("SKIN", "ti_par", "spcgp1.hcp"):
        shutil.copy(os.path.join(GOLDEN, "ex2", f), os.path.join(d, f))
    path = os.path.join(d, "SKIN")
    # the mesh line right-justified: 12 divisions, not the 12000 that blank='zero' reads
    text = open(path).read().replace("\n12   12   12 ", "\n   12   12   12")
    open(path, "w").write(text)
    return read_skin(path)


@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_MIXED])
@pytest.mark.parametrize("mode", [3, 1])
def test_ex2_hcp(ctx, ex2, mode, precision):
    for j in (0, 12):
        _, _, st, km = ex2.structures[j]
        _check(ctx, st, ex2.params, km, ex2.tkb, mode, precision)
