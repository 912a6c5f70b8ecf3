"""The parameter forms nltype 1 (real overlap), 2 (Harrison signs), 3 (both)
and 90000 (H-atom ss-sigma) on the GPU path against the oracle: the Slater-
Koster tables, densities and on-site terms with their volume derivatives, and
a whole mode-4 run in both precision forms, on fcc1 (k subset) with overlap
parameters scaled to 0.05 and on a two-species B2 cell (the forms act on
like-species pairs only).  Tolerances as for the other parity tests."""
from dataclasses import replace

import numpy as np
import pytest

import oracle
from nrltb import KMesh, Opts, Structure, abi, synth

pytestmark = pytest.mark.gpu

KBAR = 1.0 / 147105.08
FORMS = [(1, 1), (2, 1), (3, 1), (90000, 1), (90000, 0)]


def _fcc(nltype, jsover):
    st, _, km, o = synth.fcc1()
    idx = np.arange(0, km.nk, 131)
    par = synth.make_params([9], [10.0], 12, s_scale=0.05)
    return st, replace(par, nltype=nltype, jsover=jsover), KMesh(km.k[idx], km.w[idx] / km.w[idx].sum()), o["tkb"]


def _b2(nltype, jsover):
    a = 5.6
    plv = np.eye(3) * a
    st = Structure([1, 2], [[0, 0, 0], [a / 2, a / 2, a / 2]], plv, synth.search_box(plv, 16.5), a ** 3)
    par = synth.make_params([9, 4], [10.0, 3.0], 7, s_scale=0.05)   # S positive definite at every k
    return st, replace(par, nltype=nltype, jsover=jsover), synth.mp_mesh(3), 0.01


@pytest.mark.parametrize("nltype,jsover", FORMS)
@pytest.mark.parametrize("case", [_fcc, _b2])
def test_setpar_forms(ctx, case, nltype, jsover):
    st, par, _, _ = case(nltype, jsover)
    pairs, _, _ = oracle.search2(st, par)
    o = oracle.setpar(st, par, pairs, deriv=True)
    g = ctx.setpar(st, par, pairs, deriv=True)
    for key in ("hop", "over", "dhop", "dover"):
        scale = max(np.abs(o[key]).max(), 1e-300)
        np.testing.assert_allclose(g[key], o[key], rtol=1e-13, atol=1e-15 * scale, err_msg=key)
    for key in ("den", "paros", "dparos"):
        np.testing.assert_allclose(g[key], o[key], rtol=1e-12, atol=1e-15, err_msg=key)


@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_MIXED])
@pytest.mark.parametrize("nltype,jsover", FORMS)
@pytest.mark.parametrize("case", [_fcc, _b2])
def test_bande_forms(ctx, case, nltype, jsover, precision):
    st, par, km, tkb = case(nltype, jsover)
    g = ctx.bande(st, par, km, Opts(mode=4, precision=precision, tkb=tkb, eigcut=1e3, fermi_tol=1e-11))
    o = oracle.bande(st, par, km, Opts(mode=4, tkb=tkb, eigcut=1e3, fermi_tol=1e-11))
    assert o.nonphysical_k == 0 and g.nonphysical_k == 0
    assert np.abs(g.eig - o.eig).max() <= (1e-10 if precision == abi.PREC_FP64 else 1e-9)
    assert abs(g.efermi - o.efermi) <= 1e-9
    assert abs(g.e_total - o.e_total) / st.natoms <= 1e-8
    assert abs(g.pressure - o.pressure) <= 1e-3 * KBAR


def test_setham_with_phase_offsets(ctx):
    """Per-atom Bloch phase offsets (rotate.f:144-146) in the GPU Bloch sums."""
    st, par, km, _ = synth.bcc32()
    rng = np.random.default_rng(4)
    st = Structure(st.kkind, st.posn, st.plv, st.nd, st.volume, st.zcharge, rng.uniform(-0.5, 0.5, (32, 3)))
    sub = KMesh(km.k[[0, 9, 37, 63]], np.full(4, 0.25))
    for which in (0, 1):
        gh, gs = ctx.setham(st, par, sub, which)
        oh, os_ = oracle.setham(st, par, sub, which)
        for g, o in ((gh, oh), (gs, os_)):
            assert np.abs(g - o).max() <= 1e-13 * max(np.abs(o).max(), 1e-300)
