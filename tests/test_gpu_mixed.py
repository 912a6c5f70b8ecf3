"""Mixed-precision form (FP32 eigensolve + FP64-accurate refinement) against the
FP64 oracle.  Tolerances: eigenvalues 1e-9 Ry, E_F 1e-9 Ry, E_total 1e-8 Ry/atom,
pressure 1e-3 kbar (6.8e-9 Ry/bohr^3)."""
import numpy as np
import pytest

import oracle
from nrltb import KMesh, Opts, abi, synth

pytestmark = pytest.mark.gpu

KBAR = 1.0 / 147105.08
P_TOL = 1e-3 * KBAR
MIXED = abi.PREC_MIXED


def _sub(km, idx):
    idx = np.asarray(idx)
    return KMesh(km.k[idx], km.w[idx] / km.w[idx].sum())


def _check(ctx, H, S):
    ge, gz, gst = ctx.diag(H, S, precision=MIXED)
    oe, _, ost = oracle.diag(H, S, vectors=False)
    assert (gst == 0).all() and (ost == 0).all(), gst
    err = np.abs(ge - oe).max()
    assert err <= 1e-9, err
    for k in range(H.shape[0]):
        Z = gz[k]
        res = H[k] @ Z - (S[k] @ Z) * ge[k][None, :]
        assert np.abs(res).max() < 1e-6
    return err


def test_mixed_diag_n9(ctx, ex1):
    st, par, km = ex1.structures[0][2], ex1.params, ex1.structures[0][3]
    H, S = oracle.setham(st, par, km)
    _check(ctx, H, S)


def test_mixed_diag_n288(ctx):
    st, par, km, _ = synth.bcc32()
    H, S = oracle.setham(st, par, _sub(km, [0, 21, 42]))
    _check(ctx, H, S)


def test_mixed_diag_n1152(ctx):
    st, par, km, _ = synth.fcc128()
    H, S = oracle.setham(st, par, _sub(km, [0, 13]))
    _check(ctx, H, S)


def test_mixed_diag_n1404_two_species(ctx):
    st, par, km, _ = synth.b2_216()
    H, S = oracle.setham(st, par, _sub(km, [0]))
    _check(ctx, H, S)


def test_mixed_diag_degenerate(ctx):
    rng = np.random.default_rng(7)
    A = rng.normal(size=(8, 8)) + 1j * rng.normal(size=(8, 8))
    A = A + A.conj().T
    H = np.zeros((1, 32, 32), complex)
    for b in range(4):
        H[0, 8 * b:8 * b + 8, 8 * b:8 * b + 8] = A
    S = np.eye(32)[None].astype(complex)
    _check(ctx, H, S)


def _compare(ctx, st, par, km, tkb):
    opts_m = Opts(mode=4, precision=MIXED, tkb=tkb, eigcut=1e3, fermi_tol=1e-11)
    opts_o = Opts(mode=4, tkb=tkb, eigcut=1e3, fermi_tol=1e-11)
    g = ctx.bande(st, par, km, opts_m)
    o = oracle.bande(st, par, km, opts_o)
    assert (g.k_status == 0).all()
    assert np.abs(g.eig - o.eig).max() <= 1e-9
    assert abs(g.efermi - o.efermi) <= 1e-9
    assert abs(g.e_total - o.e_total) / st.natoms <= 1e-8
    assert abs(g.pressure - o.pressure) <= P_TOL
    return g, o


def test_mixed_bande_fcc1(ctx):
    st, par, km, o = synth.fcc1()
    _compare(ctx, st, par, km, o["tkb"])


def test_mixed_bande_bcc32(ctx):
    st, par, km, o = synth.bcc32()
    _compare(ctx, st, par, _sub(km, [0, 21, 42, 63]), o["tkb"])


def test_mixed_bande_fcc128_two_k(ctx):
    st, par, km, o = synth.fcc128()
    _compare(ctx, st, par, _sub(km, [0, 13]), o["tkb"])


def test_mixed_bande_ex1_against_skout(ctx, ex1, ex1_gold):
    for idx in (0, 9):
        _, _, st, km = ex1.structures[idx]
        r = ctx.bande(st, ex1.params, km, Opts(mode=4, precision=MIXED, tkb=ex1.tkb, eigcut=ex1.eigcut))
        assert r.efermi == pytest.approx(ex1_gold["efermi"][idx], abs=1e-9)
        assert r.e_total == pytest.approx(ex1_gold["e_total"][idx], abs=1e-9)
        assert r.pressure == pytest.approx(ex1_gold["pressure"][idx], abs=P_TOL)
