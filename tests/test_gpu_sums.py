"""Fermi level and the band-energy / pressure / entropy sums (fermi.f,
bande.f:1162-1330) on caller eigenvalues through nrltb_sums.

* Against the oracle's own sums on a realistic spectrum (bcc32, modes 4 and
  2): E_F to its stopping tolerance, E(T) 1e-8 Ry per atom, P 1e-3 kbar.
* Ill-conditioned sums: fully occupied states at +-1e8 Ry whose energy and
  pressure terms cancel to O(1).  The device sums are compensated, so E(T) and
  P(T) equal the exact sum of the rounded terms (Fractions) to 1e-9 absolute,
  where a plain FP64 accumulation of the same terms is off by ~1e-7 or more.
"""
import ctypes as C
from fractions import Fraction

import numpy as np
import pytest

import oracle
from nrltb import KMesh, Opts, abi, synth

pytestmark = pytest.mark.gpu

KBAR = 1.0 / 147105.08


def _sums(ctx, eig, deig, w, mode, el, tkb, zfill, tol=1e-12):
    out = np.zeros(8)
    eig = np.ascontiguousarray(eig, dtype=np.float64)
    w = np.ascontiguousarray(w, dtype=np.float64)
    dp = None if deig is None else np.ascontiguousarray(deig, dtype=np.float64).ctypes.data_as(abi._dp)
    rc = ctx.lib.nrltb_sums(ctx.h, eig.shape[1], eig.shape[0], eig.ctypes.data_as(abi._dp), dp,
                            w.ctypes.data_as(abi._dp), mode, el, tkb, zfill, tol, out.ctypes.data_as(abi._dp))
    assert rc == abi.NRLTB_OK, ctx.lib.nrltb_last_error()
    return out


@pytest.mark.parametrize("mode", [4, 2])
def test_sums_match_oracle(ctx, mode):
    st, par, km, o = synth.bcc32()
    sub = KMesh(km.k[::8], km.w[::8] / km.w[::8].sum())
    opts = Opts(mode=mode, tkb=o["tkb"], eigcut=1e3, fermi_tol=1e-11)
    r = oracle.bande(st, par, sub, opts)
    zfill = st.natoms * par.valence[0] + st.zcharge
    out = _sums(ctx, r.eig, r.deig, sub.w, mode, 2.0, o["tkb"], zfill, 1e-11)
    assert abs(out[0] - r.efermi) <= 1e-9
    assert abs(out[1] - r.e_total) / st.natoms <= 1e-8
    assert abs(out[2] - r.pressure) <= 1e-3 * KBAR
    if mode == 2:
        assert abs(out[4] - r.entropy) <= 1e-9


def _cancelling_spectrum(nk, nocc, seed):
    """Rows of ascending eigenvalues of an insulator: nocc occupied states,
    half near -1e8 and half near +1e8 - 10 Ry, whose energy terms cancel
    pairwise to O(1); a 14 Ry gap; 16 empty states.  Their derivatives deig
    are +-1e8 Ry/bohr^3 and cancel the same way."""
    rng = np.random.default_rng(seed)
    X = 1.0e8
    eig = np.zeros((nk, nocc + 16))
    deig = np.zeros_like(eig)
    for k in range(nk):
        a = rng.uniform(0.0, 1.0, nocc // 2)
        b = rng.uniform(0.0, 1.0, nocc // 2)
        eig[k] = np.concatenate([np.sort(-X + a), np.sort(X - 10.0 + b), X + 5.0 + np.sort(rng.uniform(0, 1, 16))])
        deig[k, :nocc] = rng.permutation(np.concatenate([1e8 + rng.uniform(-1, 1, nocc // 2),
                                                         -1e8 + rng.uniform(-1, 1, nocc // 2)]))
        deig[k, nocc:] = rng.uniform(-1.0, 1.0, 16)
    return eig, deig


def test_compensated_sums_ill_conditioned(ctx):
    nk, nocc, tkb, el = 8, 2000, 0.005, 2.0
    eig, deig = _cancelling_spectrum(nk, nocc, 11)
    w = np.full(nk, 1.0 / nk)
    out = _sums(ctx, eig, deig, w, 4, el, tkb, el * nocc)
    # insulator: E_F at mid-gap, every occupied f = 1, no window states, so
    # E(T) = sum w el e and P(T) = -sum w el deig over the occupied states:
    # exact sums of the rounded terms, as the kernel forms them (wt = el w)
    assert abs(out[0] - 0.5 * (eig[:, nocc - 1].max() + eig[:, nocc].min())) <= 1e-6
    exact_e = Fraction(0)
    exact_d = Fraction(0)
    plain_e = plain_d = 0.0
    for k in range(nk):
        wt = el * w[k]
        for i in range(nocc):
            t, u = wt * eig[k, i], wt * deig[k, i]
            exact_e += Fraction(t)
            exact_d += Fraction(u)
            plain_e += t
            plain_d += u
    exact_e, exact_p = float(exact_e), -float(exact_d)
    assert abs(out[1] - exact_e) <= 1e-9, (out[1], exact_e)
    assert abs(out[2] - exact_p) <= 1e-9, (out[2], exact_p)
    # the test is ill-conditioned: plain accumulations miss by far more
    assert abs(plain_e - exact_e) > 1e-7 and abs(-plain_d - exact_p) > 1e-7
