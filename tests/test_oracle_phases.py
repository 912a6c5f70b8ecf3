"""The per-atom Bloch phase offsets posq (/fazon/, input1.f:795; rotate.f:144-146):
they enter the phase of every pair as k . (dlv - posq(atom 2) + posq(atom 1)),
that is H(k) -> D H(k) D^H and S(k) -> D S(k) D^H with D diagonal and unitary
(one phase per atom), so the eigenvalues, E_F, E(T) and P(T) do not depend on
them, while the matrices do."""
import numpy as np
import pytest

import oracle
from nrltb import KMesh, Opts, Structure, synth


def _case(posq):
    st, par, km, o = synth.bcc32()
    idx = np.array([0, 9, 37, 63])
    km = KMesh(km.k[idx], km.w[idx] / km.w[idx].sum())
    st = Structure(st.kkind, st.posn, st.plv, st.nd, st.volume, st.zcharge, posq)
    return st, par, km, o["tkb"]


def test_offsets_are_a_gauge():
    rng = np.random.default_rng(4)
    st0, par, km, tkb = _case(None)
    st1, _, _, _ = _case(rng.uniform(-0.5, 0.5, (32, 3)))
    h0, s0 = oracle.setham(st0, par, km)
    h1, s1 = oracle.setham(st1, par, km)
    assert np.abs(h1 - h0).max() > 1e-3                       # the matrices change
    # D = diag(exp(2 pi i k . posq_atom)) on every orbital of the atom
    orb_atom = np.repeat(np.arange(32), par.kbas[st0.kkind - 1])
    for k in range(km.nk):
        ph = np.exp(2j * np.pi * (st1.posq[orb_atom] @ km.k[k]))
        for a, b in ((h0[k], h1[k]), (s0[k], s1[k])):
            assert np.abs(ph[:, None] * a * ph.conj()[None, :] - b).max() <= 1e-12 * np.abs(a).max()
    op = Opts(mode=4, tkb=tkb, eigcut=1e3, fermi_tol=1e-12)
    r0, r1 = oracle.bande(st0, par, km, op), oracle.bande(st1, par, km, op)
    assert np.abs(r0.eig - r1.eig).max() <= 1e-11
    assert r1.e_total == pytest.approx(r0.e_total, abs=1e-10)
    assert r1.pressure == pytest.approx(r0.pressure, abs=1e-12)
