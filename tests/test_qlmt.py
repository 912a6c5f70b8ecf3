"""The eigenvalue files of modes 6, 8, 9, 10 (static.f:759-781, 1132-1145;
bande.f:1568-1700) and the Lowdin orbital charges behind them (diag.f:526-700).

* The C writer nrltb_qlmt_write against a separate Python restatement of the
  reference's records and edit descriptors (F fields that overflow print
  asterisks; E and D print a 0.ddd mantissa), on hand-made results that reach
  the corner cases: eigenvalues past -10 and 100, the eigcut cut, four
  eigenvalues (QAPW's slash), two spin blocks, s, p and spd atoms, 1x1.
* The oracle's charges: each state's charges sum to 1, they equal numpy's
  |S^1/2 z|^2 summed over degenerate groups, an orthogonal set gives |z|^2,
  and a k point whose overlap is not positive definite gives -1.
"""
import math
import os
from dataclasses import replace

import numpy as np
import pytest
import scipy.linalg as sl

import oracle
from nrltb import KMesh, Opts, Result, Structure, synth, write_qlmt


# ---- Fortran edit descriptors, restated ---------------------------------------
def F(v, w, d):
    s = "%*.*f" % (w, d, v)
    return "*" * w if len(s) > w else s


def E(v, w, d, letter="E"):
    if v == 0.0:
        body = "0." + "0" * d + letter + "+00"
    else:
        m, x = ("%.*e" % (d - 1, abs(v))).split("e")
        ex = int(x) + 1
        body = ("-" if v < 0 else "") + "0." + m.replace(".", "") + letter + ("-" if ex < 0 else "+") + "%02d" % abs(ex)
    return body.rjust(w)


def krec(k, w, ntot):
    return "".join(F(c, 10, 6) for c in k) + "  " + F(w, 10, 5) + "%10d" % ntot + E(w, 20, 10, "D") + " K"


def expected(mode, st, par, km, eigcut, eig, orb):
    nv = eig.shape[1]
    noncol = st.spinat is not None
    nsp = 1 if noncol else par.jspins
    atoms = list(range(st.natoms)) * (2 if noncol else 1)   # diag.f:670-693
    out = []
    if mode in (6, 10):
        out.append("%5d%5d%5d%5d     SPINS, WIND., SC. WIND." % (1, 1, 0, st.natoms))
    elif mode == 9:
        out.append("%5d%5d%5d%5d     SPINS, WIND., SC. WIND." % (1, 1, 0, 0))
    for js in range(nsp):
        for k in range(km.nk):
            row = js * km.nk + k
            en = eig[row]
            if mode == 8:
                line = " " + "".join(F(c, 9, 6) for c in km.k[k]) + " " * 10
                for i, e in enumerate(en):
                    if i and i % 4 == 0:
                        out.append(line)
                        line = " " * 38
                    line += F(e, 9, 5)
                out.append(line)
                if nv == 4:
                    out.append("")
                continue
            if mode == 9:
                out.append(krec(km.k[k], km.w[k], nv))
                out += [F(e, 12, 7) + E(0.0, 15, 6) for e in en]
                continue
            ntot = next((i for i, e in enumerate(en) if e > eigcut), nv)
            if nv == 1:
                ntot = 1
            out.append(krec(km.k[k], km.w[k], ntot))
            for n in range(ntot):
                e = en[n]
                big = mode == 6 and (e <= -10.0 or e >= 100.0)
                out.append(F(e, 10, 6 if big else 7) + E(0.0, 15, 6))
                i0 = 0
                for a in atoms:
                    nb = int(par.kbas[st.kkind[a] - 1])
                    oc = orb[row, n, i0:i0 + nb]
                    if mode == 6:
                        s, p, d = oc[0], 0.0, 0.0
                        for q in range(1, min(nb, 4)):
                            p = p + oc[q]
                        for q in range(4, nb):
                            d = d + oc[q]
                        out.append("".join(F(x, 15, 9) for x in (s, p, d, 0.0)))
                    else:
                        out.append("".join(F(x, 15, 9) for x in oc))
                    i0 += nb
    return out


def _case(kbas, nk, nsp, seed):
    rng = np.random.default_rng(seed)
    natoms = len(kbas)
    par = synth.make_params(sorted(set(kbas)), [4.0] * len(set(kbas)), 1)
    kinds = {b: i + 1 for i, b in enumerate(sorted(set(kbas)))}
    if nsp == 2:
        par = replace(par, param=np.concatenate([par.param, par.param]), jspins=2)
    st = Structure([kinds[b] for b in kbas], rng.uniform(0, 5, (natoms, 3)), np.eye(3) * 6, (1, 1, 1), 216.0)
    km = KMesh(rng.uniform(-0.5, 0.5, (nk, 3)), rng.dirichlet(np.ones(nk)))
    nv = sum(kbas)
    eig = np.sort(rng.uniform(-1.5, 1.5, (nsp * nk, nv)), axis=1)
    eig[0, 0] = -12.345678912        # f10.6 in mode 6, asterisks in f9.5
    eig[0, -1] = 123.456789          # f10.6 in mode 6, asterisks in f10.7
    orb = rng.dirichlet(np.ones(nv), size=(nsp * nk, nv))
    return st, par, km, eig, orb


@pytest.mark.parametrize("mode", [6, 8, 9, 10])
@pytest.mark.parametrize("kbas,nsp", [([9, 4], 1), ([4], 1), ([1, 9, 4], 2), ([1], 1)])
def test_writer_matches_restated_records(tmp_path, mode, kbas, nsp):
    st, par, km, eig, orb = _case(kbas, 3, nsp, len(kbas) + mode)
    res = Result(0.0, 0.0, 0.0, 0.0, 0.0, 0, eig.shape[1], km.nk, 0, 0, eig=eig, orbocc=orb)
    path = str(tmp_path / "Q")
    eigcut = 0.7
    write_qlmt(path, mode, st, par, km, eigcut, res)
    write_qlmt(path, mode, st, par, km, eigcut, res, append=True)   # a second structure appends
    got = open(path).read().split("\n")
    assert got[-1] == ""
    want = expected(mode, st, par, km, eigcut, eig, orb)
    assert got[:-1] == want + want


def test_fortran_edit_descriptors():
    assert F(-12.3456789, 9, 5) == "-12.34568"
    assert F(-123.456789, 9, 5) == "*********"
    assert F(-12.3456789, 10, 7) == "**********"
    assert F(-0.5, 10, 7) == "-0.5000000"
    assert E(0.0, 15, 6) == "   0.000000E+00"
    assert E(0.0123, 20, 10, "D") == "    0.1230000000D-01"
    assert E(1.0, 20, 10, "D") == "    0.1000000000D+01"


def _fcc(kidx):
    st, par, km, o = synth.fcc1()
    return st, par, KMesh(km.k[kidx], km.w[kidx] / km.w[kidx].sum()), o["tkb"]


@pytest.mark.parametrize("mode", [6, 10])
def test_oracle_charges(mode):
    st, par, km, tkb = _fcc(np.arange(0, 1728, 191))
    r = oracle.bande(st, par, km, Opts(mode=mode, tkb=tkb, eigcut=1e3))
    assert r.orbocc.shape == (km.nk, r.nv, r.nv)
    assert np.abs(r.orbocc.sum(axis=2) - 1.0).max() <= 1e-13
    H, S = oracle.setham(st, par, km)
    for k in range(km.nk):
        w, V = np.linalg.eigh(S[k])
        U = (V * np.sqrt(w)) @ V.conj().T
        e, Z = sl.eigh(H[k], S[k])
        occ = np.abs(U @ Z) ** 2                       # occ[orbital, state]
        grp = np.concatenate([[0], np.cumsum(np.diff(e) > 1e-8)])
        for g in np.unique(grp):
            m = grp == g
            assert np.abs(occ[:, m].sum(axis=1) - r.orbocc[k][m].sum(axis=0)).max() <= 1e-12


def test_oracle_charges_orthogonal():
    st, par, km, tkb = _fcc(np.arange(0, 1728, 301))
    par = replace(par, jsover=0)
    r = oracle.bande(st, par, km, Opts(mode=6, tkb=tkb, eigcut=1e3))
    H, _ = oracle.setham(st, par, km)
    for k in range(km.nk):
        e, Z = np.linalg.eigh(H[k])
        occ = np.abs(Z) ** 2
        grp = np.concatenate([[0], np.cumsum(np.diff(e) > 1e-8)])
        for g in np.unique(grp):
            m = grp == g
            assert np.abs(occ[:, m].sum(axis=1) - r.orbocc[k][m].sum(axis=0)).max() <= 1e-12


def test_oracle_charges_nonpositive_overlap():
    st, _, km, _ = synth.fcc1()
    par = synth.make_params([9], [11.0], 11)            # S(k) indefinite at some k
    sub = KMesh(km.k[[0, 340, 471, 900, 1727]], np.full(5, 0.2))
    r = oracle.bande(st, par, sub, Opts(mode=6, tkb=0.005, eigcut=1e3))
    bad = r.k_status != 0
    assert bad.sum() >= 2
    assert (r.orbocc[bad] == -1.0).all()
    assert np.abs(r.orbocc[~bad].sum(axis=2) - 1.0).max() <= 1e-12


@pytest.mark.parametrize("mode", [6, 9, 10])
def test_writer_noncollinear_records(tmp_path, mode):
    """A non-collinear run: one block of 2N eigenvalues per k, charges on the
    spin-up then the spin-down copies of every atom."""
    st, par, km, eig, orb = _case([9, 4], 2, 2, 5)
    nv2 = 2 * eig.shape[1]
    rng = np.random.default_rng(9)
    eig = np.sort(rng.uniform(-1.5, 1.5, (km.nk, nv2)), axis=1)
    orb = rng.dirichlet(np.ones(nv2), size=(km.nk, nv2))
    st = replace(st, spinat=np.array([[0.0, 0.0, 1.0], [1.0, 0.0, 0.0]]))
    res = Result(0.0, 0.0, 0.0, 0.0, 0.0, 0, nv2, km.nk, 0, 0, eig=eig, orbocc=orb)
    path = str(tmp_path / "Q")
    write_qlmt(path, mode, st, par, km, 0.7, res)
    assert open(path).read().split("\n")[:-1] == expected(mode, st, par, km, 0.7, eig, orb)


def test_writer_errors(tmp_path):
    import ctypes as C
    from nrltb import abi
    st, par, km, eig, orb = _case([9], 2, 1, 1)
    lib = abi.load_host()
    r = abi.Result_()
    r.nv, r.nk = eig.shape[1], km.nk
    e = np.ascontiguousarray(eig)
    r.eig = e.ctypes.data_as(C.POINTER(C.c_double))
    cs, cp, ck = st.to_c(), par.to_c(), km.to_c()
    args = (C.byref(cs), C.byref(cp), C.byref(ck), 0.7, C.byref(r))
    path = str(tmp_path / "Q").encode()
    assert lib.nrltb_qlmt_write(path, 0, 5, *args) == abi.NRLTB_E_UNSUPPORTED    # mode 5 is not written
    assert lib.nrltb_qlmt_write(path, 0, 4, *args) == abi.NRLTB_E_UNSUPPORTED
    assert lib.nrltb_qlmt_write(path, 0, 6, *args) == abi.NRLTB_E_ARG            # charges required
    assert lib.nrltb_qlmt_write(str(tmp_path / "no" / "Q").encode(), 0, 9, *args) == abi.NRLTB_E_IO
    assert lib.nrltb_qlmt_write(None, 0, 9, *args) == abi.NRLTB_E_ARG
    assert lib.nrltb_qlmt_write(path, 0, 9, *args) == 0
