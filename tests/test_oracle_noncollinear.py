"""Non-collinear spins (spin flag N, input1.f:754-771; setpar.f/setparv.f lnoncol
branches; spinham.f; addspins.f) in the reader and the oracle.

The reference records no non-collinear run.  The oracle's 2N x 2N problem is
pinned on a CsCl cell of one spd species with a two-set parameter file whose
sets share their hopping and overlap integrals:

* all spins along z: the problem splits into the two collinear channels, so
  the eigenvalues are those of the collinear two-set run, merged, and E_F,
  E(T), P(T) agree;
* the same direction for every atom, any direction: the same spectrum (the
  spin terms are sigma . m per orbital, unitarily equivalent for every unit m);
* antiparallel spins: the collinear run with the second atom flipped;
* canted spins: P(T) = -dE/dV by a five-point difference.

The cross-species on-site terms follow the reference's lnoncol code, which
differs from its collinear form (setpar.f:768-794); they are checked against
a numpy restatement of those lines.
"""
import math
import os
from dataclasses import replace

import numpy as np
import pytest

import oracle
from nrltb import Opts, Structure, abi, read_skin, synth

A, TKB = 5.6, 0.01


def _dirs(angles):
    return np.array([[math.sin(math.radians(t)) * math.cos(math.radians(p)),
                      math.sin(math.radians(t)) * math.sin(math.radians(p)), math.cos(math.radians(t))]
                     for t, p in angles])


def _cscl(a=A, flip=None, angles=None, dnn=16.5, kinds=(1, 1)):
    plv = np.eye(3) * a
    return Structure(list(kinds), [[0, 0, 0], [a / 2, a / 2, a / 2]], plv, synth.search_box(plv, dnn), a ** 3,
                     flip=None if flip is None else np.array(flip),
                     spinat=None if angles is None else _dirs(angles))


def _opts(mode=4, tol=1e-12):
    return Opts(mode=mode, tkb=TKB, eigcut=1e3, fermi_tol=tol)


@pytest.fixture(scope="module")
def mag():
    return synth.make_magnetic_params([9], [10.0], 7, split=0.08)


@pytest.fixture(scope="module")
def km():
    return synth.mp_mesh(3)


def _merged(r, nk):
    return np.sort(np.concatenate([r.eig[:nk], r.eig[nk:]], axis=1), axis=1)


def test_spins_along_z_are_the_collinear_run(mag, km):
    col = oracle.bande(_cscl(), mag, km, _opts())
    nc = oracle.bande(_cscl(angles=[(0, 0), (0, 0)]), mag, km, _opts())
    assert nc.nv == 2 * col.nv and nc.eig.shape == (km.nk, 2 * col.nv)
    assert np.abs(_merged(col, km.nk) - nc.eig).max() <= 1e-13
    assert nc.efermi == pytest.approx(col.efermi, abs=1e-11)
    assert nc.e_total == pytest.approx(col.e_total, abs=1e-11)
    assert nc.pressure == pytest.approx(col.pressure, abs=1e-13)
    assert nc.smag == 0.0   # bande.f:1336: no populations for the one doubled problem


@pytest.mark.parametrize("theta,phi", [(37.0, 110.0), (180.0, 0.0), (90.0, -45.0)])
def test_common_direction_does_not_matter(mag, km, theta, phi):
    z = oracle.bande(_cscl(angles=[(0, 0), (0, 0)]), mag, km, _opts())
    r = oracle.bande(_cscl(angles=[(theta, phi), (theta, phi)]), mag, km, _opts())
    assert np.abs(r.eig - z.eig).max() <= 1e-13
    assert r.e_total == pytest.approx(z.e_total, abs=1e-12)
    assert r.pressure == pytest.approx(z.pressure, abs=1e-13)


def test_antiparallel_spins_are_the_flipped_run(mag, km):
    col = oracle.bande(_cscl(flip=[0, 1]), mag, km, _opts())
    nc = oracle.bande(_cscl(angles=[(0, 0), (180, 0)]), mag, km, _opts())
    assert np.abs(_merged(col, km.nk) - nc.eig).max() <= 1e-13
    assert nc.e_total == pytest.approx(col.e_total, abs=1e-11)
    assert nc.pressure == pytest.approx(col.pressure, abs=1e-13)


def test_canted_pressure_is_minus_dE_dV(mag, km):
    par = replace(mag, dnn=np.full_like(mag.dnn, 24.0))
    angles = [(0, 0), (90, 30)]

    def energy(eps):
        s = (1.0 + eps) ** (1.0 / 3.0)
        return oracle.bande(_cscl(A * s, angles=angles, dnn=24.0), par, km, _opts(3, 1e-13)).e_total

    r0 = oracle.bande(_cscl(A, angles=angles, dnn=24.0), par, km, _opts(4, 1e-13))
    h = 0.0025
    dedv = (8.0 * (energy(h) - energy(-h)) - (energy(2 * h) - energy(-2 * h))) / (12.0 * h * A ** 3)
    assert abs(-dedv - r0.pressure) <= 1e-3 / 147105.08
    # the canted order lies between the parallel and antiparallel energies
    e_fm = oracle.bande(_cscl(A, angles=[(0, 0), (0, 0)], dnn=24.0), par, km, _opts(3)).e_total
    e_afm = oracle.bande(_cscl(A, angles=[(0, 0), (180, 0)], dnn=24.0), par, km, _opts(3)).e_total
    assert min(e_fm, e_afm) < r0.e_total < max(e_fm, e_afm)


def test_needs_two_parameter_sets(km):
    p1 = synth.make_params([9], [10.0], 7)
    with pytest.raises(AssertionError):
        oracle.bande(_cscl(angles=[(0, 0), (0, 0)]), p1, km, _opts())


def test_cross_species_onsite_terms_restated():
    mag2 = synth.make_magnetic_params([9, 9], [10.0, 9.0], 3, split=0.05)
    st = _cscl(angles=[(0, 0), (0, 0)], kinds=(1, 2))
    pairs, _, _ = oracle.search2(st, mag2)
    nc = oracle.noncol_onsite(st, mag2, pairs)
    paros, spinos = nc["paros"], nc["spinos"]
    npar = mag2.param.size // 2
    p1 = replace(mag2, param=mag2.param[:npar], jspins=1)
    p2 = replace(mag2, param=mag2.param[npar:], jspins=1)
    st0 = replace(st, spinat=None)
    den1 = oracle.setpar(st0, p1, pairs, deriv=False)["den"]
    den2 = oracle.setpar(st0, p2, pairs, deriv=False)["den"]
    P1, P2 = np.concatenate([[0.0], p1.param]), np.concatenate([[0.0], p2.param])   # 1-based
    kinds = 2
    for iat, jk1 in enumerate(st.kkind):
        ip = (jk1 - 1) * 17 + 1
        up, dn = den1[iat, jk1 - 1] ** (2 / 3), den2[iat, jk1 - 1] ** (2 / 3)
        want_p, want_s = np.zeros(4), np.zeros(4)
        for k in range(4):
            pu = P1[ip + 1] + up * (P1[ip + 2] + up * (P1[ip + 3] + up * P1[ip + 4]))
            pd = P2[ip + 1] + dn * (P2[ip + 2] + dn * (P2[ip + 3] + dn * P2[ip + 4]))
            want_p[k], want_s[k] = 0.5 * (pu + pd), 0.5 * (pu - pd)
            ip += 4
        for jk2 in range(1, kinds + 1):
            if jk2 == jk1 or not max(den1[iat, jk2 - 1], den2[iat, jk2 - 1]) > 0:
                continue
            up, dn = den1[iat, jk2 - 1] ** (2 / 3), den2[iat, jk2 - 1] ** (2 / 3)
            jkx, jkm = max(jk1, jk2), min(jk1, jk2)
            ip = kinds * 17 + 24 * ((jkx - 1) * (jkx - 2) // 2 + jkm - 1)
            if jk2 < jkx:
                ip += 12
            for k in range(4):   # replaces, 4 coefficients, stride 4, full difference
                pu = P1[ip + 1] + up * (P1[ip + 2] + up * (P1[ip + 3] + up * P1[ip + 4]))
                pd = P2[ip + 1] + dn * (P2[ip + 2] + dn * (P2[ip + 3] + dn * P2[ip + 4]))
                want_p[k], want_s[k] = 0.5 * (pu + pd), pu - pd
                ip += 4
        np.testing.assert_allclose(paros[iat], want_p, rtol=1e-13, atol=1e-15)
        np.testing.assert_allclose(spinos[iat], want_s, rtol=1e-13, atol=1e-15)


def test_reader_spin_directions(tmp_path, mag, km):
    st = _cscl(angles=[(30, 40), (150, -70)])
    synth.write_skin(str(tmp_path), [(st, km)], mag, mode=4, tkb=TKB)
    s2 = read_skin(os.path.join(str(tmp_path), "SKIN")).structures[0][2]
    assert s2.spinat is not None and s2.flip is None
    np.testing.assert_allclose(s2.spinat, st.spinat, atol=1e-14)


def _sd(mode=3):
    return Opts(mode=mode, tkb=TKB, eigcut=1e3, fermi_tol=1e-12, flags=abi.OPT_SPIN_DIRECTIONS)


def test_spin_directions(mag, km):
    """diag.f:458-524 / bande.f:1480-1560: each atom's occupied-state spin
    vector (the reference's sign convention: along -m for a common m)."""
    z = oracle.bande(_cscl(angles=[(0, 0), (0, 0)]), mag, km, _sd())
    assert z.spdir.shape == (2, 3)
    assert np.abs(z.spdir[:, :2]).max() == 0.0 and (z.spdir[:, 2] < -0.5).all()
    for t, p in ((37, 110), (150, -70)):
        r = oracle.bande(_cscl(angles=[(t, p), (t, p)]), mag, km, _sd())
        m = _dirs([(t, p)])[0]
        for j in range(2):   # the vectors turn with the common direction
            np.testing.assert_allclose(r.spdir[j], z.spdir[j, 2] * m, atol=1e-12)
    afm = oracle.bande(_cscl(angles=[(0, 0), (180, 0)]), mag, km, _sd())
    np.testing.assert_allclose(afm.spdir[1], -afm.spdir[0], atol=1e-12)
    assert afm.spdir[0, 2] < -0.5


def test_spin_directions_count_the_moment_for_an_orthogonal_set(mag, km):
    """Without an overlap the z components are populations: their sum is the
    collinear run's spin-down minus spin-up electrons."""
    orth = replace(mag, jsover=0)
    col = oracle.bande(_cscl(), orth, km, _opts(3))
    nc = oracle.bande(_cscl(angles=[(0, 0), (0, 0)]), orth, km, _sd())
    assert nc.spdir[:, 2].sum() == pytest.approx(-col.smag, abs=1e-9)


def test_reader_spin_options(tmp_path, mag, km):
    for flag, want in (("FS", 1), ("FD", 2), ("FN", 0)):
        d = os.path.join(str(tmp_path), flag)
        synth.write_skin(d, [(_cscl(angles=[(10, 20), (30, 40)]), km)], mag, mode=3, tkb=TKB)
        path = os.path.join(d, "SKIN")
        text = open(path).read().replace("\nFN\n", "\n%s\n" % flag)
        open(path, "w").write(text)
        sk = read_skin(path)
        assert sk.spin_options == [want] and sk.structures[0][2].spinat is not None
