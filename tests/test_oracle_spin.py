"""Collinear spin-polarized parameter sets ("M" files, jspins = 2) and spin
flips (input1.f:778-787) in the readers and the oracle.

The reference records no magnetic run, so the oracle's spin path is pinned by
properties on a CsCl cell of one spd species (two atoms, 4^3 k points):

* two identical parameter sets give the spin-restricted result (one electron
  per band over both channels equals two per band over one), moment 0;
* exchanging the two sets changes the sign of the moment and nothing else;
* with the second atom flipped (antiferromagnetic order) the two channels are
  one another under the translation that exchanges the atoms: equal
  eigenvalues and moment exactly 0, where the ferromagnetic order has 2.27;
* P(T) = -dE/dV by a five-point difference, with and without flips;
* E_F solves sum_spins sum_k w_k sum_i f = N with one electron per band, and
  the moment is the window sum of bande.f:1336-1395, both restated here in numpy.

Two spd atoms carry 20 electrons over 18 bands, so with one electron per band
the Fermi bracket's band index (nfill = 20) lies past the computed bands: the
clamped bracket of the oracle and the GPU kernel is exercised here.
"""
import math
import os
from dataclasses import replace

import numpy as np
import pytest

import oracle
from nrltb import Opts, Structure, read_skin, synth

A = 5.6
TKB = 0.01


def _cscl(a=A, flip=None, dnn=16.5):
    plv = np.eye(3) * a
    return Structure([1, 1], [[0, 0, 0], [a / 2, a / 2, a / 2]], plv, synth.search_box(plv, dnn), a ** 3,
                     flip=None if flip is None else np.array(flip))


def _opts(mode=4, tol=1e-12):
    return Opts(mode=mode, tkb=TKB, eigcut=1e3, fermi_tol=tol)


@pytest.fixture(scope="module")
def mag():
    return synth.make_magnetic_params([9], [10.0], 7, split=0.08)


@pytest.fixture(scope="module")
def km():
    return synth.mp_mesh(4)


def test_identical_sets_are_spin_restricted(km):
    p1 = synth.make_params([9], [10.0], 7)
    p2 = replace(p1, param=np.concatenate([p1.param, p1.param]), jspins=2)
    st = _cscl()
    r1 = oracle.bande(st, p1, km, _opts())
    r2 = oracle.bande(st, p2, km, _opts())
    assert r2.eig.shape == (2 * km.nk, r1.nv)
    assert np.array_equal(r2.eig[:km.nk], r1.eig) and np.array_equal(r2.eig[km.nk:], r1.eig)
    assert r2.efermi == pytest.approx(r1.efermi, abs=1e-12)
    assert r2.e_total == pytest.approx(r1.e_total, abs=1e-12)
    assert r2.pressure == pytest.approx(r1.pressure, abs=1e-13)
    assert r2.smag == 0.0 and r1.smag == 0.0


def test_exchanging_the_sets_reverses_the_moment(mag, km):
    npar = mag.param.size // 2
    swapped = replace(mag, param=np.concatenate([mag.param[npar:], mag.param[:npar]]))
    st = _cscl()
    a = oracle.bande(st, mag, km, _opts())
    b = oracle.bande(st, swapped, km, _opts())
    assert a.smag > 1.0
    assert b.smag == pytest.approx(-a.smag, abs=1e-12)
    assert b.efermi == pytest.approx(a.efermi, abs=1e-12)
    assert b.e_total == pytest.approx(a.e_total, abs=1e-12)
    assert np.array_equal(a.eig[:km.nk], b.eig[km.nk:])


def test_antiferromagnetic_order_has_no_moment(mag, km):
    fm = oracle.bande(_cscl(), mag, km, _opts())
    afm = oracle.bande(_cscl(flip=[0, 1]), mag, km, _opts())
    assert fm.smag == pytest.approx(2.2693, abs=1e-3)
    assert abs(afm.smag) <= 1e-12
    assert np.abs(afm.eig[:km.nk] - afm.eig[km.nk:]).max() <= 1e-13
    assert np.abs(fm.eig[:km.nk] - fm.eig[km.nk:]).max() > 0.05
    assert afm.e_total != fm.e_total


@pytest.mark.parametrize("flip", [None, [0, 1]])
def test_pressure_is_minus_dE_dV(mag, km, flip):
    par = replace(mag, dnn=np.full_like(mag.dnn, 24.0))   # no pair crosses the cut-off

    def energy(eps):
        s = (1.0 + eps) ** (1.0 / 3.0)
        return oracle.bande(_cscl(A * s, flip, 24.0), par, km, _opts(3, 1e-13)).e_total

    r0 = oracle.bande(_cscl(A, flip, 24.0), par, km, _opts(4, 1e-13))
    h = 0.0025
    dedv = (8.0 * (energy(h) - energy(-h)) - (energy(2 * h) - energy(-2 * h))) / (12.0 * h * A ** 3)
    assert abs(-dedv - r0.pressure) <= 1e-3 / 147105.08


@pytest.mark.parametrize("flip", [None, [0, 1]])
def test_fermi_level_and_moment_restated(mag, km, flip):
    st = _cscl(flip=flip)
    r = oracle.bande(st, mag, km, _opts(3, 1e-13))
    zfill = mag.zfill(st)
    w = np.concatenate([km.w, km.w])

    def count(mu):
        # fermi.f:319-342: 1 below mu - 20 kT, f inside the window, 0 above
        x = np.clip((r.eig - mu) / TKB, -700, 700)
        f = np.where(x < -20.0, 1.0, np.where(x < 20.0, 1.0 / (1.0 + np.exp(x)), 0.0))
        return float((w[:, None] * f).sum())

    assert count(r.efermi) == pytest.approx(zfill, abs=1e-9)
    # bande.f:1336-1395: per spin, weight w(k), 1 below E_F - 20 kT, f in the window
    efm, efp = r.efermi - 20 * TKB, r.efermi + 20 * TKB
    pops = []
    for js in range(2):
        e = r.eig[js * km.nk:(js + 1) * km.nk]
        occ = np.where(e < efm, 1.0, np.where(e < efp, 1.0 / (1.0 + np.exp((e - r.efermi) / TKB)), 0.0))
        pops.append(float((km.w[:, None] * occ).sum()))
    assert r.smag == pytest.approx(pops[0] - pops[1], abs=1e-12)
    assert pops[0] + pops[1] == pytest.approx(zfill, abs=1e-9)


def test_flips_need_two_sets(km):
    p1 = synth.make_params([9], [10.0], 7)
    with pytest.raises(AssertionError):
        oracle.bande(_cscl(flip=[0, 1]), p1, km, _opts())


def test_reader_magnetic_file_and_flips(tmp_path, mag, km):
    st = _cscl(flip=[0, 1])
    synth.write_skin(str(tmp_path), [(st, km)], mag, mode=4, tkb=TKB)
    head = open(os.path.join(str(tmp_path), "par")).readline()
    assert head.startswith("NM")
    sk = read_skin(os.path.join(str(tmp_path), "SKIN"))
    assert sk.params.jspins == 2
    assert np.array_equal(sk.params.param, mag.param)
    s2 = sk.structures[0][2]
    assert s2.flip is not None and s2.flip.tolist() == [0, 1]
    # the ferromagnetic form: the spin flag line stays plain, no flips
    synth.write_skin(str(tmp_path / "fm"), [(_cscl(), km)], mag, mode=4, tkb=TKB)
    s3 = read_skin(os.path.join(str(tmp_path / "fm"), "SKIN")).structures[0][2]
    assert s3.flip is None


@pytest.mark.parametrize("flag,code", [("D", "-5"), ("S", "-5"), ("N", "-5")])
def test_reader_non_collinear_flags_need_directions(tmp_path, km, flag, code):
    """The non-collinear flags N, D (torques) and S (spin directions) need a
    direction (theta, phi) on every atom line."""
    d = str(tmp_path)
    synth.write_skin(d, [(_cscl(), km)], synth.make_params([9], [10.0], 7), mode=4, tkb=TKB)
    path = os.path.join(d, "SKIN")
    lines = open(path).read().splitlines()
    i = next(j for j, ln in enumerate(lines) if ln == "F")
    lines[i] = "F" + flag
    open(path, "w").write("\n".join(lines) + "\n")
    with pytest.raises(RuntimeError, match=code):
        read_skin(path)
