"""Orthogonal parameter sets ("O" in the parameter file, input.f:149-204): S is
the identity, diag.f:368-412 calls zhpev on H alone, and the volume derivative
carries no overlap term.  The oracle's path for them against numpy's
eigensolver and against -dE/dV, and the reader's handling of the flag."""
import os
from dataclasses import replace

import numpy as np
import pytest

import oracle
from nrltb import KMesh, Opts, Structure, read_skin, synth


def _case(dnn=None):
    st, par, km, o = synth.fcc1()
    idx = np.arange(0, km.nk, 97)
    km = KMesh(km.k[idx], km.w[idx] / km.w[idx].sum())
    par = replace(par, jsover=0)
    if dnn:
        par = replace(par, dnn=np.full_like(par.dnn, dnn))
    return st, par, km, o["tkb"]


def test_reader_orthogonal_flag(tmp_path):
    st, par, km, tkb = _case()
    synth.write_skin(str(tmp_path), [(st, km)], par, mode=4, tkb=tkb)
    assert open(os.path.join(str(tmp_path), "par")).readline().startswith("ON")
    sk = read_skin(os.path.join(str(tmp_path), "SKIN"))
    assert sk.params.jsover == 0
    assert np.array_equal(sk.params.param, par.param)


def test_eigenvalues_are_those_of_h(tmp_path):
    st, par, km, tkb = _case()
    r = oracle.bande(st, par, km, Opts(mode=4, tkb=tkb, eigcut=1e3))
    H, S = oracle.setham(st, par, km)
    assert np.abs(S).max() == 0.0              # no overlap matrix is built
    assert np.abs(np.linalg.eigvalsh(H) - r.eig).max() <= 1e-13
    assert r.nonphysical_k == 0


def test_overlap_parameters_are_ignored():
    st, par, km, tkb = _case()
    p2 = par.param.copy()
    nl = 17 + 40                                 # one species: 17 on-site, 10 H bonds x 4
    p2[nl:] = 0.0                                # the S bond parameters
    a = oracle.bande(st, par, km, Opts(mode=4, tkb=tkb, eigcut=1e3))
    b = oracle.bande(st, replace(par, param=p2), km, Opts(mode=4, tkb=tkb, eigcut=1e3))
    assert (a.efermi, a.e_total, a.pressure) == (b.efermi, b.e_total, b.pressure)
    assert np.array_equal(a.eig, b.eig)


def test_pressure_is_minus_dE_dV():
    # cut-off raised to 24 bohr so that no pair crosses it as the cell scales
    st0, par, km, tkb = _case(dnn=24.0)

    def scaled(eps):
        s = (1.0 + eps) ** (1.0 / 3.0)
        plv = st0.plv * s
        return Structure(st0.kkind, st0.posn * s, plv, synth.search_box(plv, 24.0), st0.volume * (1.0 + eps))

    r0 = oracle.bande(scaled(0.0), par, km, Opts(mode=4, tkb=tkb, eigcut=1e3, fermi_tol=1e-13))

    def energy(eps):
        return oracle.bande(scaled(eps), par, km, Opts(mode=3, tkb=tkb, eigcut=1e3, fermi_tol=1e-13)).e_total

    h = 0.0025
    dedv = (8.0 * (energy(h) - energy(-h)) - (energy(2 * h) - energy(-2 * h))) / (12.0 * h * st0.volume)
    assert abs(-dedv - r0.pressure) <= 1e-3 / 147105.08
