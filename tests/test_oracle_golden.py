"""The oracle and the host readers against the reference's own recorded run.

ex1 (Pd fcc/bcc, mode 4) is the only recorded output of the reference for this
path: SKENG prints E_F, E(T), P(T) to 9 decimals and SKOUT to full precision.
"""
import numpy as np
import pytest

import oracle
from nrltb import Opts


def test_reader_ex1_shapes(ex1):
    assert ex1.mode == 4
    assert ex1.tkb == pytest.approx(0.005)
    assert ex1.eigcut == pytest.approx(0.5)
    p = ex1.params
    assert p.kinds == 1 and p.kbas.tolist() == [9] and p.jsover == 1 and p.nltype == 0
    assert p.dnn.tolist() == [10.5] and p.screenl.tolist() == [0.5]
    assert p.param.size == 97 and p.param[0] == pytest.approx(1.38475106319)
    assert len(ex1.structures) == 18
    nks = [km.nk for (_, _, _, km) in ex1.structures]
    assert nks == [85] * 9 + [55] * 9
    for _, _, st, km in ex1.structures:
        assert km.w.sum() == pytest.approx(1.0, abs=1e-14)
        assert st.natoms == 1 and tuple(st.nd) == (4, 4, 4)


def test_reader_volumes(ex1, ex1_gold):
    for (_, label, st, _), g in zip(ex1.structures, ex1_gold["skeng"]):
        assert st.volume == pytest.approx(g[0], abs=5e-7)


def test_pair_counts_and_dismin(ex1, ex1_gold):
    for i, (_, _, st, _) in enumerate(ex1.structures):
        pairs, kout, dmin = oracle.search2(st, ex1.params)
        assert len(pairs["dist"]) == ex1_gold["npairs"][i]
        assert dmin == pytest.approx(ex1_gold["dismin"][i], rel=1e-14)


@pytest.mark.parametrize("idx", range(18))
def test_oracle_matches_skout(ex1, ex1_gold, idx):
    _, _, st, km = ex1.structures[idx]
    r = oracle.bande(st, ex1.params, km, Opts(mode=ex1.mode, tkb=ex1.tkb, eigcut=ex1.eigcut))
    # full-precision SKOUT values: the restatement reproduces them to rounding
    assert r.efermi == pytest.approx(ex1_gold["efermi"][idx], abs=1e-13)
    assert r.e_total == pytest.approx(ex1_gold["e_total"][idx], abs=1e-13)
    assert r.pressure == pytest.approx(ex1_gold["pressure"][idx], abs=1e-14)
    assert r.fermi_shift == pytest.approx(ex1_gold["fermi_shift"][idx], abs=1e-14)
    assert r.npairs == ex1_gold["npairs"][idx]
    # and the 9-decimal SKENG line
    sk = ex1_gold["skeng"][idx]
    assert abs(r.efermi - sk[1]) <= 5.01e-10
    assert abs(r.e_total - sk[2]) <= 5.01e-10
    assert abs(r.pressure - sk[3]) <= 5.01e-10


def test_oracle_fermi_insulator_and_bisection():
    # two flat bands, one filled: insulator branch (fermi.f:273-282)
    eig = np.array([[-1.0, 1.0], [-1.1, 0.9]])
    w = np.array([0.5, 0.5])
    ef = oracle.fermi(eig, w, 0.005, 2.0)
    assert ef == pytest.approx(0.5 * (-1.0 + 0.9))
    # metal: N(mu) = zfill after convergence
    rng = np.random.default_rng(1)
    eig = np.sort(rng.uniform(-1, 1, (7, 20)), axis=1)
    w = np.full(7, 1 / 7)
    ef = oracle.fermi(eig, w, 0.01, 17.3, tol=1e-12)
    f = 1 / (1 + np.exp((eig - ef) / 0.01))
    f[eig < ef - 0.2] = 1
    f[eig >= ef + 0.2] = 0
    assert 2 * (w[:, None] * f).sum() == pytest.approx(17.3, abs=1e-10)
