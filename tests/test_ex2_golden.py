"""The readers, search2 and the k-mesh generator against the reference's ex2 run
(Ti hcp from the (V, c/a) lattice form, two atoms, spd, a space-group file in
lattice coordinates).

The recorded SKOUT stops at the first structure's k mesh: the SKIN file is read
with blank='zero' (static.f:682), so the mesh line "12   12   12" under (5I5)
becomes 12000 divisions per axis and kptgen.f stops at its array bound.  The C
reader reads the line the same way and refuses the mesh with
NRLTB_E_UNSUPPORTED; with the line right-justified (12 divisions) the rest of
the file reads, and structure 1 is checked against what SKOUT recorded.
"""
import json
import os
import shutil

import numpy as np
import pytest

import kptgen as okpt
import oracle
from conftest import GOLDEN
from nrltb import read_skin

SRC = os.path.join(GOLDEN, "ex2")


@pytest.fixture(scope="module")
def gold():
    with open(os.path.join(GOLDEN, "ex2_golden.json")) as f:
        return json.load(f)


def _copy(dirname, right_justify):
    os.makedirs(dirname, exist_ok=True)
    for f in ("SKIN", "ti_par", "spcgp1.hcp"):
        shutil.copy(os.path.join(SRC, f), os.path.join(dirname, f))
    if right_justify:
        path = os.path.join(dirname, "SKIN")
        text = open(path).read().replace("\n12   12   12 ", "\n   12   12   12")
        open(path, "w").write(text)
    return os.path.join(dirname, "SKIN")


@pytest.fixture(scope="module")
def ex2(tmp_path_factory):
    return read_skin(_copy(str(tmp_path_factory.mktemp("ex2")), True))


def test_verbatim_mesh_line_is_refused(tmp_path, gold):
    # 12000 divisions per axis, as the reference read them
    assert gold["kdiv_as_read"] == [12000] * 3
    with pytest.raises(Exception, match=r"-7 at line 21"):
        read_skin(_copy(str(tmp_path), False))


def test_all_structures_read(ex2):
    assert ex2.mode == 3 and ex2.tkb == pytest.approx(0.005) and ex2.eigcut == pytest.approx(0.5)
    p = ex2.params
    assert p.kinds == 1 and p.kbas.tolist() == [9] and p.jsover == 1
    assert p.dnn.tolist() == [16.5] and p.screenl.tolist() == [0.5]
    assert len(ex2.structures) == 13
    for j, (_, label, st, km) in enumerate(ex2.structures):
        ca = 1.30 + 0.05 * j
        assert label.split() == ["hcp", "%.2f" % ca]
        assert st.natoms == 2 and st.volume == pytest.approx(238.0, rel=1e-13)
        c = st.plv[2][2]
        a = np.linalg.norm(st.plv[0])
        assert c / a == pytest.approx(ca, rel=1e-13)
        assert km.w.sum() == pytest.approx(1.0, abs=1e-14)


def test_structure1_geometry(ex2, gold):
    _, _, st, _ = ex2.structures[0]
    assert np.abs(np.array(st.plv) - np.array(gold["plv"])).max() <= 5.01e-7
    assert st.volume == pytest.approx(gold["volume"], rel=1e-14)
    assert np.abs(np.array(st.posn) - np.array(gold["cartesian"])).max() <= 5.01e-8
    assert ex2.params.nv(st) == gold["nv"]
    zfill = st.zcharge + sum(ex2.params.valence[k - 1] for k in st.kkind)
    assert zfill == gold["electrons"]


def test_structure1_pairs_and_minimum_distance(ex2, gold):
    _, _, st, _ = ex2.structures[0]
    pairs, _, dmin = oracle.search2(st, ex2.params)
    assert len(pairs["dist"]) == gold["npairs"]
    assert dmin == pytest.approx(gold["dismin"], rel=1e-14)


def test_structure1_reciprocal_lattice(ex2, gold):
    _, _, st, _ = ex2.structures[0]
    _, bvec, bij, _ = okpt.recip(np.array(st.plv, float).tolist())
    b = np.array(bvec)
    assert np.abs(b.T - np.array(gold["recip"])).max() <= 5.01e-7
    np.testing.assert_allclose(np.array(bij), np.array(gold["metric"]), rtol=1e-7, atol=1e-12)


def test_hex_mesh_matches_restatement(ex2):
    # LATTIC=4 with the space group in lattice coordinates (ILAT=T), 12^3 mesh
    _, _, st, km = ex2.structures[0]
    plv = np.array(st.plv, float)
    q, w, _ = okpt.kptin_mesh(plv, 4, os.path.join(SRC, "spcgp1.hcp"), True, (12, 12, 12))
    assert np.array_equal(km.k, q) and np.array_equal(km.w, w)
    assert w.sum() == pytest.approx(1.0, abs=1e-14)
