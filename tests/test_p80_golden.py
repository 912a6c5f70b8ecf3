"""The readers against the reference's P80 example (carbon, 24-atom bcc cell,
new-style overlap parameters, mode 9, a 999 k path).

The recorded SKOUT stops where the first atom line is read: the SKIN file
has a comment line there that list-directed input cannot read as an integer.
The C reader stops at the same line.  With that line removed, the rest reads,
and what SKOUT recorded -- the parameter file as read, the bcc lattice, the
volume -- is checked, together with the 999 path's points and weights
(kptin.f:223-256: KD equally spaced points per segment, every weight equal
to the number of points)."""
import json
import os
import shutil

import numpy as np
import pytest

import oracle
from conftest import GOLDEN
from nrltb import Opts, read_skin

SRC = os.path.join(GOLDEN, "P80")


@pytest.fixture(scope="module")
def gold():
    with open(os.path.join(GOLDEN, "p80_golden.json")) as f:
        return json.load(f)


def _copy(dirname, drop_comment):
    os.makedirs(dirname, exist_ok=True)
    for f in ("SKIN", "C_par", "spcgrp.bcc"):
        shutil.copy(os.path.join(SRC, f), os.path.join(dirname, f))
    path = os.path.join(dirname, "SKIN")
    if drop_comment:
        lines = open(path).read().splitlines()
        lines = [ln for ln in lines if not ln.strip().startswith("(Position of atom")]
        open(path, "w").write("\n".join(lines) + "\n")
    return path


@pytest.fixture(scope="module")
def p80(tmp_path_factory):
    return read_skin(_copy(str(tmp_path_factory.mktemp("p80")), True))


def test_verbatim_stops_at_the_first_atom_line(tmp_path):
    with pytest.raises(RuntimeError, match=r"-5 at line 13"):
        read_skin(_copy(str(tmp_path), False))


def test_parameter_file_as_recorded(p80, gold):
    assert p80.mode == gold["mode"] == 9
    assert p80.tkb == pytest.approx(gold["tkb"]) and p80.eigcut == pytest.approx(gold["eigcut"])
    p = p80.params
    assert p.kinds == 1 and p.jspins == 1 and p.jsover == 1 and gold["non_orthogonal"] and gold["spin_restricted"]
    assert p.nltype == 1 and gold["new_overlap"]          # "NN00001": the real-overlap form
    assert p.kbas.tolist() == [gold["kbas"]] == [4]
    assert p.dnn.tolist() == [gold["dnn"]] and p.screenl.tolist() == [gold["screenl"]]
    # SKOUT prints 10 significant digits
    np.testing.assert_allclose(p.param, gold["params"], rtol=5.1e-10, atol=1e-300)


def test_structure_and_k_path(p80, gold):
    _, label, st, km = p80.structures[0]
    assert label.split() == ["bcc", "equilibrium"]
    assert st.natoms == gold["natoms"] == 24
    assert np.abs(np.array(st.plv) - np.array(gold["plv"])).max() <= 5.01e-7
    assert st.volume == pytest.approx(gold["volume"], rel=1e-14)
    # 7 segments of 41 points, each point weighted by the number of points
    assert km.nk == 287 and (km.w == 287.0).all()
    ends = [((0, 0, 0), (0.5, -0.5, 0.5)), ((0.5, -0.5, 0.5), (0.25, 0.25, 0.25)), ((0.25, 0.25, 0.25), (0, 0, 0)),
            ((0, 0, 0), (0, 0, 0.5)), ((0, 0, 0.5), (0.25, 0.25, 0.25)), ((0.25, 0.25, 0.25), (0.5, 0.5, 0)),
            ((0.5, 0.5, 0), (0.5, 0.5, 0.5))]
    for s, (a, b) in enumerate(ends):
        seg = km.k[41 * s:41 * (s + 1)]
        np.testing.assert_allclose(seg[0], a, atol=0)
        np.testing.assert_allclose(seg[-1], b, atol=1e-14)
        np.testing.assert_allclose(np.diff(seg, axis=0), np.tile((np.array(b) - a) / 40.0, (40, 1)), atol=1e-15)


def test_oracle_runs_mode_9(p80):
    _, _, st, km = p80.structures[0]
    sub = type(km)(km.k[::41], km.w[::41])
    r = oracle.bande(st, p80.params, sub, Opts(mode=9, tkb=p80.tkb, eigcut=p80.eigcut))
    assert r.nv == 96 and r.nonphysical_k == 0 and np.isfinite(r.eig).all()
