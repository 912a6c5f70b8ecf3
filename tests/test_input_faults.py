"""Host-side fault injection on the inputs (no device involved): truncated
SKIN and parameter files give an error code, never a crash, and a structure
with no electrons (zfill <= 0, where fermi.f:165 stops) is refused."""
import os
import shutil

import numpy as np
import pytest

import oracle
from conftest import GOLDEN
from nrltb import Opts, Structure, read_skin, synth


def _ex1(tmp_path):
    src = os.path.join(GOLDEN, "ex1")
    for f in os.listdir(src):
        shutil.copy(os.path.join(src, f), tmp_path / f)
    return tmp_path


def test_truncated_skin_never_crashes(tmp_path):
    d = _ex1(tmp_path)
    lines = (d / "SKIN").read_text().splitlines(keepends=True)
    seen = set()
    for cut in range(len(lines)):
        (d / "SKIN").write_text("".join(lines[:cut]))
        try:
            sk = read_skin(str(d / "SKIN"))
            seen.add(len(sk.structures))
        except RuntimeError:
            seen.add("error")
    assert "error" in seen and 17 in seen            # partial structures are refused, whole ones kept


def test_truncated_parameter_file_never_crashes(tmp_path):
    d = _ex1(tmp_path)
    full = (d / "pd_par").read_text().splitlines(keepends=True)
    outcomes = []
    for cut in range(len(full)):
        (d / "pd_par").write_text("".join(full[:cut]))
        try:
            sk = read_skin(str(d / "SKIN"))
            outcomes.append(int(np.count_nonzero(sk.params.param)))
        except RuntimeError:
            outcomes.append(None)
    # the header lines are required; a short parameter list reads with zeros (input.f:330-351)
    assert outcomes[0] is None and outcomes[-1] is not None
    assert all(o is None or o <= 97 for o in outcomes)


def test_no_electrons_is_refused():
    st, par, km, o = synth.fcc1()
    st = Structure(st.kkind, st.posn, st.plv, st.nd, st.volume, zcharge=-float(par.valence.sum()))
    with pytest.raises(AssertionError):
        oracle.bande(st, par, km, Opts(mode=3, tkb=o["tkb"]))
