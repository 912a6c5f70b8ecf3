"""nrltb_bande refuses a structure with no electrons (zfill <= 0, where
fermi.f:165 stops) before any device work, with NRLTB_E_ARG and a message."""
import pytest

from nrltb import NrltbError, Opts, Structure, synth

pytestmark = pytest.mark.gpu


def test_no_electrons_is_refused(ctx):
    st, par, km, o = synth.fcc1()
    st = Structure(st.kkind, st.posn, st.plv, st.nd, st.volume, zcharge=-float(par.valence.sum()))
    with pytest.raises(NrltbError, match="zfill"):
        ctx.bande(st, par, km, Opts(mode=3, tkb=o["tkb"]))
    st_ok = Structure(st.kkind, st.posn, st.plv, st.nd, st.volume)
    r = ctx.bande(st_ok, par, km, Opts(mode=3, tkb=o["tkb"]))   # the context stays usable
    assert r.nv == par.nv(st_ok)
