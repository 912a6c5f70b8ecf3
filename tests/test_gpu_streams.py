"""The mixed form on a caller's stream.  A context forks independent work onto
its internal streams (the refinement's digits and the dH, dS Bloch sums during
the tridiagonalisation, the back-transform's WY factors during the tridiagonal
solve, the rotated residuals outside clusters beside the cluster solves) and
joins it back with events to whatever stream the context runs on.  A call on a
caller's stream must therefore give bit for bit the results of the same call
on the context's own stream, before and after."""
import numpy as np
import pytest

from nrltb import Context, KMesh, Opts, abi, synth

pytestmark = pytest.mark.gpu


def _sub(km, idx):
    idx = np.asarray(idx)
    return KMesh(km.k[idx], km.w[idx] / km.w[idx].sum())


def _same(a, b):
    assert np.array_equal(a.eig, b.eig)
    assert np.array_equal(a.k_status, b.k_status)
    assert a.efermi == b.efermi
    assert a.e_total == b.e_total
    assert a.pressure == b.pressure


def test_mixed_on_caller_stream_is_bit_identical():
    torch = pytest.importorskip("torch")
    st, par, km, o = synth.bcc32()
    km4 = _sub(km, [0, 21, 42, 63])
    opts = Opts(mode=4, precision=abi.PREC_MIXED, tkb=o["tkb"], eigcut=1e3, fermi_tol=1e-11)
    c = Context(0)
    try:
        own = c.bande(st, par, km4, opts)
        s = torch.cuda.Stream()
        c.set_stream(s.cuda_stream)
        on_caller = c.bande(st, par, km4, opts)
        again = c.bande(st, par, km4, opts)
        c.set_stream(0)
        back = c.bande(st, par, km4, opts)
    finally:
        c.close()
    assert (own.k_status == 0).all()
    _same(own, on_caller)
    _same(own, again)
    _same(own, back)
