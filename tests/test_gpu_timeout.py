"""A bounded device wait that runs out reaches the caller.

The tcgen05 kernels give every barrier wait a time limit; on expiry a kernel
raises its context's expiry word and leaves its output untouched.  The word
is turned into a per-k status (NRLTB_K_TIMEOUT, the per-k error of the
reference's ioverr, diag.f:429-455) and an NRLTB_E_TIMEOUT return instead of
stale results.  No device wait is made to run out here: the test raises the
word from the host (nrltb_bench_raise_fault_word) and checks the path from
there."""
import ctypes as C

import numpy as np
import pytest

import oracle
from nrltb import KMesh, NrltbError, Opts, abi, synth

pytestmark = pytest.mark.gpu


def _sub(km, idx):
    idx = np.asarray(idx)
    return KMesh(km.k[idx], km.w[idx] / km.w[idx].sum())


def test_raised_word_fails_the_solve_with_timeout(ctx):
    st, par, km, o = synth.bcc32()
    sub = _sub(km, [0, 21])
    H, S = oracle.setham(st, par, sub)
    nk, nv = H.shape[0], H.shape[1]
    Hc = np.ascontiguousarray(H.transpose(0, 2, 1))
    Sc = np.ascontiguousarray(S.transpose(0, 2, 1))
    eig = np.zeros((nk, nv))
    status = np.zeros(nk, np.int32)
    assert ctx.lib.nrltb_bench_raise_fault_word(ctx.h) == abi.NRLTB_OK
    rc = ctx.lib.nrltb_diag(ctx.h, nv, nk, Hc.ctypes.data_as(abi._dp), Sc.ctypes.data_as(abi._dp),
                            abi.PREC_MIXED, eig.ctypes.data_as(abi._dp), None,
                            status.ctypes.data_as(C.POINTER(C.c_int)))
    assert rc == abi.NRLTB_E_TIMEOUT
    assert (status == abi.NRLTB_K_TIMEOUT).all()
    assert b"bounded device wait" in ctx.lib.nrltb_last_error()
    # the word was cleared when it was read: the same solve now succeeds
    ge, _, gst = ctx.diag(H, S, precision=abi.PREC_MIXED, vectors=False)
    assert (gst == 0).all()


@pytest.mark.parametrize("precision", [abi.PREC_MIXED, abi.PREC_FP64])
def test_raised_word_fails_bande_with_timeout(ctx, precision):
    st, par, km, o = synth.bcc32()
    sub = _sub(km, [0, 21, 42])
    opts = Opts(mode=4, precision=precision, tkb=o["tkb"], eigcut=1e3)
    assert ctx.lib.nrltb_bench_raise_fault_word(ctx.h) == abi.NRLTB_OK
    with pytest.raises(NrltbError) as ei:
        ctx.bande(st, par, sub, opts)
    assert ei.value.code == abi.NRLTB_E_TIMEOUT
    g = ctx.bande(st, par, sub, opts)
    assert (g.k_status == 0).all()
