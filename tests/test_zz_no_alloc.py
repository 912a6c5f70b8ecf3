"""nrltb_search2_noalloc: the neighbour list for callers that cannot allocate
device memory (their own allocator owns the GPU, or a cudaMalloc would stall
their pipeline).  Checked against the allocating entry point nrltb_search2,
twice in a row, since every call reuses the same fixed scratch array.

This file is collected last on purpose: if it fails, a run that stops at the
first failure has already run every other test."""
import ctypes as C

import numpy as np
import pytest

from nrltb import abi, synth

pytestmark = pytest.mark.gpu


def _noalloc(lib, st, par, capacity, stream, kneigh_in=0):
    import torch
    dev = torch.device("cuda", 0)
    kk = torch.from_numpy(st.kkind.copy()).to(dev)
    pos = torch.from_numpy(st.posn.copy()).to(dev)
    out = dict(tt=torch.zeros((capacity, 3), dtype=torch.float64, device=dev),
               dlv=torch.zeros((capacity, 3), dtype=torch.int32, device=dev),
               dist=torch.zeros(capacity, dtype=torch.float64, device=dev),
               screen=torch.zeros(capacity, dtype=torch.float64, device=dev),
               dscrn=torch.zeros(capacity, dtype=torch.float64, device=dev),
               jkind=torch.zeros((capacity, 2), dtype=torch.int32, device=dev),
               jatm=torch.zeros((capacity, 2), dtype=torch.int32, device=dev))
    torch.cuda.synchronize()
    plv = (C.c_double * 9)(*st.plv.reshape(-1))
    nd = (C.c_int * 3)(*st.nd)
    npairs, kout, dmin = C.c_int(), C.c_int(), C.c_double()
    rc = lib.nrltb_search2_noalloc(
        0, C.c_void_p(stream), st.natoms, C.c_void_p(kk.data_ptr()), C.c_void_p(pos.data_ptr()),
        C.cast(plv, abi._dp), C.cast(nd, abi._ip), par.kinds, par.dnn.ctypes.data_as(abi._dp),
        par.screenl.ctypes.data_as(abi._dp), kneigh_in, capacity,
        *[C.c_void_p(out[k].data_ptr()) for k in ("tt", "dlv", "dist", "screen", "dscrn", "jkind", "jatm")],
        C.byref(npairs), C.byref(kout), C.byref(dmin))
    res = {k: v[:npairs.value].cpu().numpy() for k, v in out.items()}
    return rc, res, npairs.value, kout.value, dmin.value


def test_search2_noalloc_matches_allocating_entry_point(ctx):
    import torch
    lib = abi.load_gpu()
    stream = torch.cuda.current_stream().cuda_stream
    for st, par in (synth.bcc32()[:2], synth.fcc128()[:2], synth.b2_216()[:2]):
        ref, rk, rd = ctx.search2(st, par)
        n = len(ref["dist"])
        for _ in range(2):                       # two calls in a row share the scratch array
            rc, got, npairs, kout, dmin = _noalloc(lib, st, par, n + 16, stream)
            assert rc == abi.NRLTB_OK
            assert npairs == n and kout == rk and dmin == rd
            for key in ("dlv", "jkind", "jatm"):
                assert np.array_equal(got[key], ref[key]), key
            np.testing.assert_array_equal(got["dist"], ref["dist"])
            np.testing.assert_array_equal(got["tt"], ref["tt"])
            np.testing.assert_allclose(got["screen"], ref["screen"], rtol=1e-14, atol=0)
            np.testing.assert_allclose(got["dscrn"], ref["dscrn"], rtol=1e-13, atol=1e-300)


def test_search2_noalloc_limits():
    import torch
    lib = abi.load_gpu()
    stream = torch.cuda.current_stream().cuda_stream
    st, par = synth.fcc128()[:2]
    # too small an output: full count reported, NRLTB_E_CAPACITY returned
    rc, got, npairs, _, _ = _noalloc(lib, st, par, 100, stream)
    assert rc == abi.NRLTB_E_CAPACITY and npairs > 100
    # a search box beyond the fixed scratch is rejected before any device work
    big = synth.Structure(st.kkind, st.posn, st.plv, (30, 30, 30), st.volume)
    rc, _, _, _, _ = _noalloc(lib, big, par, 1, stream)
    assert rc == abi.NRLTB_E_CAPACITY
    assert b"no-allocation path takes at most" in lib.nrltb_last_error()
    # an atom kind outside 1..kinds is refused before the search reads it
    bad = synth.Structure(st.kkind.copy(), st.posn, st.plv, st.nd, st.volume)
    bad.kkind[5] = par.kinds + 1
    rc, _, _, _, _ = _noalloc(lib, bad, par, 1, stream)
    assert rc == abi.NRLTB_E_ARG
    assert b"outside 1.." in lib.nrltb_last_error()
    # and the next well-formed call is unaffected
    ref_rc, _, npairs, _, _ = _noalloc(lib, st, par, 1, stream)
    assert ref_rc == abi.NRLTB_E_CAPACITY and npairs > 1
