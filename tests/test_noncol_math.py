"""The non-collinear formulas the GPU kernels evaluate (csrc/noncol_math.h:
k_noncol_onsite, k_noncol_spin_terms, k_noncol_expand call these functions),
compiled for the host with gcc and checked against the oracle's independent
restatement (oracle/nrltb_oracle.c) and against the doubled matrix written
out with numpy.  The kernels themselves are checked on the GPU by
tests/test_gpu_spin_noncollinear.py."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

import oracle
from conftest import REPO
from nrltb import Structure, synth

CSRC = os.path.join(REPO, "tight-binding_gb300", "csrc")


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("nc") / "libnc.so")
    subprocess.run(["gcc", "-std=gnu11", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-I", CSRC,
                    os.path.join(REPO, "tests", "noncol_harness.c"), "-o", so, "-lm"], check=True)
    return C.CDLL(so)


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _cell(kinds, angles):
    a = 5.6
    plv = np.eye(3) * a
    sp = np.array([[np.sin(np.radians(t)) * np.cos(np.radians(p)), np.sin(np.radians(t)) * np.sin(np.radians(p)),
                    np.cos(np.radians(t))] for t, p in angles])
    return Structure(list(kinds), [[0, 0, 0], [a / 2, a / 2, a / 2]], plv, synth.search_box(plv, 16.5), a ** 3,
                     spinat=sp)


@pytest.mark.parametrize("kbas,kinds", [([9], (1, 1)), ([9, 9], (1, 2)), ([9, 4], (1, 2)), ([4, 1], (2, 1))])
def test_onsite_matches_oracle(lib, kbas, kinds):
    par = synth.make_magnetic_params(kbas, [10.0] * len(kbas), 3, split=0.05)
    st = _cell(kinds, [(0, 0), (40, 10)])
    pairs, _, _ = oracle.search2(st, par)
    o = oracle.noncol_onsite(st, par, pairs)
    npar = par.param.size // 2
    P1, P2 = np.ascontiguousarray(par.param[:npar]), np.ascontiguousarray(par.param[npar:])
    out = {k: np.zeros((st.natoms, 4)) for k in ("paros", "spinos", "dparos", "dspnos")}
    lib.h_onsite(st.natoms, par.kinds, _p(st.kkind), _p(o["den1"]), _p(o["den2"]), _p(o["vden1"]), _p(o["vden2"]),
                 _p(P1), _p(P2), 1, _p(out["paros"]), _p(out["spinos"]), _p(out["dparos"]), _p(out["dspnos"]))
    for k in out:
        assert np.array_equal(out[k], o[k]), k


def test_spin_terms_and_doubling(lib):
    rng = np.random.default_rng(2)
    nbas = np.array([9, 4, 1], np.int32)
    nv = int(nbas.sum())
    spinos = rng.normal(size=(3, 4))
    m = rng.normal(size=(3, 3))
    m /= np.linalg.norm(m, axis=1)[:, None]
    diag, mre, mim = np.zeros(nv), np.zeros(nv), np.zeros(nv)
    lib.h_spin_terms(3, _p(nbas), _p(spinos), _p(m), _p(diag), _p(mre), _p(mim))
    # spinham.f:141-157: classes s | p p p | t2g t2g t2g | eg eg per atom
    cls = [0, 1, 1, 1, 2, 2, 2, 3, 3]
    want = []
    for a, nb in enumerate(nbas):
        for k in range(nb):
            s = spinos[a, cls[k]]
            want.append((s * m[a, 2], s * m[a, 0], s * m[a, 1]))
    want = np.array(want)
    assert np.array_equal(diag, want[:, 0]) and np.array_equal(mre, want[:, 1]) and np.array_equal(mim, want[:, 2])
    batch = 3
    H = rng.normal(size=(batch, nv, nv)) + 1j * rng.normal(size=(batch, nv, nv))
    H = H + H.conj().transpose(0, 2, 1)
    Hc = np.ascontiguousarray(H.transpose(0, 2, 1))            # column-major per matrix
    out = np.zeros((batch, 2 * nv, 2 * nv), complex)
    lib.h_expand(nv, batch, _p(Hc), _p(diag), _p(mre), _p(mim), _p(out))
    H2 = out.transpose(0, 2, 1)                                # back to row-major
    D, M = np.diag(diag), np.diag(mre + 1j * mim)
    for b in range(batch):
        ref = np.block([[H[b] + D, M], [M.conj().T, H[b] - D]])   # addspins.f:77-110
        assert np.array_equal(H2[b], ref)
    lib.h_expand(nv, batch, _p(Hc), None, None, None, _p(out))
    H2 = out.transpose(0, 2, 1)
    for b in range(batch):
        z = np.zeros((nv, nv))
        assert np.array_equal(H2[b], np.block([[H[b], z], [z, H[b]]]))
