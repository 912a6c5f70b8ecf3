"""ctypes front end of the C oracle (oracle/nrltb_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, as the checker.  The product never imports it.

The LAPACK driver the reference calls (zhpgv / zhpev, diag.f:396-412) is taken
from SciPy's bundled LAPACK through scipy.linalg.cython_lapack's exported
function pointers, so the same code works on x86_64 and aarch64 hosts.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD_DIR, "liboracle.so")
REPO = os.path.dirname(HERE)
INCLUDE = os.path.join(REPO, "include")


def build(force=False):
    """Compile the oracle with gcc (no FMA contraction, OpenMP over k)."""
    src = os.path.join(HERE, "nrltb_oracle.c")
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= os.path.getmtime(src)
            and os.path.getmtime(LIB) >= os.path.getmtime(os.path.join(INCLUDE, "nrltb.h"))):
        return LIB
    os.makedirs(BUILD_DIR, exist_ok=True)
    cmd = ["gcc", "-std=gnu11", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-I", INCLUDE, src, "-o", LIB + ".tmp", "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


_lib = None


def _capsule_ptr(cap):
    get_name = C.pythonapi.PyCapsule_GetName
    get_name.restype = C.c_char_p
    get_name.argtypes = [C.py_object]
    get_ptr = C.pythonapi.PyCapsule_GetPointer
    get_ptr.restype = C.c_void_p
    get_ptr.argtypes = [C.py_object, C.c_char_p]
    return get_ptr(cap, get_name(cap))


def load():
    global _lib
    if _lib is not None:
        return _lib
    build()
    lib = C.CDLL(LIB)
    import scipy.linalg.cython_lapack as cl
    lib.oracle_set_lapack.argtypes = [C.c_void_p, C.c_void_p]
    lib.oracle_set_lapack.restype = None
    lib.oracle_set_lapack(_capsule_ptr(cl.__pyx_capi__["zhpgv"]),
                          _capsule_ptr(cl.__pyx_capi__["zhpev"]))
    vp = C.c_void_p
    for name, args in [
        ("oracle_search2", [vp, vp, C.c_int, vp, vp, vp]),
        ("oracle_setpar", [vp, vp, vp, vp, vp, vp, vp]),
        ("oracle_setparv", [vp, vp, vp, vp, vp, vp, vp]),
        ("oracle_setham", [vp, vp, vp, C.c_int, C.c_int, vp, vp]),
        ("oracle_diag_dense", [C.c_int, C.c_int, vp, vp, vp, vp, vp]),
        ("oracle_bande", [vp, vp, vp, vp, vp, C.c_int]),
        ("oracle_ksolve_sample", [vp, vp, vp, vp, C.c_int, C.c_int, C.c_int, vp]),
        ("oracle_pair_bound", [vp]),
        ("oracle_noncol_onsite", [vp] * 11),
    ]:
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = C.c_int
    lib.oracle_fermi.argtypes = [C.c_int, C.c_int, vp, vp, C.c_double, C.c_double, C.c_double, vp]
    lib.oracle_fermi.restype = C.c_double
    _lib = lib
    return lib


def _ref(x):
    return C.cast(C.byref(x), C.c_void_p)


def _p(a):
    return a.ctypes.data if a is not None else None


def search2(st, par, kneigh_in=0):
    from nrltb import api
    lib = load()
    cs, cp = st.to_c(), par.to_c()
    cap = api.pair_capacity(st)
    p, arrays = api.new_pairs(cap)
    kout, dmin = C.c_int(), C.c_double()
    rc = lib.oracle_search2(_ref(cs), _ref(cp), kneigh_in, _ref(p), _ref(kout), _ref(dmin))
    assert rc == 0, rc
    n = p.npairs
    return {k: v[:n].copy() for k, v in arrays.items()}, kout.value, dmin.value


def setpar(st, par, pairs, deriv=True):
    from nrltb import api
    lib = load()
    cs, cp = st.to_c(), par.to_c()
    cpr = api.pairs_to_c(pairs)
    P = pairs["dist"].shape[0]
    out = dict(hop=np.zeros((P, 14)), over=np.zeros((P, 14)), paros=np.zeros((st.natoms, 4)),
               den=np.zeros((st.natoms, par.kinds)))
    lib.oracle_setpar(_ref(cs), _ref(cp), _ref(cpr), _p(out["hop"]), _p(out["over"]),
                      _p(out["paros"]), _p(out["den"]))
    if deriv:
        out.update(dhop=np.zeros((P, 14)), dover=np.zeros((P, 14)),
                   dparos=np.zeros((st.natoms, 4)))
        lib.oracle_setparv(_ref(cs), _ref(cp), _ref(cpr), _p(out["den"]), _p(out["dhop"]),
                           _p(out["dover"]), _p(out["dparos"]))
    return out


def noncol_onsite(st, par, pairs):
    """Non-collinear on-site terms: dict of both sets' densities den1, den2 and
    their volume derivatives vden1, vden2 (natoms, kinds), and paros, spinos,
    dparos, dspnos (natoms, 4)."""
    from nrltb import api
    lib = load()
    cs, cp, cpr = st.to_c(), par.to_c(), api.pairs_to_c(pairs)
    out = {k: np.zeros((st.natoms, par.kinds)) for k in ("den1", "den2", "vden1", "vden2")}
    out.update({k: np.zeros((st.natoms, 4)) for k in ("paros", "spinos", "dparos", "dspnos")})
    keys = ("den1", "den2", "vden1", "vden2", "paros", "spinos", "dparos", "dspnos")
    rc = lib.oracle_noncol_onsite(_ref(cs), _ref(cp), _ref(cpr), *[_p(out[k]) for k in keys])
    assert rc == 0, rc
    return out


def setham(st, par, km, which=0, kneigh_in=0):
    """Dense Hermitian H, S (which=0) or dH, dS (which=1): (nk, nv, nv) complex."""
    lib = load()
    nv = par.nv(st)
    H = np.zeros((km.nk, nv, nv), np.complex128)
    S = np.zeros((km.nk, nv, nv), np.complex128)
    cs, cp, ck = st.to_c(), par.to_c(), km.to_c()
    lib.oracle_setham(_ref(cs), _ref(cp), _ref(ck), which, kneigh_in, _p(H), _p(S))
    return H.transpose(0, 2, 1).copy(), S.transpose(0, 2, 1).copy()


def diag(H, S, vectors=True):
    """zhpgv on each k: H, S (nk, nv, nv) complex, row-major numpy."""
    lib = load()
    nk, nv = H.shape[0], H.shape[1]
    Hc = np.ascontiguousarray(H.transpose(0, 2, 1))
    Sc = np.ascontiguousarray(S.transpose(0, 2, 1))
    eig = np.zeros((nk, nv))
    Z = np.zeros((nk, nv, nv), np.complex128) if vectors else None
    st = np.zeros(nk, np.int32)
    lib.oracle_diag_dense(nv, nk, _p(Hc), _p(Sc), _p(eig), _p(Z), _p(st))
    if vectors:
        Z = Z.transpose(0, 2, 1).copy()
    return eig, Z, st


def fermi(eig, w, tkb, zfill, tol=0.0):
    lib = load()
    eig = np.ascontiguousarray(eig, dtype=np.float64)
    w = np.ascontiguousarray(w, dtype=np.float64)
    it = C.c_int()
    return lib.oracle_fermi(eig.shape[1], eig.shape[0], _p(eig), _p(w), tkb, zfill, tol, _ref(it))


def bande(st, par, km, opts, nthreads=0):
    from nrltb import abi, api
    lib = load()
    (nv, jsp), nk = api.result_shape(st, par), km.nk
    nsd = st.natoms if (st.spinat is not None and opts.flags & abi.OPT_SPIN_DIRECTIONS) else 0
    r, arrays = api.new_result(nv, nk, jspins=jsp, want_orbocc=opts.mode in (5, 6, 10), natoms_spdir=nsd)
    cs, cp, ck, co = st.to_c(), par.to_c(), km.to_c(), opts.to_c()
    rc = lib.oracle_bande(_ref(cs), _ref(cp), _ref(ck), _ref(co), _ref(r), nthreads)
    assert rc == 0, rc
    return api.result_from_c(r, arrays)


def ksolve_sample(st, par, km, opts, k0, k1, nthreads=0):
    """setham + zhpgv (+ sethamv + perturb in mode 4) over k in [k0, k1)."""
    lib = load()
    cs, cp, ck, co = st.to_c(), par.to_c(), km.to_c(), opts.to_c()
    eig = np.zeros((k1 - k0, par.nv(st)))
    rc = lib.oracle_ksolve_sample(_ref(cs), _ref(cp), _ref(ck), _ref(co), k0, k1, nthreads, _p(eig))
    assert rc == 0, rc
    return eig
