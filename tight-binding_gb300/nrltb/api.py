"""Python view of the C ABI: numpy-backed structures, the SKIN reader and a
context wrapper around libnrltb_gb300.so.

Everything numeric runs in the shared library; this module only marshals
arrays.  The product path has no Python or CPU fallback: if the CUDA library is
missing, ``Context`` raises.
"""
import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

from . import abi


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None


def _iptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_int)) if a is not None else None


@dataclass
class Structure:
    """A periodic structure in Cartesian bohr (after static.f:1088-1103)."""
    kkind: np.ndarray            # (natoms,) int32, 1-based species
    posn: np.ndarray             # (natoms, 3) float64 Cartesian
    plv: np.ndarray              # (3, 3) float64, plv[i] = i-th primitive vector
    nd: tuple                    # search box half-widths
    volume: float
    zcharge: float = 0.0
    posq: np.ndarray = None      # (natoms, 3) phase offsets, default zero
    flip: np.ndarray = None      # (natoms,) nonzero = spin flipped (two-spin sets only)
    spinat: np.ndarray = None    # (natoms, 3) unit spin directions: non-collinear spins

    def __post_init__(self):
        self.kkind = np.ascontiguousarray(self.kkind, dtype=np.int32)
        self.posn = np.ascontiguousarray(self.posn, dtype=np.float64).reshape(-1, 3)
        self.plv = np.ascontiguousarray(self.plv, dtype=np.float64).reshape(3, 3)
        if self.posq is None:
            self.posq = np.zeros_like(self.posn)
        self.posq = np.ascontiguousarray(self.posq, dtype=np.float64).reshape(-1, 3)
        if self.flip is not None:
            self.flip = np.ascontiguousarray(self.flip, dtype=np.int32).reshape(-1)
        if self.spinat is not None:
            self.spinat = np.ascontiguousarray(self.spinat, dtype=np.float64).reshape(-1, 3)

    @property
    def natoms(self):
        return int(self.kkind.shape[0])

    def to_c(self):
        s = abi.Structure_()
        s.natoms = self.natoms
        s.kkind = _iptr(self.kkind)
        s.posn = _dptr(self.posn)
        s.posq = _dptr(self.posq)
        for i in range(3):
            for j in range(3):
                s.plv[i][j] = float(self.plv[i, j])
            s.nd[i] = int(self.nd[i])
        s.volume = float(self.volume)
        s.zcharge = float(self.zcharge)
        s.flip = _iptr(self.flip)
        s.spinat = _dptr(self.spinat)
        s._keep = (self,)
        return s


@dataclass
class Params:
    """An NRL parameter set (input.f): one set of kinds(29 + 68 kinds) values, or
    two (jspins = 2, a collinear spin-polarized set, spin 1 first)."""
    kinds: int
    kbas: np.ndarray
    valence: np.ndarray
    dnn: np.ndarray
    screenl: np.ndarray
    param: np.ndarray
    jsover: int = 1
    nltype: int = 0
    jspins: int = 1

    def __post_init__(self):
        self.kbas = np.ascontiguousarray(self.kbas, dtype=np.int32)
        self.valence = np.ascontiguousarray(self.valence, dtype=np.float64)
        self.dnn = np.ascontiguousarray(self.dnn, dtype=np.float64)
        self.screenl = np.ascontiguousarray(self.screenl, dtype=np.float64)
        self.param = np.ascontiguousarray(self.param, dtype=np.float64)
        assert self.param.size == self.jspins * self.kinds * (29 + 68 * self.kinds)

    def to_c(self):
        p = abi.Params_()
        p.kinds = self.kinds
        p.jsover = self.jsover
        p.nltype = self.nltype
        p.kbas = _iptr(self.kbas)
        p.valence = _dptr(self.valence)
        p.dnn = _dptr(self.dnn)
        p.screenl = _dptr(self.screenl)
        p.param = _dptr(self.param)
        p.jspins = self.jspins
        p._keep = (self,)
        return p

    def nv(self, st):
        return int(self.kbas[st.kkind - 1].sum())

    def zfill(self, st):
        return float(st.zcharge + self.valence[st.kkind - 1].sum())


@dataclass
class KMesh:
    """Explicit k list, reciprocal-lattice coordinates, weights summing to 1."""
    k: np.ndarray
    w: np.ndarray

    def __post_init__(self):
        self.k = np.ascontiguousarray(self.k, dtype=np.float64).reshape(-1, 3)
        self.w = np.ascontiguousarray(self.w, dtype=np.float64).reshape(-1)

    @property
    def nk(self):
        return int(self.k.shape[0])

    def to_c(self):
        m = abi.KMesh_()
        m.nk = self.nk
        m.k = _dptr(self.k)
        m.w = _dptr(self.w)
        m._keep = (self,)
        return m


@dataclass
class Opts:
    mode: int = 4
    precision: int = abi.PREC_FP64
    tkb: float = 0.005
    eigcut: float = 1e3
    fermi_tol: float = 0.0
    kneigh_in: int = 0
    flags: int = 0               # abi.OPT_* bits

    def to_c(self):
        o = abi.Opts_()
        o.mode, o.precision = self.mode, self.precision
        o.tkb, o.eigcut, o.fermi_tol = self.tkb, self.eigcut, self.fermi_tol
        o.kneigh_in, o.flags = self.kneigh_in, self.flags
        return o


@dataclass
class Result:
    efermi: float
    e_total: float
    pressure: float
    fermi_shift: float
    dismin: float
    npairs: int
    nv: int
    nk: int
    kneigh_out: int
    nonphysical_k: int
    eig: np.ndarray = None
    deig: np.ndarray = None
    ncut: np.ndarray = None
    k_status: np.ndarray = None
    entropy: float = 0.0
    free_energy: float = 0.0
    entropy_shift: float = 0.0
    earg1: float = 0.0
    earg2: float = 0.0
    smag: float = 0.0
    spdir: np.ndarray = None    # (natoms, 3) spin vector per atom, non-collinear runs
    orbocc: np.ndarray = None   # (jspins*nk, nv states, nv orbitals), modes 5, 6, 10


def result_shape(st, par):
    """(order of the secular equation, spin blocks of rows) of nrltb_bande's
    per-k outputs: 2N and one block for non-collinear spins, else N and jspins."""
    nv = par.nv(st)
    if st.spinat is not None:
        return 2 * nv, 1
    return nv, max(par.jspins, 1)


def new_result(nv, nk, want_eig=True, want_deig=True, jspins=1, want_orbocc=False, natoms_spdir=0):
    """Result struct with per-k arrays of jspins * nk rows (spin 1's k points
    first); want_orbocc adds the (rows, states, orbitals) Lowdin charges."""
    nrow = max(jspins, 1) * nk
    arrays = dict(eig=np.zeros((nrow, nv)) if want_eig else None,
                  deig=np.zeros((nrow, nv)) if want_deig else None,
                  ncut=np.zeros(nrow, np.int32), k_status=np.zeros(nrow, np.int32),
                  orbocc=np.zeros((nrow, nv, nv)) if want_orbocc else None,
                  spdir=np.zeros((natoms_spdir, 3)) if natoms_spdir else None)
    r = abi.Result_()
    r.eig = _dptr(arrays["eig"])
    r.deig = _dptr(arrays["deig"])
    r.orbocc = _dptr(arrays["orbocc"])
    r.spdir = _dptr(arrays["spdir"])
    r.ncut = _iptr(arrays["ncut"])
    r.k_status = _iptr(arrays["k_status"])
    r._keep = arrays
    return r, arrays


def result_from_c(r, arrays):
    return Result(r.efermi, r.e_total, r.pressure, r.fermi_shift, r.dismin, r.npairs, r.nv,
                  r.nk, r.kneigh_out, r.nonphysical_k, **arrays, entropy=r.entropy,
                  free_energy=r.free_energy, entropy_shift=r.entropy_shift, earg1=r.earg1,
                  earg2=r.earg2, smag=r.smag)


def write_qlmt(path, mode, st, par, km, eigcut, result, append=False, lib=None):
    """Append (or start) the QLMT / QAPW records of one structure through the C
    writer nrltb_qlmt_write: result is a Result with eig (and orbocc in modes 6
    and 10) for par.jspins spin blocks."""
    lib = lib or abi.load_host()
    keep = [np.ascontiguousarray(result.eig, dtype=np.float64)]
    r = abi.Result_()
    r.nv, r.nk = result.nv, result.nk
    r.eig = _dptr(keep[0])
    if result.orbocc is not None:
        keep.append(np.ascontiguousarray(result.orbocc, dtype=np.float64))
        r.orbocc = _dptr(keep[1])
    cs, cp, ck = st.to_c(), par.to_c(), km.to_c()
    rc = lib.nrltb_qlmt_write(os.fsencode(path), int(append), mode, C.byref(cs), C.byref(cp), C.byref(ck),
                              float(eigcut), C.byref(r))
    if rc != 0:
        raise RuntimeError(f"nrltb_qlmt_write returned {rc}")


def new_pairs(capacity):
    arrays = dict(tt=np.zeros((capacity, 3)), dlv=np.zeros((capacity, 3), np.int32),
                  dist=np.zeros(capacity), screen=np.zeros(capacity), dscrn=np.zeros(capacity),
                  jkind=np.zeros((capacity, 2), np.int32), jatm=np.zeros((capacity, 2), np.int32))
    p = abi.Pairs_()
    p.capacity = capacity
    p.npairs = 0
    for k, a in arrays.items():
        setattr(p, k, _iptr(a) if a.dtype == np.int32 else _dptr(a))
    p._keep = arrays
    return p, arrays


def pairs_to_c(arrays):
    """Pairs_ over existing numpy arrays (npairs = len(dist))."""
    arrays = {k: np.ascontiguousarray(v) for k, v in arrays.items()}
    p = abi.Pairs_()
    p.capacity = p.npairs = int(arrays["dist"].shape[0])
    for k, a in arrays.items():
        setattr(p, k, _iptr(a) if a.dtype == np.int32 else _dptr(a))
    p._keep = arrays
    return p


def pair_capacity(st):
    box = (2 * st.nd[0] + 1) * (2 * st.nd[1] + 1) * (2 * st.nd[2] + 1)
    return st.natoms * (st.natoms + 1) // 2 * box


# ---- SKIN reader -------------------------------------------------------------
@dataclass
class SkinFile:
    mode: int
    tkb: float
    eigcut: float
    params: Params
    structures: list = field(default_factory=list)   # (title, label, Structure, KMesh)
    spin_options: list = field(default_factory=list)  # per structure: bit 1 directions, 2 torques


def read_skin(path, lib=None):
    """Parse a SKIN file with the C readers (input.f / input1.f / setlat.f / kptin.f)."""
    lib = lib or abi.load_host()
    h = C.c_void_p()
    rc = lib.nrltb_skin_open(os.fsencode(path), C.byref(h))
    if rc != 0:
        raise RuntimeError(f"nrltb_skin_open({path}) failed: {rc}")
    try:
        mode, tkb, eigcut = C.c_int(), C.c_double(), C.c_double()
        cp = abi.Params_()
        lib.nrltb_skin_info(h, C.byref(mode), C.byref(tkb), C.byref(eigcut), C.byref(cp))
        nint = cp.kinds * (cp.kinds + 1) // 2
        npar = max(cp.jspins, 1) * cp.kinds * (29 + 68 * cp.kinds)
        params = Params(cp.kinds, np.ctypeslib.as_array(cp.kbas, (cp.kinds,)).copy(),
                        np.ctypeslib.as_array(cp.valence, (cp.kinds,)).copy(),
                        np.ctypeslib.as_array(cp.dnn, (nint,)).copy(),
                        np.ctypeslib.as_array(cp.screenl, (nint,)).copy(),
                        np.ctypeslib.as_array(cp.param, (npar,)).copy(), cp.jsover, cp.nltype,
                        max(cp.jspins, 1))
        out = SkinFile(mode.value, tkb.value, eigcut.value, params)
        while True:
            cs, ck = abi.Structure_(), abi.KMesh_()
            title, label = C.create_string_buffer(72), C.create_string_buffer(24)
            rc = lib.nrltb_skin_next(h, C.byref(cs), C.byref(ck), title, label)
            if rc == abi.NRLTB_E_EOF:
                break
            if rc != 0:
                raise RuntimeError(f"SKIN parse error {rc} at line {lib.nrltb_skin_error_line(h)}")
            n = cs.natoms
            st = Structure(np.ctypeslib.as_array(cs.kkind, (n,)).copy(),
                           np.ctypeslib.as_array(cs.posn, (n, 3)).copy(),
                           np.array([[cs.plv[i][j] for j in range(3)] for i in range(3)]),
                           tuple(cs.nd), cs.volume, cs.zcharge,
                           np.ctypeslib.as_array(cs.posq, (n, 3)).copy(),
                           np.ctypeslib.as_array(cs.flip, (n,)).copy() if cs.flip else None,
                           np.ctypeslib.as_array(cs.spinat, (n, 3)).copy() if cs.spinat else None)
            km = KMesh(np.ctypeslib.as_array(ck.k, (ck.nk, 3)).copy(),
                       np.ctypeslib.as_array(ck.w, (ck.nk,)).copy())
            out.structures.append((title.value.decode(), label.value.decode(), st, km))
            out.spin_options.append(lib.nrltb_skin_spin_options(h))
        return out
    finally:
        lib.nrltb_skin_close(h)


# ---- GPU context ---------------------------------------------------------------
class NrltbError(RuntimeError):
    """A library call returned a negative NRLTB_E_* code (``code``)."""

    def __init__(self, msg, code=None):
        super().__init__(msg)
        self.code = code


class Context:
    """One CUDA device, one stream, library-owned device buffers."""

    def __init__(self, device=0):
        self.lib = abi.load_gpu()
        h = C.c_void_p()
        rc = self.lib.nrltb_ctx_create(C.byref(h), device)
        self._check(rc, "nrltb_ctx_create")
        self.h = h

    def _check(self, rc, what):
        if rc != 0:
            raise NrltbError(f"{what} returned {rc}: {self.lib.nrltb_last_error().decode()}", rc)

    def close(self):
        if getattr(self, "h", None):
            self.lib.nrltb_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_handle):
        self._check(self.lib.nrltb_ctx_set_stream(self.h, C.c_void_p(stream_handle)), "set_stream")

    def launch_count(self):
        return int(self.lib.nrltb_ctx_launch_count(self.h))

    def bande(self, st, par, km, opts, want_eig=True, want_orbocc=None):
        (nv, nsp), nk = result_shape(st, par), km.nk
        if want_orbocc is None:
            want_orbocc = opts.mode in (5, 6, 10)
        nsd = st.natoms if (st.spinat is not None and opts.flags & abi.OPT_SPIN_DIRECTIONS) else 0
        r, arrays = new_result(nv, nk, want_eig, want_eig, nsp, want_orbocc, nsd)
        cs, cp, ck, co = st.to_c(), par.to_c(), km.to_c(), opts.to_c()
        self._check(self.lib.nrltb_bande(self.h, C.byref(cs), C.byref(cp), C.byref(ck),
                                         C.byref(co), C.byref(r)), "nrltb_bande")
        return result_from_c(r, arrays)

    def stage(self, st, par, km, opts):
        nv, nsp = result_shape(st, par)
        self._staged = (st.to_c(), par.to_c(), km.to_c(), opts.to_c(), nv, km.nk, nsp)
        cs, cp, ck, co = self._staged[:4]
        self._check(self.lib.nrltb_stage(self.h, C.byref(cs), C.byref(cp), C.byref(ck),
                                         C.byref(co)), "nrltb_stage")

    def run(self):
        self._check(self.lib.nrltb_run(self.h), "nrltb_run")

    def fetch(self, want_eig=True):
        nv, nk = self._staged[4], self._staged[5]
        r, arrays = new_result(nv, nk, want_eig, want_eig, self._staged[6])
        self._check(self.lib.nrltb_fetch(self.h, C.byref(r)), "nrltb_fetch")
        return result_from_c(r, arrays)

    def search2(self, st, par, kneigh_in=0):
        cap = pair_capacity(st)
        p, arrays = new_pairs(cap)
        kout, dmin = C.c_int(), C.c_double()
        cs, cp = st.to_c(), par.to_c()
        self._check(self.lib.nrltb_search2(self.h, C.byref(cs), C.byref(cp), kneigh_in,
                                           C.byref(p), C.byref(kout), C.byref(dmin)), "search2")
        n = p.npairs
        return {k: v[:n].copy() for k, v in arrays.items()}, kout.value, dmin.value

    def setpar(self, st, par, pairs, deriv=True):
        P = pairs["dist"].shape[0]
        cpairs = pairs_to_c(pairs)
        hop, over = np.zeros((P, 14)), np.zeros((P, 14))
        paros, den = np.zeros((st.natoms, 4)), np.zeros((st.natoms, par.kinds))
        dhop = np.zeros((P, 14)) if deriv else None
        dover = np.zeros((P, 14)) if deriv else None
        dparos = np.zeros((st.natoms, 4)) if deriv else None
        cs, cp = st.to_c(), par.to_c()
        self._check(self.lib.nrltb_setpar(self.h, C.byref(cs), C.byref(cp), C.byref(cpairs),
                                          _dptr(hop), _dptr(over), _dptr(paros), _dptr(den),
                                          _dptr(dhop), _dptr(dover), _dptr(dparos)), "setpar")
        return dict(hop=hop, over=over, paros=paros, den=den, dhop=dhop, dover=dover,
                    dparos=dparos)

    def setham(self, st, par, km, which=0):
        nv = par.nv(st)
        H = np.zeros((km.nk, nv, nv), np.complex128)
        S = np.zeros((km.nk, nv, nv), np.complex128)
        cs, cp, ck = st.to_c(), par.to_c(), km.to_c()
        self._check(self.lib.nrltb_setham(self.h, C.byref(cs), C.byref(cp), C.byref(ck), which,
                                          H.ctypes.data_as(C.POINTER(C.c_double)),
                                          S.ctypes.data_as(C.POINTER(C.c_double))), "setham")
        # column-major on the C side: element (i, j) of k at H[k, j, i]
        return H.transpose(0, 2, 1).copy(), S.transpose(0, 2, 1).copy()

    def diag(self, H, S, precision=abi.PREC_FP64, vectors=True):
        """H, S: (nk, nv, nv) complex128 (row-major numpy, Hermitian)."""
        nk, nv = H.shape[0], H.shape[1]
        Hc = np.ascontiguousarray(H.transpose(0, 2, 1))
        Sc = np.ascontiguousarray(S.transpose(0, 2, 1))
        eig = np.zeros((nk, nv))
        Z = np.zeros((nk, nv, nv), np.complex128) if vectors else None
        st = np.zeros(nk, np.int32)
        self._check(self.lib.nrltb_diag(self.h, nv, nk, Hc.ctypes.data_as(C.POINTER(C.c_double)),
                                        Sc.ctypes.data_as(C.POINTER(C.c_double)), precision,
                                        _dptr(eig),
                                        Z.ctypes.data_as(C.POINTER(C.c_double)) if vectors else None,
                                        _iptr(st)), "diag")
        if vectors:
            Z = Z.transpose(0, 2, 1).copy()
        return eig, Z, st

    def fermi(self, eig, w, tkb, zfill, tol=0.0):
        eig = np.ascontiguousarray(eig, dtype=np.float64)
        w = np.ascontiguousarray(w, dtype=np.float64)
        ef = C.c_double()
        self._check(self.lib.nrltb_fermi(self.h, eig.shape[1], eig.shape[0], _dptr(eig), _dptr(w),
                                         tkb, zfill, tol, C.byref(ef)), "fermi")
        return ef.value
