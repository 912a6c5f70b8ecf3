"""ctypes mirror of include/nrltb.h and include/nrltb_input.h.

The structs here are byte-for-byte the C ABI's; the library handles returned by
``load_gpu()`` / ``load_host()`` are the in-tree shared objects built by
``nrltb.build``.  Loading the GPU library without a CUDA device is allowed (no
entry point touches the device until a context is created).
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
PKG_ROOT = os.path.dirname(HERE)                    # tight-binding_gb300/
REPO_ROOT = os.path.dirname(PKG_ROOT)
LIB_DIR = os.path.join(HERE, "_lib")
GPU_LIB = os.path.join(LIB_DIR, "libnrltb_gb300.so")
HOST_LIB = os.path.join(LIB_DIR, "libnrltb_host.so")

NRLTB_OK = 0
NRLTB_E_ARG = -1
NRLTB_E_CUDA = -2
NRLTB_E_NOMEM = -3
NRLTB_E_CAPACITY = -4
NRLTB_E_PARSE = -5
NRLTB_E_IO = -6
NRLTB_E_UNSUPPORTED = -7
NRLTB_E_EOF = -8
NRLTB_E_NODEVICE = -9
NRLTB_E_TIMEOUT = -10

NRLTB_K_OK = 0
NRLTB_K_S_NOT_PD = 1
NRLTB_K_NOT_CONVERGED = 3
NRLTB_K_TIMEOUT = 4

PREC_FP64 = 0
PREC_MIXED = 1
OPT_SPIN_DIRECTIONS = 1

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class Structure_(C.Structure):
    _fields_ = [("natoms", C.c_int), ("kkind", _ip), ("posn", _dp), ("posq", _dp),
                ("plv", (C.c_double * 3) * 3), ("nd", C.c_int * 3),
                ("volume", C.c_double), ("zcharge", C.c_double), ("flip", _ip), ("spinat", _dp)]


class Params_(C.Structure):
    _fields_ = [("kinds", C.c_int), ("jsover", C.c_int), ("nltype", C.c_int),
                ("kbas", _ip), ("valence", _dp), ("dnn", _dp), ("screenl", _dp),
                ("param", _dp), ("jspins", C.c_int)]


class KMesh_(C.Structure):
    _fields_ = [("nk", C.c_int), ("k", _dp), ("w", _dp)]


class Opts_(C.Structure):
    _fields_ = [("mode", C.c_int), ("precision", C.c_int), ("tkb", C.c_double),
                ("eigcut", C.c_double), ("fermi_tol", C.c_double), ("kneigh_in", C.c_int),
                ("flags", C.c_int)]


class Pairs_(C.Structure):
    _fields_ = [("capacity", C.c_int), ("npairs", C.c_int), ("tt", _dp), ("dlv", _ip),
                ("dist", _dp), ("screen", _dp), ("dscrn", _dp), ("jkind", _ip), ("jatm", _ip)]


class Result_(C.Structure):
    _fields_ = [("efermi", C.c_double), ("e_total", C.c_double), ("pressure", C.c_double),
                ("fermi_shift", C.c_double), ("dismin", C.c_double), ("npairs", C.c_int),
                ("nv", C.c_int), ("nk", C.c_int), ("kneigh_out", C.c_int),
                ("nonphysical_k", C.c_int), ("eig", _dp), ("deig", _dp), ("ncut", _ip),
                ("k_status", _ip), ("entropy", C.c_double), ("free_energy", C.c_double),
                ("entropy_shift", C.c_double), ("earg1", C.c_double), ("earg2", C.c_double),
                ("smag", C.c_double), ("spdir", _dp), ("orbocc", _dp)]


_vp = C.c_void_p
_sp = C.POINTER(Structure_)
_pp = C.POINTER(Params_)
_kp = C.POINTER(KMesh_)
_op = C.POINTER(Opts_)
_rp = C.POINTER(Result_)
_prp = C.POINTER(Pairs_)

# (name, restype, argtypes) for every entry point of include/nrltb.h
GPU_SYMBOLS = [
    ("nrltb_abi_version", C.c_int, []),
    ("nrltb_last_error", C.c_char_p, []),
    ("nrltb_ctx_create", C.c_int, [C.POINTER(_vp), C.c_int]),
    ("nrltb_ctx_destroy", C.c_int, [_vp]),
    ("nrltb_ctx_set_stream", C.c_int, [_vp, _vp]),
    ("nrltb_ctx_launch_count", C.c_longlong, [_vp]),
    ("nrltb_bande", C.c_int, [_vp, _sp, _pp, _kp, _op, _rp]),
    ("nrltb_bande_batch", C.c_int, [_vp, C.c_int, _sp, _pp, _kp, _op, _rp]),
    ("nrltb_stage", C.c_int, [_vp, _sp, _pp, _kp, _op]),
    ("nrltb_run", C.c_int, [_vp]),
    ("nrltb_fetch", C.c_int, [_vp, _rp]),
    ("nrltb_search2", C.c_int, [_vp, _sp, _pp, C.c_int, _prp, _ip, _dp]),
    ("nrltb_setpar", C.c_int, [_vp, _sp, _pp, _prp, _dp, _dp, _dp, _dp, _dp, _dp, _dp]),
    ("nrltb_setham", C.c_int, [_vp, _sp, _pp, _kp, C.c_int, _dp, _dp]),
    ("nrltb_diag", C.c_int, [_vp, C.c_int, C.c_int, _dp, _dp, C.c_int, _dp, _dp, _ip]),
    ("nrltb_fermi", C.c_int, [_vp, C.c_int, C.c_int, _dp, _dp, C.c_double, C.c_double,
                              C.c_double, _dp]),
    ("nrltb_sums", C.c_int, [_vp, C.c_int, C.c_int, _dp, _dp, _dp, C.c_int, C.c_double, C.c_double,
                             C.c_double, C.c_double, _dp]),
    ("nrltb_search2_noalloc", C.c_int, [C.c_int, _vp, C.c_int, _vp, _vp, _dp, _ip, C.c_int, _dp, _dp,
                                        C.c_int, C.c_int, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _ip, _ip, _dp]),
    # measurement hooks (include/nrltb_bench.h)
    ("nrltb_bench_peak", C.c_int, [_vp, C.c_int, _dp]),
    ("nrltb_bench_zgemm", C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_int, _dp, _dp]),
    ("nrltb_bench_refprod", C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_int, _dp, _dp]),
    ("nrltb_bench_refprod_run", C.c_int, [_vp, C.c_int, C.c_int, C.c_int, _vp, _vp, _vp]),
    ("nrltb_bench_kernel_timing", C.c_int, [_vp, C.c_int]),
    ("nrltb_bench_kernel_stats", C.c_int, [_vp, C.c_int, _dp, _dp, C.POINTER(C.c_int)]),
    ("nrltb_bench_cgemm_run", C.c_int, [_vp] + [C.c_int] * 9 + [_vp, _vp, _vp, C.c_int, _vp, C.c_int, _vp,
                                                                  C.c_int]),
    ("nrltb_bench_umma_fault", C.c_int, [C.c_int]),
    ("nrltb_bench_raise_fault_word", C.c_int, [_vp]),
]

HOST_SYMBOLS = [
    ("nrltb_skin_open", C.c_int, [C.c_char_p, C.POINTER(_vp)]),
    ("nrltb_skin_info", C.c_int, [_vp, _ip, _dp, _dp, _pp]),
    ("nrltb_skin_next", C.c_int, [_vp, _sp, _kp, C.c_char_p, C.c_char_p]),
    ("nrltb_skin_error_line", C.c_int, [_vp]),
    ("nrltb_skin_spin_options", C.c_int, [_vp]),
    ("nrltb_skin_close", None, [_vp]),
    ("nrltb_parfile_read", C.c_int, [C.c_char_p, C.POINTER(_vp), _pp]),
    ("nrltb_parfile_close", None, [_vp]),
    ("nrltb_nparams", C.c_int, [C.c_int]),
    ("nrltb_qlmt_write", C.c_int, [C.c_char_p, C.c_int, C.c_int, _sp, _pp, _kp, C.c_double, _rp]),
]

_cache = {}


def _bind(path, symbols):
    if path in _cache:
        return _cache[path]
    if not os.path.exists(path):
        raise OSError(f"{os.path.basename(path)} is not built (run nrltb.build.build_all())")
    lib = C.CDLL(path)
    for name, res, args in symbols:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _cache[path] = lib
    return lib


def load_gpu():
    """The CUDA library (libnrltb_gb300.so): the product path.  Raises if absent."""
    return _bind(GPU_LIB, GPU_SYMBOLS + HOST_SYMBOLS)


def load_host():
    """Host-only readers (libnrltb_host.so), usable without CUDA."""
    return _bind(HOST_LIB, HOST_SYMBOLS)
