"""The eigensolver's FP32 complex GEMM on the tensor cores (3xTF32) against a
float64 product of the same masked operands, over every op / triangle form
the solver uses, on ragged sizes.  Bound: 2^-20 (|alpha| |op(A)| |op(B)| +
|beta| |C|) per element for the SIMT FP32 kernel, 2^-18 for the tensor-core
kernels (3xTF32 with FP32 accumulation in the tensor cores; both the tcgen05
and the mma.sync kernel measure 1.3e-6 at k = 333); elements whose bound is 0
must be exact.  Methods: 1 the library's dispatch, 2 SIMT, 3 the tcgen05
kernel (op(A) = A), 4 the mma.sync tensor-core kernel."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _op(M, op):
    return M.conj().T if op else M


def _tri_mask_a(m, k, tri):
    i, j = np.arange(m)[:, None], np.arange(k)[None, :]   # element (m, k) of op(A)
    return np.ones((m, k), bool) if tri == 0 else (j <= i if tri == 1 else j >= i)


def _tri_mask_b(k, n, tri):
    i, j = np.arange(k)[:, None], np.arange(n)[None, :]   # element (k, n) of op(B)
    return np.ones((k, n), bool) if tri == 0 else (i <= j if tri == 1 else i >= j)


def _run(ctx, method, m, n, k, opA, opB, triA, triB, triC, alpha, beta, seed):
    rng = np.random.default_rng(seed)
    cplx = lambda r, c: (rng.standard_normal((r, c)) + 1j * rng.standard_normal((r, c))).astype(np.complex64)
    A = cplx(k, m) if opA else cplx(m, k)
    B = cplx(n, k) if opB else cplx(k, n)
    C0 = cplx(m, n)
    Af, Bf, Cf = (np.asfortranarray(x) for x in (A, B, C0.copy()))
    al = (C.c_float * 2)(alpha.real, alpha.imag)
    be = (C.c_float * 2)(beta.real, beta.imag)
    rc = ctx.lib.nrltb_bench_cgemm_run(ctx.h, method, m, n, k, opA, opB, triA, triB, triC, al, be,
                                       Af.ctypes.data_as(C.c_void_p), A.shape[0], Bf.ctypes.data_as(C.c_void_p),
                                       B.shape[0], Cf.ctypes.data_as(C.c_void_p), m)
    assert rc == 0, ctx.lib.nrltb_last_error()
    oA = _op(A.astype(np.complex128), opA) * _tri_mask_a(m, k, triA)
    oB = _op(B.astype(np.complex128), opB) * _tri_mask_b(k, n, triB)
    ref = alpha * (oA @ oB) + beta * C0.astype(np.complex128)
    bound = abs(alpha) * (np.abs(oA) @ np.abs(oB)) + abs(beta) * np.abs(C0)
    # triC: only tiles touching the requested triangle are guaranteed
    i, j = np.arange(m)[:, None], np.arange(n)[None, :]
    sel = np.ones((m, n), bool) if triC == 0 else (i >= j if triC == 1 else i <= j)
    err, bnd = np.abs(Cf - ref)[sel], bound[sel]
    ratio = np.where(bnd > 0, err / np.where(bnd > 0, bnd, 1.0), np.where(err == 0, 0.0, np.inf))
    return ratio.max()


CASES = [
    # m, n, k, opA, opB, triA, triB, triC
    (150, 77, 93, 0, 0, 0, 0, 0),
    (150, 77, 93, 1, 0, 0, 0, 0),
    (150, 77, 93, 0, 1, 0, 0, 0),
    (150, 77, 93, 1, 1, 0, 0, 0),
    (130, 130, 130, 0, 0, 1, 0, 0),
    (130, 130, 130, 0, 0, 2, 0, 0),
    (130, 130, 130, 1, 0, 2, 0, 0),
    (130, 130, 130, 0, 1, 0, 1, 0),
    (130, 130, 130, 0, 0, 0, 2, 1),
    (200, 200, 32, 0, 1, 0, 0, 1),
    (200, 200, 32, 1, 0, 0, 0, 2),
    (33, 1, 250, 1, 0, 0, 0, 0),
    (1, 1, 1, 0, 0, 0, 0, 0),
    # several 128 x 64 tiles and 32-deep k slices
    (300, 200, 333, 0, 0, 0, 0, 0),
    (256, 130, 256, 0, 0, 2, 0, 0),
    (256, 256, 200, 0, 0, 0, 2, 1),
    (257, 100, 161, 0, 0, 1, 0, 0),
    (129, 65, 1, 0, 0, 0, 0, 0),
    # long K (8 or more 32-deep slices): the two-stage tcgen05 form, odd and even
    # slice counts, triangles that cut some tiles' slices to one or none
    (300, 130, 520, 0, 1, 0, 0, 0),
    (200, 150, 450, 0, 0, 2, 0, 0),
    (256, 192, 512, 0, 0, 0, 1, 0),
    (130, 300, 257, 0, 0, 1, 0, 2),
    # rank-32 / 64 updates with op(B) = B^H (Cholesky and tridiagonal trailing updates)
    (300, 300, 64, 0, 1, 0, 0, 1),
    (256, 200, 32, 0, 1, 0, 0, 0),
    (260, 130, 96, 0, 1, 0, 1, 0),
]


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("method", [1, 2, 3, 4])
def test_cgemm_forms(ctx, case, method):
    m, n, k, opA, opB, triA, triB, triC = case
    if method == 3 and opA:
        pytest.skip("the tcgen05 kernel takes op(A) = A")
    ctx.lib.nrltb_bench_umma_fault(1)
    for alpha, beta, seed in ((1 + 0j, 0j, 1), (-0.5 + 0.25j, 1 + 0j, 2)):
        r = _run(ctx, method, m, n, k, opA, opB, triA, triB, triC, alpha, beta, seed)
        assert r <= 2.0 ** (-20 if method == 2 else -18), (case, method, r)
    assert ctx.lib.nrltb_bench_umma_fault(0) == 0
