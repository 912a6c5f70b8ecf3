"""Mixed-precision form (FP32 eigensolve + FP64-accurate refinement) against the
FP64 oracle.  Tolerances: eigenvalues 1e-9 Ry, E_F 1e-9 Ry, E_total 1e-8 Ry/atom,
pressure 1e-3 kbar (6.8e-9 Ry/bohr^3).

Eigenvectors: each z_j is S-normalised to 1e-9 (z_j^H S z_j = 1 is what the
orbital charges sum to), and distinct eigenvectors are S-orthogonal to 1e-7.
The off-diagonal bound is the refinement's: its two FP32 products X'^H r' and
X' E run on the tensor cores, whose FP32 accumulation truncates, and an error
of ~1e-12 in a residual projection divided by a gap of ~1e-4 Ry leaves
~1e-8 between near-degenerate states (no output of the path depends on the
off-diagonal)."""
import numpy as np
import pytest

import oracle
from nrltb import KMesh, Opts, abi, synth

pytestmark = pytest.mark.gpu

KBAR = 1.0 / 147105.08
P_TOL = 1e-3 * KBAR
MIXED = abi.PREC_MIXED


def _sub(km, idx):
    idx = np.asarray(idx)
    return KMesh(km.k[idx], km.w[idx] / km.w[idx].sum())


def _check(ctx, H, S):
    ge, gz, gst = ctx.diag(H, S, precision=MIXED)
    oe, _, ost = oracle.diag(H, S, vectors=False)
    assert (gst == 0).all() and (ost == 0).all(), gst
    err = np.abs(ge - oe).max()
    assert err <= 1e-9, err
    for k in range(H.shape[0]):
        Z = gz[k]
        res = H[k] @ Z - (S[k] @ Z) * ge[k][None, :]
        assert np.abs(res).max() < 1e-6
        gram = Z.conj().T @ S[k] @ Z - np.eye(Z.shape[1])
        assert np.abs(np.diag(gram)).max() <= 1e-9, np.abs(np.diag(gram)).max()
        assert np.abs(gram).max() <= 1e-7, np.abs(gram).max()
    return err


def test_mixed_diag_n9(ctx, ex1):
    st, par, km = ex1.structures[0][2], ex1.params, ex1.structures[0][3]
    H, S = oracle.setham(st, par, km)
    _check(ctx, H, S)


def test_mixed_diag_n288(ctx):
    st, par, km, _ = synth.bcc32()
    H, S = oracle.setham(st, par, _sub(km, [0, 21, 42]))
    _check(ctx, H, S)


def test_mixed_diag_n1152(ctx):
    st, par, km, _ = synth.fcc128()
    H, S = oracle.setham(st, par, _sub(km, [0, 13]))
    _check(ctx, H, S)


def test_mixed_diag_n1404_two_species(ctx):
    st, par, km, _ = synth.b2_216()
    H, S = oracle.setham(st, par, _sub(km, [0]))
    _check(ctx, H, S)


def test_mixed_diag_degenerate(ctx):
    rng = np.random.default_rng(7)
    A = rng.normal(size=(8, 8)) + 1j * rng.normal(size=(8, 8))
    A = A + A.conj().T
    H = np.zeros((1, 32, 32), complex)
    for b in range(4):
        H[0, 8 * b:8 * b + 8, 8 * b:8 * b + 8] = A
    S = np.eye(32)[None].astype(complex)
    _check(ctx, H, S)


def _compare(ctx, st, par, km, tkb):
    opts_m = Opts(mode=4, precision=MIXED, tkb=tkb, eigcut=1e3, fermi_tol=1e-11)
    opts_o = Opts(mode=4, tkb=tkb, eigcut=1e3, fermi_tol=1e-11)
    g = ctx.bande(st, par, km, opts_m)
    o = oracle.bande(st, par, km, opts_o)
    assert (g.k_status == 0).all()
    assert np.abs(g.eig - o.eig).max() <= 1e-9
    assert abs(g.efermi - o.efermi) <= 1e-9
    assert abs(g.e_total - o.e_total) / st.natoms <= 1e-8
    assert abs(g.pressure - o.pressure) <= P_TOL
    return g, o


def test_mixed_bande_fcc1(ctx):
    st, par, km, o = synth.fcc1()
    _compare(ctx, st, par, km, o["tkb"])


def test_mixed_bande_bcc32(ctx):
    st, par, km, o = synth.bcc32()
    _compare(ctx, st, par, _sub(km, [0, 21, 42, 63]), o["tkb"])


def test_mixed_bande_fcc128_two_k(ctx):
    st, par, km, o = synth.fcc128()
    _compare(ctx, st, par, _sub(km, [0, 13]), o["tkb"])


def test_mixed_bande_fcc128_full_mesh(ctx):
    """The benchmarked step itself: fcc128 (N = 1152), all 27 k of the 3x3x3
    mesh, mode 4, mixed form against the oracle (the oracle's 27 solves take
    tens of seconds on the host cores)."""
    st, par, km, o = synth.fcc128()
    g, oo = _compare(ctx, st, par, km, o["tkb"])
    assert g.eig.shape == (27, 1152)


def test_mixed_batch_matches_single_calls_and_oracle(ctx):
    """The structure batch in the mixed form: nrltb_bande_batch over uneven
    structures (spd and sp3, 4-64 atoms) returns what one nrltb_bande call per
    structure returns, bit for bit, and the smallest members agree with the
    oracle within the mixed form's tolerances."""
    from nrltb.api import new_result, result_from_c
    items = synth.batch256(count=10)
    opts = [Opts(mode=4, precision=MIXED, tkb=o["tkb"], eigcut=1e3, fermi_tol=1e-11) for (_, _, _, o) in items]
    single = [ctx.bande(st, par, km, op) for (st, par, km, _), op in zip(items, opts)]
    n = len(items)
    cs = (abi.Structure_ * n)(*[it[0].to_c() for it in items])
    cp = (abi.Params_ * n)(*[it[1].to_c() for it in items])
    ck = (abi.KMesh_ * n)(*[it[2].to_c() for it in items])
    co = (abi.Opts_ * n)(*[op.to_c() for op in opts])
    made = [new_result(it[1].nv(it[0]), it[2].nk) for it in items]
    cr = (abi.Result_ * n)(*[m[0] for m in made])
    assert ctx.lib.nrltb_bande_batch(ctx.h, n, cs, cp, ck, co, cr) == 0, ctx.lib.nrltb_last_error()
    for i in range(n):
        b = result_from_c(cr[i], made[i][1])
        a = single[i]
        assert b.efermi == a.efermi and b.e_total == a.e_total and b.pressure == a.pressure
        assert np.array_equal(b.eig, a.eig) and np.array_equal(b.deig, a.deig)
    by_cost = sorted(range(n), key=lambda i: items[i][1].nv(items[i][0]) ** 3 * items[i][2].nk)
    for i in by_cost[:4]:
        st, par, km, o = items[i]
        ref = oracle.bande(st, par, km, Opts(mode=4, tkb=o["tkb"], eigcut=1e3, fermi_tol=1e-11))
        g = single[i]
        assert (g.k_status == 0).all()
        assert np.abs(g.eig - ref.eig).max() <= 1e-9
        assert abs(g.efermi - ref.efermi) <= 1e-9
        assert abs(g.e_total - ref.e_total) / st.natoms <= 1e-8
        assert abs(g.pressure - ref.pressure) <= P_TOL


def test_mixed_bande_ex1_against_skout(ctx, ex1, ex1_gold):
    for idx in (0, 9):
        _, _, st, km = ex1.structures[idx]
        r = ctx.bande(st, ex1.params, km, Opts(mode=4, precision=MIXED, tkb=ex1.tkb, eigcut=ex1.eigcut))
        assert r.efermi == pytest.approx(ex1_gold["efermi"][idx], abs=1e-9)
        assert r.e_total == pytest.approx(ex1_gold["e_total"][idx], abs=1e-9)
        assert r.pressure == pytest.approx(ex1_gold["pressure"][idx], abs=P_TOL)


def _refprod(ctx, method, A, X):
    """Y = A X through the refinement's product (nrltb_bench_refprod_run)."""
    import ctypes as C
    A = np.ascontiguousarray(A.transpose(0, 2, 1), dtype=np.complex128)    # column-major per matrix
    Xc = np.ascontiguousarray(X.transpose(0, 2, 1), dtype=np.complex64)
    Y = np.zeros_like(A)
    b, n = A.shape[0], A.shape[1]
    rc = ctx.lib.nrltb_bench_refprod_run(ctx.h, method, n, b, A.ctypes.data_as(C.c_void_p),
                                         Xc.ctypes.data_as(C.c_void_p), Y.ctypes.data_as(C.c_void_p))
    assert rc == 0, ctx.lib.nrltb_last_error()
    return Y.transpose(0, 2, 1), Xc.transpose(0, 2, 1)


@pytest.mark.parametrize("method,n", [(0, 200), (1, 200), (1, 300), (2, 200), (2, 300)])
def test_refinement_product_accuracy(ctx, method, n):
    """H X against an extended-precision product of the X the method used.
    Double-float SIMT (method 0): componentwise, the error grows like n 2^-48
    |A||X| (its low part accumulates in plain FP32).  Tensor-core digits
    (method 1): exact per 64-wide chunk; the error is the cut of A after 6
    digits and the dropped digit levels, a fixed-point error per term of at
    most 2^-43 of (largest component in row m of A) x (largest component in
    column n of X).  Three digits of A (method 2, the Hellmann-Feynman
    products): A rounded to 24 bits of its row scale, at most 2^-23 per term
    in the same measure, and unbiased (the mean signed error is far below
    the bound)."""
    rng = np.random.default_rng(5)
    b = 2
    ctx.lib.nrltb_bench_umma_fault(1)
    # Hermitian A with H-like structure: O(1) diagonal, decaying off-diagonals
    # spanning many binades, some exact zeros
    A = rng.standard_normal((b, n, n)) + 1j * rng.standard_normal((b, n, n))
    i = np.arange(n)
    A *= np.exp(-np.abs(i[:, None] - i[None, :]) / 15.0)[None]
    A[:, 50:60, 100:120] = 0
    A = 0.5 * (A + A.conj().transpose(0, 2, 1))
    # FP32 X with columns of very different scale and a decaying tail
    X = (rng.standard_normal((b, n, n)) + 1j * rng.standard_normal((b, n, n))) * \
        np.logspace(-3, 1, n)[None, None, :] * np.exp(-i / 40.0)[None, :, None]
    X = X.astype(np.complex64)
    Y, Xu = _refprod(ctx, method, A, X)
    # the rounded X stays within 2^-23 of each column's largest element (half a
    # unit of 2^(e-23), 2^(e-1) <= colmax < 2^e)
    colmax = np.maximum(np.abs(X.real), np.abs(X.imag)).max(axis=1, keepdims=True)
    dx = np.maximum(np.abs(Xu.real - X.real), np.abs(Xu.imag - X.imag))
    assert (dx <= colmax * 2.0 ** -23).all()
    if method == 0:
        assert (Xu == X).all()
    ref = np.matmul(A.astype(np.clongdouble), Xu.astype(np.clongdouble))
    err = np.abs((Y.astype(np.clongdouble) - ref).astype(np.complex128))
    comp = np.matmul(np.abs(A), np.abs(Xu.astype(np.complex128)))
    amax = np.maximum(np.abs(A.real), np.abs(A.imag)).max(axis=2)
    xmax = np.maximum(np.abs(Xu.real), np.abs(Xu.imag)).max(axis=1).astype(np.float64)
    fixed = n * amax[:, :, None] * xmax[:, None, :]
    r_comp, r_fixed = (err / comp).max(), (err / fixed).max()
    if method == 0:
        assert r_comp <= n * 2.0 ** -46, (r_comp, r_fixed)
    elif method == 1:
        assert r_fixed <= 2.0 ** -43, (r_comp, r_fixed)
    else:
        assert r_fixed <= 2.0 ** -23, (r_comp, r_fixed)
        signed = ((Y.astype(np.clongdouble) - ref).astype(np.complex128) / fixed).real
        assert abs(signed.mean()) <= 2.0 ** -23 / 100, signed.mean()
    assert ctx.lib.nrltb_bench_umma_fault(0) == 0
