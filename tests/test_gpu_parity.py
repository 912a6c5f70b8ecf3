"""GPU path (through the C ABI) against the oracle and the ex1 goldens.

Tolerances (FP64 form): eigenvalues 1e-10 Ry, E_F 1e-9 Ry, E_total 1e-8 Ry/atom,
pressure 1e-3 kbar = 6.8e-9 Ry/bohr^3; integer pair lists and their order exact.
"""
import numpy as np
import pytest

import oracle
from nrltb import KMesh, Opts, synth

pytestmark = pytest.mark.gpu

KBAR = 1.0 / 147105.08      # Ry/bohr^3 per kbar
P_TOL = 1e-3 * KBAR


def _sub(km, idx):
    idx = np.asarray(idx)
    w = km.w[idx] / km.w[idx].sum()
    return KMesh(km.k[idx], w)


def _structs(ex1):
    out = [(ex1.structures[i][2], ex1.params) for i in (0, 7, 9, 17)]
    for name in ("fcc1", "bcc32", "fcc128", "b2_216"):
        st, par, km, _ = synth.CONFIGS[name]()
        out.append((st, par))
    return out


def test_search2_bit_exact(ctx, ex1):
    for st, par in _structs(ex1):
        g, gk, gd = ctx.search2(st, par)
        o, ok, od = oracle.search2(st, par)
        assert len(g["dist"]) == len(o["dist"])
        for key in ("dlv", "jkind", "jatm"):
            assert np.array_equal(g[key], o[key]), key
        assert np.array_equal(g["dist"], o["dist"])       # same ops, no contraction
        assert np.array_equal(g["tt"], o["tt"])
        np.testing.assert_allclose(g["screen"], o["screen"], rtol=1e-14, atol=0)
        np.testing.assert_allclose(g["dscrn"], o["dscrn"], rtol=1e-13, atol=1e-300)
        assert gk == ok and gd == od


def test_search2_carried_flag(ctx, ex1):
    st, par = ex1.structures[0][2], ex1.params
    for kin in (0, 1):
        g, gk, _ = ctx.search2(st, par, kneigh_in=kin)
        o, ok, _ = oracle.search2(st, par, kneigh_in=kin)
        assert len(g["dist"]) == len(o["dist"]) and gk == ok


def test_search2_empty_pair_list(ctx):
    from nrltb import Params, Structure
    _, par, _, _ = synth.fcc1()
    tiny = Params(par.kinds, par.kbas, par.valence, np.array([1.0]), np.array([0.5]), par.param)
    plv = np.eye(3) * 10.0
    st = Structure(np.array([1], np.int32), np.zeros((1, 3)), plv, (1, 1, 1), 1000.0)
    g, _, _ = ctx.search2(st, tiny)
    assert len(g["dist"]) == 0


def test_setpar_matches_oracle(ctx, ex1):
    for st, par in _structs(ex1):
        pairs, _, _ = oracle.search2(st, par)
        o = oracle.setpar(st, par, pairs, deriv=True)
        g = ctx.setpar(st, par, pairs, deriv=True)
        for key in ("hop", "over", "dhop", "dover"):
            scale = max(np.abs(o[key]).max(), 1e-300)
            np.testing.assert_allclose(g[key], o[key], rtol=1e-13, atol=1e-15 * scale, err_msg=key)
        for key in ("den", "paros", "dparos"):
            np.testing.assert_allclose(g[key], o[key], rtol=1e-12, atol=1e-15, err_msg=key)


@pytest.mark.parametrize("which", [0, 1])
def test_setham_matches_oracle(ctx, ex1, which):
    cases = [(ex1.structures[0][2], ex1.params, ex1.structures[0][3]),
             (ex1.structures[17][2], ex1.params, ex1.structures[17][3])]
    st, par, km, _ = synth.bcc32()
    cases.append((st, par, _sub(km, [0, 5, 63])))
    st, par, km, _ = synth.fcc128()
    cases.append((st, par, _sub(km, [4])))
    st, par, km, _ = synth.b2_216()
    cases.append((st, par, _sub(km, [3])))
    for st, par, km in cases:
        gh, gs = ctx.setham(st, par, km, which)
        oh, os_ = oracle.setham(st, par, km, which)
        for g, o in ((gh, oh), (gs, os_)):
            scale = max(np.abs(o).max(), 1e-300)
            assert np.abs(g - o).max() <= 1e-13 * scale + 1e-300


def _check_eigs(ctx, H, S, tol=1e-10):
    ge, gz, gst = ctx.diag(H, S)
    oe, _, ost = oracle.diag(H, S, vectors=False)
    assert (gst == 0).all() and (ost == 0).all()
    assert np.abs(ge - oe).max() <= tol, np.abs(ge - oe).max()
    for k in range(H.shape[0]):
        Z = gz[k]
        res = H[k] @ Z - (S[k] @ Z) * ge[k][None, :]
        assert np.abs(res).max() < 1e-10 * max(1.0, np.abs(H[k]).max())
        G = Z.conj().T @ S[k] @ Z
        assert np.abs(G - np.eye(len(G))).max() < 1e-10
    return ge


def test_diag_fp64_small(ctx, ex1):
    st, par, km = ex1.structures[0][2], ex1.params, ex1.structures[0][3]
    H, S = oracle.setham(st, par, km)
    _check_eigs(ctx, H, S)


def test_diag_fp64_n288(ctx):
    st, par, km, _ = synth.bcc32()
    H, S = oracle.setham(st, par, _sub(km, [0, 21]))
    _check_eigs(ctx, H, S)


def test_diag_fp64_n1152(ctx):
    st, par, km, _ = synth.fcc128()
    H, S = oracle.setham(st, par, _sub(km, [13]))
    _check_eigs(ctx, H, S)


def test_diag_degenerate_and_tiny(ctx):
    # exactly degenerate spectrum (block-diagonal copies) and a 1x1 problem
    rng = np.random.default_rng(5)
    A = rng.normal(size=(6, 6)) + 1j * rng.normal(size=(6, 6))
    A = A + A.conj().T
    H = np.zeros((1, 18, 18), complex)
    for b in range(3):
        H[0, 6 * b:6 * b + 6, 6 * b:6 * b + 6] = A
    S = np.eye(18)[None].astype(complex)
    _check_eigs(ctx, H, S)
    H1 = np.array([[[2.5 + 0j]]])
    S1 = np.array([[[1.25 + 0j]]])
    ge, gz, _ = ctx.diag(H1, S1)
    assert ge[0, 0] == pytest.approx(2.0, abs=1e-15)


def test_diag_overlap_not_positive_definite(ctx):
    # a host-made failure: indefinite S is reported per k, nothing faults
    H = np.diag([1.0, 2.0, 3.0]).astype(complex)[None]
    S = np.diag([1.0, -0.5, 1.0]).astype(complex)[None]
    _, _, st = ctx.diag(H, S)
    assert st[0] == 1


def test_fermi_matches_oracle(ctx):
    rng = np.random.default_rng(3)
    eig = np.sort(rng.uniform(-1, 1, (27, 40)), axis=1)
    w = np.full(27, 1 / 27)
    for zfill, tkb in ((31.0, 0.005), (40.0, 0.01), (2.0, 0.001)):
        ef_g = ctx.fermi(eig, w, tkb, zfill, tol=1e-12)
        ef_o = oracle.fermi(eig, w, tkb, zfill, tol=1e-12)
        assert ef_g == pytest.approx(ef_o, abs=1e-11)


@pytest.mark.parametrize("idx", [0, 4, 8, 9, 13, 17])
def test_bande_ex1_against_skout(ctx, ex1, ex1_gold, idx):
    _, _, st, km = ex1.structures[idx]
    r = ctx.bande(st, ex1.params, km, Opts(mode=4, tkb=ex1.tkb, eigcut=ex1.eigcut))
    assert r.npairs == ex1_gold["npairs"][idx]
    assert r.efermi == pytest.approx(ex1_gold["efermi"][idx], abs=1e-10)
    assert r.e_total == pytest.approx(ex1_gold["e_total"][idx], abs=1e-10)
    assert r.pressure == pytest.approx(ex1_gold["pressure"][idx], abs=1e-11)
    assert r.fermi_shift == pytest.approx(ex1_gold["fermi_shift"][idx], abs=1e-11)


def _compare_bande(ctx, st, par, km, tkb, nthreads=0, mode=4):
    opts = Opts(mode=mode, tkb=tkb, eigcut=1e3, fermi_tol=1e-11)
    g = ctx.bande(st, par, km, opts)
    o = oracle.bande(st, par, km, opts, nthreads=nthreads)
    assert g.npairs == o.npairs and g.nv == o.nv
    assert np.abs(g.eig - o.eig).max() <= 1e-10
    assert abs(g.efermi - o.efermi) <= 1e-9
    assert abs(g.e_total - o.e_total) / st.natoms <= 1e-8
    if mode == 4:
        assert abs(g.pressure - o.pressure) <= P_TOL
        # group sums of deig are invariant under rotations inside degenerate groups
        for k in range(km.nk):
            e = o.eig[k]
            grp = np.concatenate([[0], np.cumsum(np.abs(np.diff(e)) > 1e-8)])
            for gid in np.unique(grp):
                m = grp == gid
                assert abs(g.deig[k][m].sum() - o.deig[k][m].sum()) <= 1e-9 * max(1, m.sum())
    return g, o


def test_bande_fcc1_full_mesh(ctx):
    st, par, km, o = synth.fcc1()
    _compare_bande(ctx, st, par, km, o["tkb"])


def test_bande_bcc32_subset(ctx):
    st, par, km, o = synth.bcc32()
    _compare_bande(ctx, st, par, _sub(km, [0, 9, 18, 27, 36, 45, 54, 63]), o["tkb"])


def test_bande_mode3_energy_only(ctx, ex1):
    _, _, st, km = ex1.structures[2]
    _compare_bande(ctx, st, ex1.params, km, ex1.tkb, mode=3)


def test_bande_nonpositive_overlap_kpoints(ctx):
    # A parameter draw whose S(k) is indefinite at some k (made on the host, no
    # device fault): those k carry the eigenvalues of S and no pressure terms,
    # as diag.f:429-455 and bande.f:997-1003 leave them, and are counted.
    st, _, km, _ = synth.fcc1()
    par = synth.make_params([9], [11.0], 11)
    sub = _sub(km, [0, 340, 471, 900, 1727])
    g, o = _compare_bande(ctx, st, par, sub, 0.005)
    assert o.nonphysical_k >= 2
    assert g.nonphysical_k == o.nonphysical_k
    assert np.array_equal(g.k_status, o.k_status)


def test_host_driver_ex1_skeng(tmp_path, ex1_gold):
    # the C driver (static.f's structure loop) over the ex1 SKIN reproduces the
    # reference's SKENG to its printed 9 decimals
    import os
    import shutil
    import subprocess
    from conftest import GOLDEN
    from nrltb import build
    src = os.path.join(GOLDEN, "ex1")
    for f in os.listdir(src):
        shutil.copy(os.path.join(src, f), tmp_path / f)
    r = subprocess.run([build.DRIVER, "SKIN"], cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    lines = (tmp_path / "SKENG").read_text().splitlines()
    assert len(lines) == 18
    for line, gold, label in zip(lines, ex1_gold["skeng"], ex1_gold["labels"]):
        assert line[:20].split() == label.split()
        vals = [float(x) for x in line[20:].split()]
        assert abs(vals[0] - gold[0]) <= 5e-7
        for v, g in zip(vals[1:], gold[1:]):
            assert abs(v - g) <= 1.01e-9
    out = (tmp_path / "SKOUT").read_text()
    assert out.count("Number of pairs =") == 18


def test_pressure_matches_energy_derivative_b2_216(ctx):
    """The two-species N=1404 configuration (8 Gamma-centred k, kT = 0.01): the
    Hellmann-Feynman pressure against -dE/dV from E(T) at V0 (1 +- h),
    (1 +- 2h), h = 0.25% (five-point difference), uniform scaling of the cell
    and the atoms.  FP64 form.  The pair cut-off is raised from 16.5 to 24
    bohr for this check: at 16.5 the screened integrals are still ~1e-5 Ry, so
    the pairs that cross the cut-off as the cell scales make E(V) jump (a
    ~3e-5 relative offset of the difference quotient, present in the
    reference model too; ~8e-7 at 20 bohr); at 24 bohr the jumps are below
    1e-13 Ry."""
    from dataclasses import replace
    from nrltb import Structure
    st0, par0, km, o = synth.b2_216()
    par = replace(par0, dnn=np.full_like(par0.dnn, 24.0))

    def scaled(eps):
        s = (1.0 + eps) ** (1.0 / 3.0)
        plv = st0.plv * s
        return Structure(st0.kkind, st0.posn * s, plv, synth.search_box(plv, 24.0), st0.volume * (1.0 + eps))

    st = scaled(0.0)
    opts4 = Opts(mode=4, tkb=o["tkb"], eigcut=1e3, fermi_tol=1e-12)
    opts3 = Opts(mode=3, tkb=o["tkb"], eigcut=1e3, fermi_tol=1e-12)
    r0 = ctx.bande(st, par, km, opts4, want_eig=False)

    def energy(eps):
        return ctx.bande(scaled(eps), par, km, opts3, want_eig=False).e_total

    h = 0.0025
    e1p, e1m, e2p, e2m = energy(h), energy(-h), energy(2 * h), energy(-2 * h)
    dedv = (8.0 * (e1p - e1m) - (e2p - e2m)) / (12.0 * h * st.volume)
    assert abs(-dedv - r0.pressure) <= P_TOL, (-dedv, r0.pressure)


def test_bande_batch_matches_single_calls(ctx):
    """nrltb_bande_batch over a mixed list of structures (spd and sp3, 4-64
    atoms, 2^3..5^3 meshes) returns what one nrltb_bande call per structure
    returns, bit for bit, and a small member agrees with the oracle."""
    import ctypes as C
    from nrltb import abi
    from nrltb.api import new_result, result_from_c
    items = synth.batch256(count=12)
    opts = [Opts(mode=4, tkb=o["tkb"], eigcut=1e3, fermi_tol=1e-12) for (_, _, _, o) in items]
    single = [ctx.bande(st, par, km, op) for (st, par, km, _), op in zip(items, opts)]
    n = len(items)
    cs = (abi.Structure_ * n)(*[it[0].to_c() for it in items])
    cp = (abi.Params_ * n)(*[it[1].to_c() for it in items])
    ck = (abi.KMesh_ * n)(*[it[2].to_c() for it in items])
    co = (abi.Opts_ * n)(*[op.to_c() for op in opts])
    made = [new_result(it[1].nv(it[0]), it[2].nk) for it in items]
    cr = (abi.Result_ * n)(*[m[0] for m in made])
    rc = ctx.lib.nrltb_bande_batch(ctx.h, n, cs, cp, ck, co, cr)
    assert rc == 0, ctx.lib.nrltb_last_error()
    for i in range(n):
        b = result_from_c(cr[i], made[i][1])
        a = single[i]
        assert b.efermi == a.efermi and b.e_total == a.e_total and b.pressure == a.pressure
        assert np.array_equal(b.eig, a.eig) and np.array_equal(b.deig, a.deig)
    small = min(range(n), key=lambda i: items[i][1].nv(items[i][0]) * items[i][2].nk)
    st, par, km, _ = items[small]
    ref = oracle.bande(st, par, km, opts[small])
    assert abs(single[small].efermi - ref.efermi) <= 1e-9
    assert np.abs(single[small].eig - ref.eig).max() <= 1e-10
