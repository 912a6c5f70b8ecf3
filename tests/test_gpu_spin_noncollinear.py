"""Non-collinear spins on the GPU path against the oracle: the doubled 2N x 2N
problem (k_noncol_onsite, k_noncol_spin_terms, k_noncol_expand, then the
solve, Hellmann-Feynman and Fermi sums at order 2N), in both precision forms,
modes 4 and 2, on the CsCl cell of the oracle's tests (parallel, rotated,
antiparallel and canted spins), an orthogonal set, two species, and the
orbital charges of mode 6.

Tolerances: eigenvalues 1e-10 Ry (FP64) / 1e-9 Ry (mixed), E_F 1e-9 Ry,
E(T) 1e-8 Ry/atom, P 1e-3 kbar."""
import math
from dataclasses import replace

import numpy as np
import pytest

import oracle
from nrltb import Opts, Structure, abi, synth

pytestmark = pytest.mark.gpu

KBAR = 1.0 / 147105.08
A, TKB = 5.6, 0.01


def _dirs(angles):
    return np.array([[math.sin(math.radians(t)) * math.cos(math.radians(p)),
                      math.sin(math.radians(t)) * math.sin(math.radians(p)), math.cos(math.radians(t))]
                     for t, p in angles])


def _cscl(angles, kinds=(1, 1)):
    plv = np.eye(3) * A
    return Structure(list(kinds), [[0, 0, 0], [A / 2, A / 2, A / 2]], plv, synth.search_box(plv, 16.5), A ** 3,
                     spinat=_dirs(angles))


def _check(ctx, st, par, km, mode, precision):
    g = ctx.bande(st, par, km, Opts(mode=mode, precision=precision, tkb=TKB, eigcut=1e3, fermi_tol=1e-11))
    o = oracle.bande(st, par, km, Opts(mode=mode, tkb=TKB, eigcut=1e3, fermi_tol=1e-11))
    assert g.nv == o.nv == 2 * par.nv(st) and g.eig.shape == o.eig.shape
    assert (g.k_status == 0).all() and (o.k_status == 0).all()
    assert np.abs(g.eig - o.eig).max() <= (1e-10 if precision == abi.PREC_FP64 else 1e-9)
    assert abs(g.efermi - o.efermi) <= 1e-9
    assert abs(g.e_total - o.e_total) / st.natoms <= 1e-8
    assert abs(g.earg1 - o.earg1) / st.natoms <= 1e-8
    if mode in (2, 4):
        assert abs(g.pressure - o.pressure) <= 1e-3 * KBAR
        assert abs(g.earg2 - o.earg2) <= 1e-3 * KBAR
    assert g.smag == 0.0
    return g, o


@pytest.fixture(scope="module")
def mag():
    return synth.make_magnetic_params([9], [10.0], 7, split=0.08)


@pytest.fixture(scope="module")
def km():
    return synth.mp_mesh(3)


ORDERS = [[(0, 0), (0, 0)], [(37, 110), (37, 110)], [(0, 0), (180, 0)], [(0, 0), (90, 30)]]


@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_MIXED])
@pytest.mark.parametrize("mode", [4, 2])
@pytest.mark.parametrize("angles", ORDERS)
def test_noncollinear_against_oracle(ctx, mag, km, angles, mode, precision):
    _check(ctx, _cscl(angles), mag, km, mode, precision)


def test_noncollinear_orthogonal_and_two_species(ctx, km):
    mag = synth.make_magnetic_params([9], [10.0], 7, split=0.08)
    _check(ctx, _cscl([(0, 0), (90, 30)]), replace(mag, jsover=0), km, 4, abi.PREC_FP64)
    mag2 = synth.make_magnetic_params([9, 4], [10.0, 3.0], 7, split=0.05)
    _check(ctx, _cscl([(20, 0), (120, 60)], kinds=(1, 2)), mag2, km, 4, abi.PREC_FP64)


def test_noncollinear_orbital_charges(ctx, mag, km):
    st = _cscl([(0, 0), (90, 30)])
    g = ctx.bande(st, mag, km, Opts(mode=6, tkb=TKB, eigcut=1e3, fermi_tol=1e-11))
    o = oracle.bande(st, mag, km, Opts(mode=6, tkb=TKB, eigcut=1e3, fermi_tol=1e-11))
    assert g.orbocc.shape == o.orbocc.shape == (km.nk, 2 * mag.nv(st), 2 * mag.nv(st))
    for row in range(km.nk):
        e = o.eig[row]
        grp = np.concatenate([[0], np.cumsum(np.diff(e) > 1e-8)])
        for gid in np.unique(grp):
            m = grp == gid
            assert np.abs(g.orbocc[row][m].sum(axis=0) - o.orbocc[row][m].sum(axis=0)).max() <= 1e-9 * m.sum()


def test_noncollinear_needs_two_sets(ctx, km):
    from nrltb import NrltbError
    p1 = synth.make_params([9], [10.0], 7)
    with pytest.raises(NrltbError):
        ctx.bande(_cscl([(0, 0), (0, 0)]), p1, km, Opts(mode=3, tkb=TKB))


@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_MIXED])
@pytest.mark.parametrize("angles", [[(37, 110), (37, 110)], [(0, 0), (180, 0)], [(0, 0), (90, 30)]])
def test_spin_directions(ctx, mag, km, angles, precision):
    st = _cscl(angles)
    op = dict(tkb=TKB, eigcut=1e3, fermi_tol=1e-11, flags=abi.OPT_SPIN_DIRECTIONS)
    g = ctx.bande(st, mag, km, Opts(mode=3, precision=precision, **op))
    o = oracle.bande(st, mag, km, Opts(mode=3, **op))
    assert g.spdir.shape == o.spdir.shape == (2, 3)
    assert np.abs(g.spdir - o.spdir).max() <= 1e-8


def test_host_driver_spin_directions(tmp_path, mag, km):
    import subprocess
    from nrltb import build, read_skin
    sts = [(_cscl([(0, 0), (90, 30)]), km), (_cscl([(20, 40), (160, -30)]), km)]
    synth.write_skin(str(tmp_path), sts, mag, mode=3, tkb=TKB)
    path = tmp_path / "SKIN"
    path.write_text(path.read_text().replace("\nFN\n", "\nFS\n"))
    r = subprocess.run([build.DRIVER, "SKIN"], cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    lines = (tmp_path / "SPNDIR").read_text().splitlines()
    assert len(lines) == 4
    sk = read_skin(str(path))
    for j, (_, label, s2, k2) in enumerate(sk.structures):
        o = oracle.bande(s2, sk.params, k2, Opts(mode=3, tkb=sk.tkb, eigcut=sk.eigcut,
                                                 flags=abi.OPT_SPIN_DIRECTIONS))
        for i in range(2):
            line = lines[2 * j + i]
            assert line[:20].split() == label.split() and int(line[20:25]) == i + 1
            vals = [float(x) for x in line[25:].split()]
            np.testing.assert_allclose(vals[:3], o.spdir[i], atol=1.01e-6)
            assert vals[3] == pytest.approx(np.linalg.norm(o.spdir[i]), abs=1.01e-6)
    skeng = (tmp_path / "SKENG").read_text().splitlines()
    assert len(skeng) == 2 and len(skeng[0][20:].split()) == 3   # volume, E_F, E(T): no moment column
