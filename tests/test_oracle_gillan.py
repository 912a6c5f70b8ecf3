"""Gillan's T -> 0 extrapolation (modes 1 and 2, bande.f:1100-1476) in the oracle.

The reference records no run in these modes, so the oracle's new terms are
pinned three ways on the Pd parameters and fcc k set of ex1:

* a numpy restatement of the sums (bande.f:1189-1242, 1290-1316) and of the
  outputs (bande.f:1409-1476) over the oracle's own eigenvalues and dE_i/dV;
* thermodynamics: P(T) = -dE/dV and P_A(T) = P(T) - shift = -dA/dV by central
  differences in the volume, and dA/dT = -S at fixed volume (the occupations
  minimise A at fixed electron count, so only the explicit T term is left);
* modes 1 and 2 leave E_F, E(T), P(T) and the Fermi-level shift exactly as
  modes 3 and 4 give them.
"""
import math
import os
import shutil

import numpy as np
import pytest

import oracle
from conftest import GOLDEN
from nrltb import Opts, read_skin


def _skin(dirname, mode, tkb, alats, eigcut=0.5):
    """Pd fcc at the given cubic lattice constants, ex1's parameters and k set."""
    os.makedirs(dirname, exist_ok=True)
    for f in ("pd_par", "spcgrp.fcc", "fcc.08"):
        shutil.copy(os.path.join(GOLDEN, "ex1", f), os.path.join(dirname, f))
    with open(os.path.join(dirname, "SKIN"), "w") as f:
        f.write("Mode=%d\n%.17g %.17g\npd_par\n" % (mode, tkb, eigcut))
        for j, a in enumerate(alats):
            f.write("Pd\n fcc %.4f\n 0.00\n 1\n %.17g\n 0\n 1\n 4 4 4\nF\n 1 0 0 0 0 0 0\n" % (a, a))
            if j == 0:
                f.write("NEWSYM=T\nLATTIC=1\nspcgrp.fcc\nILAT=F\n-1313\nfcc.08\n")
            else:
                f.write("NEWSYM=F\n")
    return read_skin(os.path.join(dirname, "SKIN"))


def _run(sk, mode, tkb):
    return [oracle.bande(st, sk.params, km, Opts(mode=mode, tkb=tkb, eigcut=sk.eigcut))
            for (_, _, st, km) in sk.structures]


def _restated(r, w, tkb, lpress):
    """bande.f's window sums and outputs from eigenvalues, dE_i/dV and ncut."""
    tkbi = 1e5 if tkb < 1e-5 else 1.0 / tkb
    ef = r.efermi
    efp, efm = ef + 20.0 * tkb, ef - 20.0 * tkb
    ent = dent1 = dent2 = 0.0
    for k in range(r.nk):
        wt = 2.0 * w[k]
        lim = int(r.ncut[k]) if lpress else r.nv
        for i in range(lim):
            e = r.eig[k, i]
            if not (e < efp) or e < efm:
                continue
            x = e - ef
            f = 1.0 / (1.0 + math.exp(tkbi * x))
            ent -= wt * (f * math.log(f) + (1.0 - f) * math.log(1.0 - f))
            if lpress:
                dfbe = -tkbi * f * (1.0 / (1.0 + math.exp(-tkbi * x)))
                con1 = dfbe * wt * x
                dent1 += con1 * r.deig[k, i]
                dent2 += con1
    free = r.e_total - tkb * ent
    out = dict(entropy=ent, free_energy=free, earg1=0.5 * (r.e_total + free), earg2=r.e_total,
               entropy_shift=0.0)
    if lpress:
        pent = r.fermi_shift * dent2 - dent1
        out["entropy_shift"] = pent
        out["earg2"] = 0.5 * (r.pressure + (r.pressure - pent))
    return out


@pytest.mark.parametrize("mode,tkb", [(1, 0.005), (2, 0.005), (2, 0.02)])
def test_gillan_terms_restated(tmp_path, mode, tkb):
    sk = _skin(str(tmp_path), mode, tkb, [7.2])
    km = sk.structures[0][3]
    r = _run(sk, mode, tkb)[0]
    ref = _restated(r, km.w, tkb, mode == 2)
    assert r.entropy > 0
    for key, v in ref.items():
        assert getattr(r, key) == pytest.approx(v, rel=1e-12, abs=1e-16), key


@pytest.mark.parametrize("tkb", [0.005, 0.02])
def test_gillan_pressures_are_volume_derivatives(tmp_path, tkb):
    h = 0.004
    sk = _skin(str(tmp_path), 2, tkb, [7.2 - h, 7.2, 7.2 + h])
    rm, r, rp = _run(sk, 2, tkb)
    vm, vp = sk.structures[0][2].volume, sk.structures[2][2].volume
    p_e = -(rp.e_total - rm.e_total) / (vp - vm)
    p_a = -(rp.free_energy - rm.free_energy) / (vp - vm)
    # central differences carry an O(h^2) error common to both, ~4e-5 relative here
    assert r.pressure == pytest.approx(p_e, rel=1e-4)
    assert r.pressure - r.entropy_shift == pytest.approx(p_a, rel=1e-4)
    # the entropy shift itself is the difference of the two derivatives
    assert -r.entropy_shift == pytest.approx(p_a - p_e, rel=1e-3)
    assert r.earg2 == pytest.approx(0.5 * (p_e + p_a), rel=1e-4)


def test_gillan_entropy_is_minus_dA_dT(tmp_path):
    t0, dt = 0.02, 0.0002
    sk = _skin(str(tmp_path), 1, t0, [7.2])
    _, _, st, km = sk.structures[0]
    a = [oracle.bande(st, sk.params, km, Opts(mode=1, tkb=t, eigcut=0.5, fermi_tol=1e-13))
         for t in (t0 - dt, t0, t0 + dt)]
    dadt = (a[2].free_energy - a[0].free_energy) / (2 * dt)
    assert -dadt == pytest.approx(a[1].entropy, rel=1e-5)
    # E(0) = (E + A)/2 removes the first order in T: E(T) - E(0) = T S / 2
    assert a[1].e_total - a[1].earg1 == pytest.approx(0.5 * t0 * a[1].entropy, rel=1e-12)


@pytest.mark.parametrize("gillan,plain", [(1, 3), (2, 4)])
def test_gillan_modes_keep_the_plain_outputs(tmp_path, gillan, plain):
    sk = _skin(str(tmp_path), gillan, 0.005, [7.0, 7.4])
    for (_, _, st, km) in sk.structures:
        g = oracle.bande(st, sk.params, km, Opts(mode=gillan, tkb=0.005, eigcut=0.5))
        p = oracle.bande(st, sk.params, km, Opts(mode=plain, tkb=0.005, eigcut=0.5))
        assert (g.efermi, g.e_total, g.pressure, g.fermi_shift) == (p.efermi, p.e_total, p.pressure, p.fermi_shift)
        assert np.array_equal(g.eig, p.eig)
        # the plain modes' outputs: E(T) and P(T) (mode 4) or 0 (mode 3), no entropy
        assert p.entropy == 0 and p.free_energy == 0 and p.entropy_shift == 0
        assert p.earg1 == p.e_total and p.earg2 == (p.pressure if plain == 4 else 0.0)
        assert g.earg1 == 0.5 * (g.e_total + g.free_energy)
        if gillan == 1:
            assert g.earg2 == g.e_total and g.entropy_shift == 0
