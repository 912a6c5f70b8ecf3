"""The host driver's own code (host/nrltb_static.c: reading, mode handling and
every output file) on the CPU, with its device calls served by the oracle
through tests/driver_harness.c.  Checked: the reference's ex1 SKENG to its 9
printed decimals (the same golden as the GPU driver test), the mode-2 and
spin-polarized SKENG columns, QLMT / QAPW records against the writer fed the
same results, SPNDIR lines, and the modes the driver refuses."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle
from conftest import GOLDEN, REPO
from nrltb import Opts, Structure, abi, read_skin, synth, write_qlmt

HOST = os.path.join(REPO, "tight-binding_gb300", "host")


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("drv") / "libdriver_oracle.so")
    srcs = [os.path.join(HOST, f) for f in ("nrltb_static.c", "nrltb_input.c", "nrltb_qlmt.c")]
    srcs += [os.path.join(REPO, "oracle", "nrltb_oracle.c"), os.path.join(REPO, "tests", "driver_harness.c")]
    subprocess.run(["gcc", "-std=gnu11", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-fopenmp",
                    "-Dmain=nrltb_static_main", "-I", os.path.join(REPO, "include")] + srcs +
                   ["-o", so, "-lm"], check=True)
    lib = C.CDLL(so)
    import scipy.linalg.cython_lapack as cl
    lib.oracle_set_lapack.argtypes = [C.c_void_p, C.c_void_p]
    lib.oracle_set_lapack(oracle._capsule_ptr(cl.__pyx_capi__["zhpgv"]), oracle._capsule_ptr(cl.__pyx_capi__["zhpev"]))
    lib.nrltb_static_main.argtypes = [C.c_int, C.POINTER(C.c_char_p)]

    def run(cwd, *args):
        argv = [b"nrltb_static"] + [a.encode() for a in args]
        arr = (C.c_char_p * len(argv))(*argv)
        old = os.getcwd()
        os.chdir(cwd)
        try:
            return lib.nrltb_static_main(len(argv), arr)
        finally:
            os.chdir(old)
    return run


def test_ex1_skeng(driver, tmp_path, ex1_gold):
    src = os.path.join(GOLDEN, "ex1")
    for f in os.listdir(src):
        shutil.copy(os.path.join(src, f), tmp_path / f)
    assert driver(tmp_path, "SKIN") == 0
    lines = (tmp_path / "SKENG").read_text().splitlines()
    assert len(lines) == 18
    for line, gold, label in zip(lines, ex1_gold["skeng"], ex1_gold["labels"]):
        assert line[:20].split() == label.split()
        vals = [float(x) for x in line[20:].split()]
        assert abs(vals[0] - gold[0]) <= 5e-7
        for v, g in zip(vals[1:], gold[1:]):
            assert abs(v - g) <= 1.01e-9
    assert (tmp_path / "SKOUT").read_text().count("Number of pairs =") == 18


def _cscl(flip=None, angles=None):
    a = 5.6
    plv = np.eye(3) * a
    sp = None
    if angles is not None:
        sp = np.array([[np.sin(np.radians(t)) * np.cos(np.radians(p)), np.sin(np.radians(t)) * np.sin(np.radians(p)),
                        np.cos(np.radians(t))] for t, p in angles])
    return Structure([1, 1], [[0, 0, 0], [a / 2] * 3], plv, synth.search_box(plv, 16.5), a ** 3,
                     flip=None if flip is None else np.array(flip), spinat=sp)


@pytest.mark.parametrize("mode", [1, 2, 3, 4])
def test_skeng_columns_by_mode_and_spin(driver, tmp_path, mode):
    mag = synth.make_magnetic_params([9], [10.0], 7, split=0.08)
    km = synth.mp_mesh(2)
    synth.write_skin(str(tmp_path), [(_cscl(), km), (_cscl(flip=[0, 1]), km)], mag, mode=mode, tkb=0.01)
    assert driver(tmp_path, "SKIN") == 0
    sk = read_skin(str(tmp_path / "SKIN"))
    lines = (tmp_path / "SKENG").read_text().splitlines()
    assert len(lines) == 2
    for line, (_, _, st, k) in zip(lines, sk.structures):
        o = oracle.bande(st, sk.params, k, Opts(mode=mode, tkb=sk.tkb, eigcut=sk.eigcut))
        vals = [float(x) for x in line[20:].split()]
        want = [o.efermi, o.earg1] + ([o.earg2] if mode != 3 else []) + [o.smag]   # static.f:1246-1253
        assert len(vals) == 1 + len(want)
        np.testing.assert_allclose(vals[1:-1], want[:-1], atol=1.01e-9)
        assert abs(vals[-1] - o.smag) <= 5.01e-7


@pytest.mark.parametrize("mode", [6, 8, 9, 10])
def test_eigenvalue_files(driver, tmp_path, mode):
    st, par, km, o = synth.fcc1()
    rng = np.random.default_rng(5)
    from nrltb import KMesh
    km = KMesh(rng.uniform(-0.5, 0.5, (4, 3)), np.full(4, 0.25))
    synth.write_skin(str(tmp_path), [(st, km)], par, mode=mode, tkb=o["tkb"], eigcut=0.5)
    assert driver(tmp_path, "SKIN") == 0
    name = "QAPW" if mode == 8 else "QLMT"
    sk = read_skin(str(tmp_path / "SKIN"))
    _, _, s, k = sk.structures[0]
    res = oracle.bande(s, sk.params, k, Opts(mode=mode, tkb=sk.tkb, eigcut=sk.eigcut))
    write_qlmt(str(tmp_path / "ref"), mode, s, sk.params, k, sk.eigcut, res)
    assert (tmp_path / name).read_text() == (tmp_path / "ref").read_text()


def test_spin_directions_file(driver, tmp_path):
    mag = synth.make_magnetic_params([9], [10.0], 7, split=0.08)
    km = synth.mp_mesh(2)
    synth.write_skin(str(tmp_path), [(_cscl(angles=[(0, 0), (90, 30)]), km)], mag, mode=3, tkb=0.01)
    path = tmp_path / "SKIN"
    path.write_text(path.read_text().replace("\nFN\n", "\nFS\n"))
    assert driver(tmp_path, "SKIN") == 0
    sk = read_skin(str(path))
    _, label, st, k = sk.structures[0]
    o = oracle.bande(st, sk.params, k, Opts(mode=3, tkb=sk.tkb, eigcut=sk.eigcut, flags=abi.OPT_SPIN_DIRECTIONS))
    lines = (tmp_path / "SPNDIR").read_text().splitlines()
    assert len(lines) == 2
    for i, line in enumerate(lines):
        vals = [float(x) for x in line[25:].split()]
        np.testing.assert_allclose(vals[:3], o.spdir[i], atol=5.01e-7)
        v = o.spdir[i]
        assert vals[4] == pytest.approx(np.degrees(np.arccos(v[2] / np.linalg.norm(v))), abs=5.01e-7)
        assert vals[5] == pytest.approx(np.degrees(np.arctan2(v[1], v[0])), abs=5.01e-7)
    assert len((tmp_path / "SKENG").read_text().splitlines()[0][20:].split()) == 3


@pytest.mark.parametrize("mode", [5, 7, 11])
def test_refused_modes(driver, tmp_path, mode):
    st, par, km, o = synth.fcc1()
    synth.write_skin(str(tmp_path), [(st, km)], par, mode=mode, tkb=o["tkb"])
    assert driver(tmp_path, "SKIN") == 1
    assert not (tmp_path / "SKENG").exists()
