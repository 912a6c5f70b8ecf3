"""The SKIN reader's lattice types and strain menus (setlat.f:147-1000): the C
reader (host/nrltb_input.c, through nrltb.read_skin) against a separate numpy
restatement of setlat.f written here, and against geometry the options are
documented to produce (cell volumes, volume-conserving strains, the magic-strain
lattices' fcc and bcc points, the 60 degree rhombohedron, c = a tetragonals)."""
import math
import os

import numpy as np
import pytest

from nrltb import read_skin, synth

H = 0.5
T3 = 1.0 / 3.0


def _write(dirname, lattice_lines, strain_lines):
    """One structure: one atom at the origin, a one-point k file."""
    par = synth.make_params([9], [10.0], seed=1)
    os.makedirs(dirname, exist_ok=True)
    synth.write_params(os.path.join(dirname, "par"), par)
    with open(os.path.join(dirname, "k1"), "w") as f:
        f.write("    1\n0 0 0 1\n")
    with open(os.path.join(dirname, "sg"), "w") as f:
        f.write("identity\n")
    with open(os.path.join(dirname, "SKIN"), "w") as f:
        f.write("Mode=3\n0.005 1000\npar\n")
        f.write("lattice test\ns0\n0\n")
        for line in lattice_lines:
            f.write(line + "\n")
        for line in strain_lines:
            f.write(line + "\n")
        f.write("1\n1 1 1\nF\n-1 0 0 0 0 0 0\n")
        f.write("NEWSYM=T\nLATTIC=1\nsg\nILAT=F\n-1313\nk1\n")


def _plv(tmp_path, name, lattice_lines, strain_lines=("0",)):
    d = os.path.join(tmp_path, name)
    _write(d, lattice_lines, list(strain_lines))
    sk = read_skin(os.path.join(d, "SKIN"))
    st = sk.structures[0][2]
    return np.array(st.plv, dtype=float), st.volume


def _ref_lattice(latnum, p):
    """setlat.f's primitive vectors, row i = vector i."""
    al = np.zeros((3, 3))
    t = abs(latnum)
    if t == 6:
        a, c = p if latnum > 0 else ((2 * abs(p[0]) / abs(p[1])) ** T3, None)
        if latnum < 0:
            c = p[1] * a
        al[0, 0] = al[1, 1] = a
        al[2] = [H * a, H * a, H * c]
    elif t == 8:
        if latnum > 0:
            a, b, c = p
        else:
            a = (abs(2 * p[0]) / abs(p[1] * p[2])) ** T3
            b, c = p[1] * a, p[2] * a
        al[0] = [H * a, -H * b, 0]
        al[1] = [H * a, H * b, 0]
        al[2] = [0, 0, c]
    elif t in (9, 10):
        if latnum > 0:
            a, c = p
        else:
            a = abs((2 if t == 9 else 4) * p[0] / p[1]) ** T3
            c = p[1] * a
        al[0] = [H * a, -H * a, 0]
        al[1] = [H * a, H * a, 0]
        al[2] = [0, 0, c] if t == 9 else [H * a, 0, H * c]
    elif t == 11:
        if latnum > 0:
            a, c = p
        else:
            a = (4 * abs(p[0]) / abs(p[1])) ** T3
            c = p[1] * a
        al[0] = [0, H * a, H * c]
        al[1] = [H * a, 0, H * c]
        al[2] = [H * a, H * a, 0]
    elif t == 12:
        if latnum > 0:
            a, b = p
        else:
            ct = math.cos(p[1])
            bo = T3 * (math.sqrt((1 + 2 * ct) / (1 - ct)) - 1)
            c = (abs(p[0]) / (1 + 3 * bo)) ** T3
            a, b = c * (1 + bo), c * bo
        al[:] = b
        np.fill_diagonal(al, a)
    elif t == 13:
        if latnum > 0:
            a, c = p
        else:
            a = (2 * abs(p[0]) / abs(p[1])) ** T3
            c = p[1] * a
        al[0] = [-H * a, H * a, H * c]
        al[1] = [H * a, -H * a, H * c]
        al[2] = [H * a, H * a, -H * c]
    elif t == 14:
        th = p[2]
        if latnum > 0:
            a, c = p[0], p[1]
        else:
            a = (p[0] / (p[1] * math.sin(th))) ** T3
            c = a * p[1]
        al[0] = [a * math.cos(th / 2), -a * math.sin(th / 2), 0]
        al[1] = [a * math.cos(th / 2), a * math.sin(th / 2), 0]
        al[2] = [0, 0, c]
    elif t in (15, 16):
        f = 0.5 if t == 15 else 0.25
        vol = f * p[0] ** 3 if latnum > 0 else p[0]
        w = (f * vol) ** T3
        sg = -1 if t == 15 else 1
        x, y, z = (w * math.exp(sg * p[1] * math.cos(p[2] + d)) for d in (2 * math.pi / 3, -2 * math.pi / 3, 0))
        if t == 15:
            al[0] = [0, y, z]
            al[1] = [x, 0, z]
            al[2] = [x, y, 0]
        else:
            al[0] = [-x, y, z]
            al[1] = [x, -y, z]
            al[2] = [x, y, -z]
    else:
        raise ValueError(latnum)
    return al


def _strained(al, e):
    est = np.diag(1 + np.asarray(e[:3], float))
    est[1, 2] = est[2, 1] = H * e[3]
    est[0, 2] = est[2, 0] = H * e[4]
    est[0, 1] = est[1, 0] = H * e[5]
    return al @ est


CASES = [
    (6, (5.1, 6.3)), (-6, (70.0, 1.2)),
    (8, (5.0, 6.0, 7.0)), (-8, (90.0, 1.1, 1.3)),
    (9, (5.0, 6.2)), (-9, (80.0, 1.15)),
    (10, (7.0, 7.7)), (-10, (85.0, 0.9)),
    (11, (7.1, 7.6)), (-11, (75.0, 1.05)),
    (12, (4.1, 1.3)), (-12, (66.0, 1.1)),
    (13, (5.3, 5.9)), (-13, (71.0, 1.2)),
    (14, (4.9, 6.1, 1.2)), (-14, (88.0, 1.3, 1.1)),
    (15, (5.4, 0.1, 0.4)), (-15, (78.0, 0.2, -0.3)),
    (16, (6.8, 0.15, 0.7)), (-16, (79.0, 0.05, 1.9)),
]


@pytest.mark.parametrize("latnum,p", CASES)
def test_lattice_types(tmp_path, latnum, p):
    plv, vol = _plv(str(tmp_path), "L%d" % latnum, ["%d" % latnum, " ".join("%.17g" % v for v in p)])
    ref = _ref_lattice(latnum, p)
    assert np.allclose(plv, ref, rtol=1e-14, atol=1e-13), (plv, ref)
    assert vol == pytest.approx(abs(np.linalg.det(ref)), rel=1e-13)
    if latnum < 0:
        # the volume forms produce the cell volume that was entered
        assert abs(np.linalg.det(plv)) == pytest.approx(abs(p[0]), rel=1e-12)


def _neighbours(plv, count):
    """Sorted distances of the nearest lattice points (excluding the origin)."""
    r = range(-3, 4)
    pts = np.array([i * plv[0] + j * plv[1] + k * plv[2] for i in r for j in r for k in r])
    d = np.sort(np.linalg.norm(pts, axis=1))[1:]
    return d[:count]


def test_special_lattices(tmp_path):
    tp = str(tmp_path)
    rm = math.log(2.0) / 3.0
    # magic strain around fcc at r = ln2/3, theta = 0: bcc with the entered a_bcc
    plv, _ = _plv(tp, "m15", ["15", "5.0 %.17g 0" % rm])
    d = _neighbours(plv, 14)
    assert np.allclose(d[:8], math.sqrt(3) / 2 * 5.0) and np.allclose(d[8:14], 5.0)
    # magic strain around bcc at the same r: fcc with the entered a_fcc
    plv, _ = _plv(tp, "m16", ["16", "7.0 %.17g 0" % rm])
    d = _neighbours(plv, 18)
    assert np.allclose(d[:12], 7.0 / math.sqrt(2)) and np.allclose(d[12:18], 7.0)
    # rhombohedron with a 60 degree angle: fcc of volume V
    plv, _ = _plv(tp, "r60", ["-12", "80.0 %.17g" % (math.pi / 3)])
    d = _neighbours(plv, 12)
    assert np.allclose(d, (4 * 80.0) ** T3 / math.sqrt(2))
    # body-centred tetragonals with c = a are bcc, face-centred ones fcc
    for lat in (6, 13):
        plv, _ = _plv(tp, "b%d" % lat, ["%d" % lat, "5.0 5.0"])
        assert np.allclose(_neighbours(plv, 8), math.sqrt(3) / 2 * 5.0)
    for lat in (10, 11):
        plv, _ = _plv(tp, "f%d" % lat, ["%d" % lat, "7.0 7.0"])
        assert np.allclose(_neighbours(plv, 12), 7.0 / math.sqrt(2))


STRAINS = [
    ("2", "0.0016", lambda x: (math.sqrt((1 + 0.04) / (1 - 0.04)) - 1, math.sqrt((1 - 0.04) / (1 + 0.04)) - 1, 0, 0, 0, 0), True),
    ("-2", "0.0016", lambda x: (0.04, -0.04, 0.0016 / (1 - 0.0016), 0, 0, 0), False),
    ("21", "-0.03", lambda x: (math.sqrt(0.97 / 1.03) - 1, math.sqrt(1.03 / 0.97) - 1, 0, 0, 0, 0), True),
    ("-21", "0.03", lambda x: (0.03, -0.03, 0.0009 / (1 - 0.0009), 0, 0, 0), False),
    ("3", "0.0025", lambda x: (math.sqrt(1 + 0.0025 / 4) - 1, math.sqrt(1 + 0.0025 / 4) - 1, 0, 0, 0, 0.05), True),
    ("-3", "0.0025", lambda x: (0, 0, 0.0025 / (4 - 0.0025), 0, 0, 0.05), False),
    ("4", "0.06", lambda x: (1.06 ** -T3 - 1, 1.06 ** -T3 - 1, 1.06 ** (2 / 3) - 1, 0, 0, 0), True),
    ("5", "0.02", lambda x: ((1.02) * 1.06 ** -T3 - 1,) * 3 + (2 * 0.02 * 1.06 ** -T3,) * 3, False),
    ("6", "-0.0004", lambda x: (0, 0, 0.0001, -0.02, 0, 0), False),
]


@pytest.mark.parametrize("opt,val,efun,conserving", STRAINS)
def test_strain_menus(tmp_path, opt, val, efun, conserving):
    base = ["4", "5.0"]                                     # simple cubic, a = 5
    plv, vol = _plv(str(tmp_path), "s" + opt.replace("-", "m"), base, [opt, val])
    e = efun(None)
    ref = _strained(5.0 * np.eye(3), e)
    assert np.allclose(plv, ref, rtol=1e-14, atol=1e-13), (plv, ref)
    if conserving:
        assert vol == pytest.approx(125.0, rel=1e-12)


def test_unknown_strain_is_an_error(tmp_path):
    d = os.path.join(str(tmp_path), "bad")
    _write(d, ["4", "5.0"], ["7", "0.1"])
    with pytest.raises(RuntimeError):
        read_skin(os.path.join(d, "SKIN"))
