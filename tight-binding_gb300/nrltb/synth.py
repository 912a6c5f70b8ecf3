"""Seeded synthetic NRL tight-binding workloads.

The reference publishes no benchmark inputs, so the workloads are synthetic
structures and parameter sets with the shapes of the five configurations the
performance targets are quoted on:

  fcc1     fcc, a = 6.82 bohr, 1 atom, spd (N = 9), 12^3 MP mesh (1728 k), 11 e/atom
  bcc32    bcc 2x2x4 conventional cells (32 atoms), a = 5.42, sigma = 0.1 bohr
           Gaussian displacements, spd (N = 288), 4^3 MP mesh, 8 e/atom
  fcc128   fcc 4x4x2 conventional cells (128 atoms), a = 6.82, sigma = 0.1,
           spd (N = 1152), 3^3 MP mesh (27 k), 11 e/atom
  batch256 256 structures: fcc / bcc / sc supercells of 4-64 atoms, half spd and
           half sp3 (N = 16-576), MP meshes 2^3-5^3, sigma = 0.1
  b2_216   B2 binary 6x6x3 cubic cells (216 atoms), a = 5.5, species A spd and
           B sp3 (N = 1404), sigma = 0.15, Gamma-centred 2^3 mesh, kT = 0.01

Parameter draws (per species / species pair, from the structure's seed):
  density lambda ~ U[1.0, 1.3]
  on-site (s, p, t2g, eg): a = offset + U[-0.2, 0.2] with offsets (0, 0.6, -0.3,
     -0.2) Ry, b ~ U[-1, 1], c ~ U[-2, 2], d ~ U[-2, 2]
  cross-species on-site terms ~ U[-0.2, 0.2]
  each H and S bond integral (a + b R + c R^2) exp(-g^2 R): a ~ U[-1, 1] Ry,
     b, c ~ U[-0.2, 0.2], g ~ U[0.8, 1.2], for H and S alike
  cutoff dnn = 16.5 bohr, screening length 0.5 bohr
Random overlap integrals can make S(k) indefinite; the parameter seeds below
are ones whose S(k) has smallest eigenvalue above 0.05 on the configuration's
mesh (the rejection rule; the test suite re-checks it), so the seed of a
parameter set is part of the workload's definition.
k meshes are explicit lists (the reference's -1313 k-file path): Monkhorst-Pack
points u_j = (2j - n - 1) / (2n), or Gamma-centred u_j = j / n, in the
reciprocal-lattice basis, equal weights, i1-major order.
"""
import math
import os

import numpy as np

from .api import KMesh, Params, Structure

# Parameter seed of every single-configuration workload: its S(k) has smallest
# eigenvalue >= 0.19 on every k of each configuration's full mesh.
PARAM_SEED = 12
BATCH_SP3_SEED = 12

FCC_BASIS = np.array([[0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0]])
BCC_BASIS = np.array([[0, 0, 0], [.5, .5, .5]])
SC_BASIS = np.array([[0, 0, 0]])


def make_params(kbas_list, valence_list, seed, dnn=16.5, screenl=0.5, s_scale=1.0):
    """Draw one NRL parameter set for len(kbas_list) species (input.f layout)."""
    rng = np.random.default_rng(seed)
    kinds = len(kbas_list)
    n = kinds * (29 + 68 * kinds)
    p = np.zeros(n)
    offs = [0.0, 0.6, -0.3, -0.2]
    for k in range(kinds):
        ip = k * 17
        p[ip] = rng.uniform(1.0, 1.3)
        for o in range(4):
            p[ip + 1 + 4 * o] = offs[o] + rng.uniform(-0.2, 0.2)
            p[ip + 2 + 4 * o] = rng.uniform(-1, 1)
            p[ip + 3 + 4 * o] = rng.uniform(-2, 2)
            p[ip + 4 + 4 * o] = rng.uniform(-2, 2)
    ncross = 24 * (kinds * (kinds - 1) // 2)
    base = 17 * kinds
    p[base:base + ncross] = rng.uniform(-0.2, 0.2, ncross)
    base += ncross

    def bond(count, scale):
        out = []
        for _ in range(count):
            out += [scale * rng.uniform(-1, 1), scale * rng.uniform(-0.2, 0.2),
                    scale * rng.uniform(-0.2, 0.2), rng.uniform(0.8, 1.2)]
        return out

    nunlike = kinds * (kinds - 1) // 2
    blocks = []
    blocks += bond(10 * kinds, 1.0)          # like H
    blocks += bond(14 * nunlike, 1.0)        # unlike H
    blocks += bond(10 * kinds, s_scale)      # like S
    blocks += bond(14 * nunlike, s_scale)    # unlike S
    p[base:base + len(blocks)] = blocks
    assert base + len(blocks) == n
    nint = kinds * (kinds + 1) // 2
    return Params(kinds, np.array(kbas_list), np.array(valence_list, float),
                  np.full(nint, dnn), np.full(nint, screenl), p, 1, 0)


def magnetic_from(base, split=0.08):
    """A collinear spin-polarized set (jspins = 2) from a spin-restricted one:
    the spin-2 set equals it except for the on-site polynomials' constant terms,
    raised by `split` Ry (an exchange splitting), and the density parameters,
    scaled by 1.05; hopping and overlap integrals are shared."""
    p2 = base.param.copy()
    for k in range(base.kinds):
        ip = k * 17
        p2[ip] *= 1.05
        for o in range(4):
            p2[ip + 1 + 4 * o] += split
    return Params(base.kinds, base.kbas, base.valence, base.dnn, base.screenl,
                  np.concatenate([base.param, p2]), base.jsover, base.nltype, 2)


def make_magnetic_params(kbas_list, valence_list, seed, split=0.08, dnn=16.5, screenl=0.5):
    """make_params' set made spin-polarized by magnetic_from."""
    return magnetic_from(make_params(kbas_list, valence_list, seed, dnn=dnn, screenl=screenl), split)


def search_box(plv, dnn):
    """Smallest search box nd that finds every image within dnn (search2.f)."""
    vol = abs(np.linalg.det(plv))
    nd = []
    for i in range(3):
        c = np.cross(plv[(i + 1) % 3], plv[(i + 2) % 3])
        h = vol / np.linalg.norm(c)
        nd.append(int(math.ceil(dnn / h)) + 1)
    return tuple(nd)


def supercell(basis, a, reps, kinds_of_site, sigma, rng, dnn=16.5):
    nx, ny, nz = reps
    plv = np.diag([nx * a, ny * a, nz * a]).astype(float)
    pos, kk = [], []
    for i in range(nx):
        for j in range(ny):
            for k in range(nz):
                for b, frac in enumerate(basis):
                    pos.append((np.array([i, j, k]) + frac) * a)
                    kk.append(kinds_of_site(b))
    pos = np.array(pos)
    if sigma > 0:
        pos = pos + rng.normal(0.0, sigma, pos.shape)
    return Structure(np.array(kk, np.int32), pos, plv, search_box(plv, dnn),
                     abs(np.linalg.det(plv)), 0.0)


def mp_mesh(n, gamma=False):
    n1, n2, n3 = (n, n, n) if np.isscalar(n) else n
    axes = [(np.arange(m) / m) if gamma else (2 * np.arange(1, m + 1) - m - 1) / (2.0 * m)
            for m in (n1, n2, n3)]
    k = np.array([[a, b, c] for a in axes[0] for b in axes[1] for c in axes[2]])
    return KMesh(k, np.full(len(k), 1.0 / len(k)))


def fcc1(seed=11):
    a = 6.82
    plv = np.array([[0, a / 2, a / 2], [a / 2, 0, a / 2], [a / 2, a / 2, 0]])
    st = Structure(np.array([1], np.int32), np.zeros((1, 3)), plv, search_box(plv, 16.5),
                   abs(np.linalg.det(plv)), 0.0)
    par = make_params([9], [11.0], PARAM_SEED)
    return st, par, mp_mesh(12), dict(tkb=0.005)


def bcc32(seed=21):
    rng = np.random.default_rng(seed)
    st = supercell(BCC_BASIS, 5.42, (2, 2, 4), lambda b: 1, 0.1, rng)
    par = make_params([9], [8.0], PARAM_SEED)
    return st, par, mp_mesh(4), dict(tkb=0.005)


def fcc128(seed=31):
    rng = np.random.default_rng(seed)
    st = supercell(FCC_BASIS, 6.82, (4, 4, 2), lambda b: 1, 0.1, rng)
    par = make_params([9], [11.0], PARAM_SEED)
    return st, par, mp_mesh(3), dict(tkb=0.005)


def b2_216(seed=41):
    rng = np.random.default_rng(seed)
    st = supercell(BCC_BASIS, 5.5, (6, 6, 3), lambda b: 1 + b, 0.15, rng)
    par = make_params([9, 4], [10.0, 4.0], PARAM_SEED)
    return st, par, mp_mesh(2, gamma=True), dict(tkb=0.01)


def batch256(seed=51, count=256, spd_seed=PARAM_SEED, sp3_seed=BATCH_SP3_SEED):
    """List of (Structure, Params, KMesh, opts) of uneven size."""
    rng = np.random.default_rng(seed)
    par_spd = make_params([9], [10.0], spd_seed)
    par_sp3 = make_params([4], [4.0], sp3_seed)
    lattices = [(FCC_BASIS, 6.82), (BCC_BASIS, 5.42), (SC_BASIS, 4.6)]
    out = []
    for s in range(count):
        while True:
            basis, a = lattices[rng.integers(0, 3)]
            reps = tuple(int(x) for x in rng.integers(1, 5, 3))
            nat = len(basis) * reps[0] * reps[1] * reps[2]
            if 4 <= nat <= 64:
                break
        st = supercell(basis, a, reps, lambda b: 1, 0.1, rng)
        par = par_spd if s % 2 == 0 else par_sp3
        km = mp_mesh(int(rng.integers(2, 6)))
        out.append((st, par, km, dict(tkb=0.005)))
    return out


CONFIGS = {"fcc1": fcc1, "bcc32": bcc32, "fcc128": fcc128, "b2_216": b2_216}


# ---- writers in the reference's file formats ---------------------------------
def write_params(path, par, title="synthetic NRL parameters"):
    with open(path, "w") as f:
        # N non-orthogonal / O orthogonal (S parameters read, ignored); then N
        # spin-restricted / M magnetic (one parameter set per spin)
        f.write("%s%s%05d\n" % ("N" if par.jsover else "O", "M" if par.jspins == 2 else "N", par.nltype))
        f.write(title[:79] + "\n")
        f.write("%d\n" % par.kinds)
        for i in range(par.dnn.size):
            f.write("%.17g %.17g\n" % (par.dnn[i], par.screenl[i]))
        for k in range(par.kinds):
            f.write("%d\n1.0\n0.0 0.0 %.17g\n" % (par.kbas[k], par.valence[k]))
        for v in par.param:
            f.write("%.17e\n" % v)


def write_kfile(path, km):
    with open(path, "w") as f:
        f.write("%5d\n" % km.nk)
        for k, w in zip(km.k, km.w):
            f.write("%.17g %.17g %.17g %.17g\n" % (k[0], k[1], k[2], w))


def write_skin(dirname, entries, par, mode=4, tkb=0.005, eigcut=1e3):
    """SKIN + parameter file + one k file per structure (lattice type 0,
    Cartesian atoms entered with negative kinds as input1.f allows)."""
    os.makedirs(dirname, exist_ok=True)
    write_params(os.path.join(dirname, "par"), par)
    with open(os.path.join(dirname, "SKIN"), "w") as f:
        f.write("Mode=%d\n%.17g %.17g\npar\n" % (mode, tkb, eigcut))
        for i, (st, km) in enumerate(entries):
            kname = "k%03d" % i
            write_kfile(os.path.join(dirname, kname), km)
            open(os.path.join(dirname, "sg"), "w").write("identity\n")
            f.write("synthetic structure %d\n" % i)
            f.write("s%-19d\n" % i)
            f.write("%.17g\n" % st.zcharge)
            f.write("0\n")
            for v in st.plv:
                f.write("%.17g %.17g %.17g\n" % tuple(v))
            flips, noncol = st.flip is not None, st.spinat is not None
            # (2a1) lphonon, spin flag: T means a magdir (1 up, 2 flipped) per atom,
            # N a spin direction (theta, phi in degrees) per atom
            flag = "FN" if noncol else "FT" if flips else "F"
            f.write("1 1 1\n0\n%d\n%d %d %d\n%s\n" % ((st.natoms,) + tuple(st.nd) + (flag,)))
            for i, (kk, p, q) in enumerate(zip(st.kkind, st.posn, st.posq)):
                f.write("%d %.17g %.17g %.17g %.17g %.17g %.17g" % ((-int(kk),) + tuple(p) + tuple(q)))
                if noncol:
                    m = st.spinat[i]
                    f.write(" %.17g %.17g\n" % (math.degrees(math.acos(max(-1.0, min(1.0, m[2])))),
                                                 math.degrees(math.atan2(m[1], m[0]))))
                else:
                    f.write(" %d\n" % (2 if st.flip[i] else 1) if flips else "\n")
            f.write("NEWSYM=T\nLATTIC=1\nsg\nILAT=F\n-1313\n%s\n" % kname)
