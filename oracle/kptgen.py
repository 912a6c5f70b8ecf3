"""CPU restatement of the reference's k-point mesh generator, test
infrastructure only (the checker of the C SKIN reader's generated meshes):

* kptin.f:94-136  reciprocal vectors and metric from the lattice vectors
* rdspgp.f:144-228  rotations in reciprocal-lattice coordinates (RSPCT)
* kptgen.f:1-286  mesh, Wigner-Seitz shift, sort by |k|, shells, star merging
* hsort.f, gdot.f, matmlt.f, mapk.f  the helpers, in their summation order
* kptin.f:292-346  information-only points, normalisation, KPST..KPEND

Matrices keep the Fortran indices: m[i][j] is M(i+1, j+1).
"""
import math

import numpy as np

TPI = 2.0 * math.pi


def matmlt(a, b):
    """matmlt.f: C = A B with c(i,k) = a(i,j) b(j,k) + c(i,k), j ascending."""
    c = [[0.0] * 3 for _ in range(3)]
    for k in range(3):
        for j in range(3):
            s = b[j][k]
            for i in range(3):
                c[i][k] = a[i][j] * s + c[i][k]
    return c


def gdot(a, b, g):
    d = 0.0
    for j in range(3):
        s = 0.0
        for i in range(3):
            s = s + a[i] * g[i][j]
        d = d + s * b[j]
    return d


def hsort(a):
    """hsort.f: heap-sort index list (1-based values)."""
    n = len(a)
    ind = list(range(1, n + 1))
    if n <= 1:
        return ind
    l, ir = n // 2 + 1, n
    while True:
        if l > 1:
            l -= 1
            indxt = ind[l - 1]
            q = a[indxt - 1]
        else:
            indxt = ind[ir - 1]
            q = a[indxt - 1]
            ind[ir - 1] = ind[0]
            ir -= 1
            if ir == 1:
                ind[0] = indxt
                return ind
        i, j = l, l + l
        while j <= ir:
            if j < ir and a[ind[j - 1] - 1] < a[ind[j] - 1]:
                j += 1
            if q < a[ind[j - 1] - 1]:
                ind[i - 1] = ind[j - 1]
                i, j = j, j + j
            else:
                j = ir + 1
        ind[i - 1] = indxt


def recip(plv):
    """AVEC(I,J) = PLV(J,I); BVEC columns are the reciprocal vectors; metric BIJ."""
    avec = [[plv[j][i] for j in range(3)] for i in range(3)]
    A = [avec[i][j] for j in range(3) for i in range(3)]
    B = [A[4] * A[8] - A[5] * A[7], A[5] * A[6] - A[3] * A[8], A[3] * A[7] - A[4] * A[6],
         A[7] * A[2] - A[8] * A[1], A[8] * A[0] - A[6] * A[2], A[6] * A[1] - A[7] * A[0],
         A[1] * A[5] - A[2] * A[4], A[2] * A[3] - A[0] * A[5], A[0] * A[4] - A[1] * A[3]]
    ws = A[0] * B[0] + A[1] * B[1] + A[2] * B[2]
    pre = TPI / ws
    bvec = [[0.0] * 3 for _ in range(3)]
    l = 0
    for j in range(3):
        for i in range(3):
            bvec[i][j] = pre * B[l]
            l += 1
    bij = [[0.0] * 3 for _ in range(3)]
    for j in range(3):
        for i in range(3):
            for k in range(3):
                bij[i][j] = bvec[k][i] * bvec[k][j] + bij[i][j]
    return avec, bvec, bij, abs(ws)


def read_spacegroup(path, ilat, lattic, avec, bvec):
    """rdspgp.f: RSPCT for every operation (translations not needed)."""
    lines = open(path).read().splitlines()
    nop = int(lines[0][10:15])
    tpiinv = 1.0 / TPI
    rspc = []
    if ilat:
        t = [[bvec[j][i] * tpiinv for j in range(3)] for i in range(3)]
        tinv = [[avec[i][j] for j in range(3)] for i in range(3)]
        vals, ln = [], 1
        while len(vals) < 9 * nop:
            s = lines[ln]
            ln += 1
            for f in range(18):
                fld = s[4 * f:4 * f + 4]
                if len(vals) < 9 * nop:
                    vals.append(float(fld) if fld.strip() else 0.0)
        for k in range(nop):
            rd = [[vals[9 * k + 3 * i + j] for j in range(3)] for i in range(3)]
            rspc.append(matmlt(tinv, matmlt(rd, t)))
    else:
        for k in range(nop):
            m = []
            for i in range(3):
                s = lines[1 + 3 * k + i]
                m.append([float(s[20 * j:20 * j + 20].replace("D", "E")) for j in range(3)])
            if lattic == 4:
                c32 = math.sqrt(3.0) / 2.0
                m = [[c32 if abs(v - c32) < 0.001 else (-c32 if abs(v + c32) < 0.001 else v) for v in row]
                     for row in m]
            rspc.append(m)
    t = [[avec[j][i] / TPI for j in range(3)] for i in range(3)]
    tinv = [[bvec[i][j] for j in range(3)] for i in range(3)]
    return [matmlt(t, matmlt(r, tinv)) for r in rspc]


def kptgen(plv, lattic, rspct, kdiv, lspec=False):
    avec, bvec, bij, wsvol = recip(plv)
    lbcc, lhex, ltet = lattic == 2, lattic == 4, lattic in (7, 8, 9)
    alat = 0.0
    if lbcc:
        alat = (2.0 * wsvol) ** 0.33333333333333333
        alat = 2.0 * TPI / alat
    k1, k2, k3 = kdiv
    if ltet:
        k1, k2 = 2 * k1, 2 * k2
    if lspec:
        if lhex:
            m1 = k1 + k1 % 2
            m2 = m1
            if k1 != k2:
                raise ValueError("KDIV error for hex lattice")
        else:
            m1, m2 = k1 + 1, k2 + 1
        m3 = k3 + 1
    else:
        m1, m2, m3 = k1, k2, k3
    f1, f2, f3 = 0.5 / k1, 0.5 / k2, 0.5 / k3
    tpiinv = 1.0 / TPI
    rk, rad, lin = [], [], []
    kin = 0
    for ii in range(-m1, m1 + 1, 2):
        for jj in range(-m2, m2 + 1, 2):
            for kk in range(-m3, m3 + 1, 2):
                uk = [f1 * ii, f2 * jj, f3 * kk]
                if lattic in (7, 8, 9):
                    uk[0], uk[1] = ii / k1, jj / k2
                    if lattic == 7:
                        uk[2] = uk[2] + 0.5 * (uk[0] - uk[1])
                    elif lattic == 8:
                        uk[2] = uk[2] + 0.5 * uk[0]
                    else:
                        uk[2] = uk[2] + 0.5 * (uk[0] + uk[1])
                u = list(uk)
                inn = -k1 < ii <= k1 and -k2 < jj <= k2 and -k3 < kk <= k3
                lin.append(inn)
                kin += inn
                if lbcc:
                    uu = [uk[j] * alat for j in range(3)]
                    u = [(uu[0] * avec[0][j] + uu[1] * avec[1][j] + uu[2] * avec[2][j]) * tpiinv for j in range(3)]
                r2, ut = 1e50, None
                for i1 in range(-3, 4):
                    for i2 in range(-3, 4):
                        for i3 in range(-3, 4):
                            uu = [u[0] + i1, u[1] + i2, u[2] + i3]
                            r = gdot(uu, uu, bij)
                            if r <= r2:
                                r2, ut = r, uu
                rk.append(ut)
                rad.append(r2)
    nk = len(rk)
    index = hsort(rad)
    srad = [rad[i - 1] for i in index]
    srk = [rk[i - 1] for i in index]
    f = 1.0 / kin
    r2 = srad[0] + 1e-4
    ist = [1]
    for j in range(2, nk + 1):
        if srad[j - 1] > r2:
            r2 = srad[j - 1] + 1e-4
            ist.append(j)
    ist.append(nk + 1)
    q, w = [], []
    for s in range(len(ist) - 1):
        first = len(q) + 1
        for j in range(ist[s], ist[s + 1]):
            ieq = 0
            xx, yy, zz = srk[j - 1]
            for k in range(first, len(q) + 1):
                u = q[k - 1]
                for r in rspct:
                    for i1 in (-1, 0, 1):
                        x = r[0][0] * u[0] + r[0][1] * u[1] + r[0][2] * u[2] + i1
                        for i2 in (-1, 0, 1):
                            y = r[1][0] * u[0] + r[1][1] * u[1] + r[1][2] * u[2] + i2
                            for i3 in (-1, 0, 1):
                                z = r[2][0] * u[0] + r[2][1] * u[1] + r[2][2] * u[2] + i3
                                if abs(x - xx) + abs(y - yy) + abs(z - zz) <= 1e-4:
                                    ieq = k
                                if ieq == 0 and abs(x + xx) + abs(y + yy) + abs(z + zz) <= 1e-4:
                                    ieq = k
            inmesh = lin[index[j - 1] - 1]
            if ieq == 0:
                q.append([xx, yy, zz])
                w.append(f if inmesh else 0.0)
            elif inmesh:
                w[ieq - 1] = w[ieq - 1] + f
    return np.array(q), np.array(w)


def kptin_mesh(plv, lattic, sgfile, ilat, kdiv, lspec=False, kpst=0, kpend=0, info=()):
    """kptin.f's mesh branch: generated points, information-only points, the
    weight normalisation and the KPST..KPEND selection, as the C reader does."""
    avec, bvec, _, _ = recip(plv)
    rspct = read_spacegroup(sgfile, ilat, lattic, avec, bvec)
    q, w = kptgen(plv, lattic, rspct, kdiv, lspec)
    q, w = [list(v) for v in q], list(w)
    for v in info:
        q.append(list(v))
        w.append(0.0)
    ws = 0.0
    for v in w:
        ws = ws + v
    if abs(ws - 1.0) > 1e-6:
        wi = 1.0 / ws
        w = [v * wi for v in w]
    nk = len(w)
    kpst = 1 if kpst <= 0 else kpst
    kpend = nk if kpend == 0 else kpend
    if kpst > 1 or kpend < nk:
        q, w = q[kpst - 1:kpend], w[kpst - 1:kpend]
        ws = 0.0
        for v in w:
            ws = ws + v
        ws = 1.0 / ws
    w = [v * ws for v in w]
    return np.array(q), np.array(w), rspct
