"""Generate the golden fixtures under tests/golden/*.npz.

An independent, loop-by-loop transliteration of the reference Fortran in
pure Python with numpy float32 scalars (one rounding per operation, Fortran
left-to-right evaluation, 1-based arrays). It is deliberately written
without reference to the C oracle so that the two restatements check each
other: tests/test_oracle_golden.py requires the C oracle to reproduce every
fixture bit for bit.

Routines transliterated (mrowan137/tristan-mp-pu-master_densdecomp):
  mover_{1,2,3}ord        code/particles_movedeposit.F90:356-1271
  densdecomp_{1,2,3}ord   code/particles.F90:678-1358
  deposit_particles       code/particles_movedeposit.F90:1281-2051
  advance_b_halfstep      code/fields.F90:586-728
  advance_e_fullstep      code/fields.F90:739-870
  bc_b1 (periodic)        code/fieldboundaries.F90:181-263, :714-785
  exchange_current        code/fieldboundaries.F90:1768-2189
  apply_filter1_opt       code/filter.F90:8-221
  reorder_particles_      code/particles.F90:406-497

Run:  python tests/golden/make_golden.py     (writes the .npz files here)
"""
from __future__ import annotations

import os

import numpy as np

F = np.float32
HERE = os.path.dirname(os.path.abspath(__file__))

half, one, two, quart = F(1) / F(2), F(1.0), F(2.0), F(1) / F(4)
thhalf, nineighth, twoth = F(3) / F(2), F(9) / F(8), F(2) / F(3)
third, sixth, negsixth, negone = F(1) / F(3), F(1) / F(6), -(F(1) / F(6)), F(-1.0)


class Grid:
    """1-based Fortran arrays a[i, j, k], i in 1..mx."""

    def __init__(self, dims, order, nx, ny, nz):
        self.dims, self.order = dims, order
        self.nghost = 5 if order == 1 else 7
        self.nghostz = 5 if dims == 2 else self.nghost
        self.mx, self.my = nx + self.nghost, ny + self.nghost
        self.mz = 1 if dims == 2 else nz + self.nghostz
        self.iy = self.mx
        self.iz = 0 if dims == 2 else self.mx * self.my

    def new(self):
        return np.zeros((self.mx + 1, self.my + 1, self.mz + 1), np.float32)

    def flat(self, a):
        return np.ascontiguousarray(a[1:, 1:, 1:].transpose(2, 1, 0)).ravel()

    def unflat(self, v):
        a = self.new()
        a[1:, 1:, 1:] = v.reshape(self.mz, self.my, self.mx).transpose(2, 1, 0)
        return a

    def lin(self, l):
        """1-based linear index (Fortran sequence association) -> (i,j,k)."""
        l0 = l - 1
        return l0 % self.mx + 1, (l0 // self.mx) % self.my + 1, l0 // (self.mx * self.my) + 1


def aint(x):
    return int(np.trunc(x))


# --- form factors, written out per order as the Fortran has them ---------
def ff(order, d, S, o):
    """fill S (dict slot->weight) for offset d with slot shift o;
    returns (min, max)."""
    if order == 1:
        S[3 + o] = F(1.0) - d
        S[4 + o] = d
        return 3 + o, 4 + o
    if order == 2:
        if d <= half:
            S[2 + o] = half * (d * d - d + quart)
            S[4 + o] = S[2 + o] + d
            S[3 + o] = one - S[4 + o] - S[2 + o]
            return 2 + o, 4 + o
        S[3 + o] = nineighth - thhalf * d + half * d * d
        S[5 + o] = S[3 + o] - one + d
        S[4 + o] = one - S[5 + o] - S[3 + o]
        return 3 + o, 5 + o
    if d <= half:
        S[2 + o] = negsixth * (d - one) * (d - one) * (d - one)
        S[3 + o] = twoth + half * (d - two) * d * d
        S[5 + o] = sixth * d * d * d
        S[4 + o] = one - S[5 + o] - S[3 + o] - S[2 + o]
    else:
        S[5 + o] = sixth * d * d * d
        S[4 + o] = twoth + half * (negone - d) * (one - d) * (one - d)
        S[2 + o] = sixth * (one - d) * (one - d) * (one - d)
        S[3 + o] = one - S[5 + o] - S[4 + o] - S[2 + o]
    return 2 + o, 5 + o


def zeros6():
    return {k: F(0.0) for k in range(0, 8)}


# --- movers ------------------------------------------------------------
def mover(g, fl, parts, qm, c):
    ex, ey, ez, bx, by, bz = fl
    c = F(c)
    qm = F(qm)
    cinv = F(1.0) / c
    if g.dims == 3:
        def cs(a, d):
            return np.roll(a[1:, 1:, 1:], 1, axis=d)
        P = {}
        for nm, a in (("ex", ex), ("ey", ey), ("ez", ez), ("bx", bx), ("by", by), ("bz", bz)):
            P[nm] = g.new()
        P["ex"][1:, 1:, 1:] = F(0.5) * (ex[1:, 1:, 1:] + cs(ex, 0))
        P["ey"][1:, 1:, 1:] = F(0.5) * (ey[1:, 1:, 1:] + cs(ey, 1))
        P["ez"][1:, 1:, 1:] = F(0.5) * (ez[1:, 1:, 1:] + cs(ez, 2))
        P["bx"][1:, 1:, 1:] = F(0.5) * (bx[1:, 1:, 1:] + cs(bx, 1))
        P["by"][1:, 1:, 1:] = F(0.5) * (by[1:, 1:, 1:] + cs(by, 0))
        bzs = bz[1:, 1:, 1:]
        P["bz"][1:, 1:, 1:] = F(0.5) * (F(0.5) * (bzs + cs(bz, 0)) +
                                        F(0.5) * (np.roll(bzs, 1, axis=1) + np.roll(np.roll(bzs, 1, axis=1), 1, axis=0)))
    out = []
    for p in parts:
        x, y, z, u, v, w = (F(p[k]) for k in ("x", "y", "z", "u", "v", "w"))
        ip = aint(x); dxp = x - F(ip)
        jp = aint(y); dyp = y - F(jp)
        kp = aint(z)
        id_ = aint(x - half); dxd = x - half - F(id_)
        jd = aint(y - half); dyd = y - half - F(jd)
        kd = aint(z - half)
        Sxp, Syp, Szp, Sxd, Syd, Szd = (zeros6() for _ in range(6))
        a1, b1 = ff(g.order, dxp, Sxp, 0)
        a2, b2 = ff(g.order, dyp, Syp, 0)
        if g.dims == 3:
            dzp = z - F(kp)
            dzd = (z - half) - F(kd)
            a3, b3 = ff(g.order, dzp, Szp, 0)
        a1, b1 = ff(g.order, dxd, Sxd, 0)
        a2, b2 = ff(g.order, dyd, Syd, 0)
        if g.dims == 3:
            a3, b3 = ff(g.order, dzd, Szd, 0)
        acc = {k: F(0.0) for k in ("ex", "ey", "ez", "bx", "by", "bz")}
        if g.dims == 3:
            for i3 in range(a3, b3 + 1):
                for i2 in range(a2, b2 + 1):
                    for nm in ("ex", "ey", "ez", "bx", "by", "bz"):
                        s = F(0.0)
                        for i1 in range(a1, b1 + 1):
                            s = s + P[nm][ip - 3 + i1, jp - 3 + i2, kp - 3 + i3] * Sxp[i1]
                        acc[nm] = acc[nm] + s * Syp[i2] * Szp[i3]
        else:
            for i2 in range(a2, b2 + 1):
                for i1 in range(a1, b1 + 1):
                    lpp = (ip - 3 + i1) + g.iy * (jp - 3 + i2 - 1)
                    lpd = (ip - 3 + i1) + g.iy * (jd - 3 + i2 - 1)
                    ldp = (id_ - 3 + i1) + g.iy * (jp - 3 + i2 - 1)
                    ldd = (id_ - 3 + i1) + g.iy * (jd - 3 + i2 - 1)
                    acc["ex"] = acc["ex"] + ex[g.lin(ldp)] * Sxd[i1] * Syp[i2]
                    acc["ey"] = acc["ey"] + ey[g.lin(lpd)] * Sxp[i1] * Syd[i2]
                    acc["ez"] = acc["ez"] + ez[g.lin(lpp)] * Sxp[i1] * Syp[i2]
                    acc["bx"] = acc["bx"] + bx[g.lin(lpd)] * Sxp[i1] * Syd[i2]
                    acc["by"] = acc["by"] + by[g.lin(ldp)] * Sxd[i1] * Syp[i2]
                    acc["bz"] = acc["bz"] + bz[g.lin(ldd)] * Sxd[i1] * Syd[i2]
        ex0 = F(0.5) * acc["ex"] * qm
        ey0 = F(0.5) * acc["ey"] * qm
        ez0 = F(0.5) * acc["ez"] * qm
        bx0 = F(0.5) * acc["bx"] * qm * cinv
        by0 = F(0.5) * acc["by"] * qm * cinv
        bz0 = F(0.5) * acc["bz"] * qm * cinv
        u0 = c * u + ex0
        v0 = c * v + ey0
        w0 = c * w + ez0
        gg = c / np.sqrt(c * c + u0 * u0 + v0 * v0 + w0 * w0)
        bx0, by0, bz0 = gg * bx0, gg * by0, gg * bz0
        f = F(2.0) / (F(1.0) + bx0 * bx0 + by0 * by0 + bz0 * bz0)
        u1 = (u0 + v0 * bz0 - w0 * by0) * f
        v1 = (v0 + w0 * bx0 - u0 * bz0) * f
        w1 = (w0 + u0 * by0 - v0 * bx0) * f
        u0 = u0 + v1 * bz0 - w1 * by0 + ex0
        v0 = v0 + w1 * bx0 - u1 * bz0 + ey0
        w0 = w0 + u1 * by0 - v1 * bx0 + ez0
        un, vn, wn = u0 * cinv, v0 * cinv, w0 * cinv
        gg = c / np.sqrt(c * c + u0 * u0 + v0 * v0 + w0 * w0)
        out.append((x + un * gg * c, y + vn * gg * c, z + wn * gg * c, un, vn, wn))
    return np.array(out, np.float32)


# --- Esirkepov deposit -------------------------------------------------------
def densdecomp(g, cur, x2, y2, z2, x1, y1, z1, q):
    curx, cury, curz = cur
    i1, i2, j1, j2, k1, k2 = aint(x1), aint(x2), aint(y1), aint(y2), aint(z1), aint(z2)
    si, sj, sk = i2 - i1, j2 - j1, k2 - k1
    dx1, dy1 = x1 - F(aint(x1)), y1 - F(aint(y1))
    dx2, dy2 = x2 - F(aint(x2)), y2 - F(aint(y2))
    dz1, dz2 = z1 - F(aint(z1)), z2 - F(aint(z2))
    deltaz = z2 - z1
    Sx1, Sx2, Sy1, Sy2, Sz1, Sz2 = (zeros6() for _ in range(6))
    if g.dims == 2:
        k1, sk = 1, 0
    ax1, bx1 = ff(g.order, dx1, Sx1, 0)
    ay1, by1 = ff(g.order, dy1, Sy1, 0)
    if g.dims == 3:
        az1, bz1 = ff(g.order, dz1, Sz1, 0)
    ax2, bx2 = ff(g.order, dx2, Sx2, si)
    ay2, by2 = ff(g.order, dy2, Sy2, sj)
    if g.dims == 3:
        az2, bz2 = ff(g.order, dz2, Sz2, sk)
    xr = range(min(ax1, ax2), max(bx1, bx2) + 1)
    yr = range(min(ay1, ay2), max(by1, by2) + 1)
    cxp = F(0.0)
    cyps = zeros6()
    cya = zeros6()
    if g.dims == 3:
        czps = {(a, b): F(0.0) for a in range(8) for b in range(8)}
        cza = {(a, b): F(0.0) for a in range(8) for b in range(8)}
        for it2 in range(min(az1, az2), max(bz1, bz2) + 1):
            for it1 in yr:
                for it in xr:
                    l2 = (i1 - 3 + it) + (j1 - 3 + it1 - 1) * g.iy + (k1 - 3 + it2 - 1) * g.iz
                    dSx, dSy, dSz = Sx2[it] - Sx1[it], Sy2[it1] - Sy1[it1], Sz2[it2] - Sz1[it2]
                    cxa = q * (dSx * (Sy1[it1] * Sz1[it2] + half * dSy * Sz1[it2] + half * Sy1[it1] * dSz +
                                      third * dSy * dSz)) + cxp
                    cya[it] = q * (dSy * (Sx1[it] * Sz1[it2] + half * dSx * Sz1[it2] + half * Sx1[it] * dSz +
                                          third * dSx * dSz)) + cyps[it]
                    cza[(it, it1)] = q * (dSz * (Sx1[it] * Sy1[it1] + half * dSx * Sy1[it1] + half * Sx1[it] * dSy +
                                                 third * dSx * dSy)) + czps[(it, it1)]
                    ijk = g.lin(l2)
                    curx[ijk] = curx[ijk] + cxa
                    cury[ijk] = cury[ijk] + cya[it]
                    curz[ijk] = curz[ijk] + cza[(it, it1)]
                    cxp = cxa
                cyps = dict(cya)
                cya = zeros6()
            czps = dict(cza)
            cza = {(a, b): F(0.0) for a in range(8) for b in range(8)}
    else:
        for it1 in yr:
            for it in xr:
                l2 = (i1 - 3 + it) + (j1 - 3 + it1 - 1) * g.iy
                dSx, dSy = Sx2[it] - Sx1[it], Sy2[it1] - Sy1[it1]
                cxa = q * (dSx * (Sy1[it1] + half * dSy)) + cxp
                cya[it] = q * (dSy * (Sx1[it] + half * dSx)) + cyps[it]
                cz = -(q * deltaz * (Sx1[it] * Sy1[it1] + half * dSx * Sy1[it1] + half * Sx1[it] * dSy +
                                     third * dSx * dSy))
                ijk = g.lin(l2)
                curx[ijk] = curx[ijk] + cxa
                cury[ijk] = cury[ijk] + cya[it]
                curz[ijk] = curz[ijk] + cz
                cxp = cxa
            cyps = dict(cya)
            cya = zeros6()


def deposit_particles(g, cur, parts, qs, c):
    """deposit loop of one species, then the periodic wrap; returns the
    wrapped positions (sizex = sizey = 1, all axes periodic)."""
    c = F(c)
    for p in parts:
        x, y, z, u, v, w, ch = (F(p[k]) for k in ("x", "y", "z", "u", "v", "w", "ch"))
        invgam = F(1.0) / np.sqrt(F(1) + u * u + v * v + w * w)
        x0 = x - u * invgam * c
        y0 = y - v * invgam * c
        z0 = z - w * invgam * c
        densdecomp(g, cur, x, y, z, x0, y0, z0, ch * F(qs))
    ng, ngz = g.nghost, g.nghostz
    maxx, minx = F(g.mx) - F(ng // 2), F(ng // 2 + 1)
    maxy, miny = F(g.my) - F(ng // 2), F(ng // 2 + 1)
    if g.dims == 3:
        maxz, minz = F(g.mz) - F(ngz // 2), F(ngz // 2 + 1)
    else:
        minz = F(ngz // 2 + 1)
        maxz = minz + F(1)
    midx, midy, midz = F(0.5) * (maxx - minx), F(0.5) * (maxy - miny), F(0.5) * (maxz - minz)
    out = []
    for p in parts:
        x, y, z = F(p["x"]), F(p["y"]), F(p["z"])
        perx = pery = perz = F(0)
        if x < minx or x > maxx:
            perx = np.copysign(midx, x - minx) + np.copysign(midx, x - maxx)
        if y < miny or y > maxy:
            pery = np.copysign(midy, y - miny) + np.copysign(midy, y - maxy)
        if z < minz or z > maxz:
            perz = np.copysign(midz, z - minz) + np.copysign(midz, z - maxz)
        if g.dims == 3 and perz < 0:
            perz = -(F(g.mz) - F(ngz))
        out.append((x - perx, y - pery, z - perz))
    return np.array(out, np.float32)


# --- fields ---------------------------------------------------------------
def advance_b(g, fl, corr, c):
    ex, ey, ez, bx, by, bz = fl
    cst = F(corr) * (F(0.5) * F(c))
    ng, ngz = g.nghost, g.nghostz
    kr = range(ngz // 2 + 1, g.mz - (ngz // 2 + 1) + 1) if g.dims == 3 else range(1, 2)
    for k in kr:
        for j in range(ng // 2 + 1, g.my - (ng // 2 + 1) + 1):
            for i in range(ng // 2 + 1, g.mx - (ng // 2 + 1) + 1):
                if g.dims == 3:
                    bx[i, j, k] = bx[i, j, k] + cst * (ey[i, j, k + 1] - ey[i, j, k] - ez[i, j + 1, k] + ez[i, j, k])
                    by[i, j, k] = by[i, j, k] + cst * (ez[i + 1, j, k] - ez[i, j, k] - ex[i, j, k + 1] + ex[i, j, k])
                    bz[i, j, k] = bz[i, j, k] + cst * (ex[i, j + 1, k] - ex[i, j, k] - ey[i + 1, j, k] + ey[i, j, k])
                else:
                    bx[i, j, k] = bx[i, j, k] + cst * (-ez[i, j + 1, k] + ez[i, j, k])
                    by[i, j, k] = by[i, j, k] + cst * (ez[i + 1, j, k] - ez[i, j, k])
                    bz[i, j, k] = bz[i, j, k] + cst * (ex[i, j + 1, k] - ex[i, j, k] - ey[i + 1, j, k] + ey[i, j, k])


def advance_e(g, fl, corr, c):
    ex, ey, ez, bx, by, bz = fl
    cst = F(corr) * F(c)
    ng, ngz = g.nghost, g.nghostz
    kr = range(ngz // 2, g.mz + 1) if g.dims == 3 else range(1, 2)
    for k in kr:
        for j in range(ng // 2 + 1, g.my - (ng // 2 + 1) + 1):
            for i in range(ng // 2 + 1, g.mx - (ng // 2 + 1) + 1):
                if g.dims == 3:
                    ex[i, j, k] = ex[i, j, k] + cst * (by[i, j, k - 1] - by[i, j, k] - bz[i, j - 1, k] + bz[i, j, k])
                    ey[i, j, k] = ey[i, j, k] + cst * (bz[i - 1, j, k] - bz[i, j, k] - bx[i, j, k - 1] + bx[i, j, k])
                    ez[i, j, k] = ez[i, j, k] + cst * (bx[i, j - 1, k] - bx[i, j, k] - by[i - 1, j, k] + by[i, j, k])
                else:
                    ex[i, j, k] = ex[i, j, k] + cst * (-bz[i, j - 1, k] + bz[i, j, k])
                    ey[i, j, k] = ey[i, j, k] + cst * (bz[i - 1, j, k] - bz[i, j, k])
                    ez[i, j, k] = ez[i, j, k] + cst * (bx[i, j - 1, k] - bx[i, j, k] - by[i - 1, j, k] + by[i, j, k])


def _copy(g, arrs, axis, lt, ls, nt, ns):
    sl = [slice(None)] * 3
    for a in arrs:
        d, s = list(sl), list(sl)
        d[axis], s[axis] = lt, ls
        a[tuple(d)] = a[tuple(s)]
    for a in arrs:
        d, s = list(sl), list(sl)
        d[axis], s[axis] = nt, ns
        a[tuple(d)] = a[tuple(s)]


def bc_periodic(g, arrs):
    ng, ngz = g.nghost, g.nghostz
    for it in range(1, ng // 2 + 1):
        _copy(g, arrs, 0, ng // 2 + 1 - it, g.mx - (ng // 2 + it), g.mx - (ng // 2 + 1) + it, ng // 2 + it)
    for it in range(1, ng // 2 + 1):
        _copy(g, arrs, 1, ng // 2 + 1 - it, g.my - (ng // 2 + it), g.my - (ng // 2 + 1) + it, ng // 2 + it)
    if g.dims == 3:
        for it in range(1, ngz // 2 + 1):
            _copy(g, arrs, 2, ngz // 2 + 1 - it, g.mz - (ngz // 2 + it), g.mz - (ngz // 2 + 1) + it, ngz // 2 + it)


def exchange_current(g, cur, q5=False):
    ng, ngz = g.nghost, g.nghostz
    curx, cury, curz = cur

    def fold(a, axis, m, n, b1=None):
        sl = lambda lo, hi: tuple(slice(lo, hi + 1) if d == axis else slice(1, None) for d in range(3))
        buf1 = a[sl(m - n // 2, m)].copy() if b1 is None else b1
        buf2 = a[sl(1, n // 2)].copy()
        a[sl(n // 2 + 1, n)] = a[sl(n // 2 + 1, n)] + buf1
        a[sl(m - (n - 1), m - (n // 2 + 1))] = a[sl(m - (n - 1), m - (n // 2 + 1))] + buf2
        return buf1

    for a in cur:
        fold(a, 0, g.mx, ng)
    b = fold(curx, 1, g.my, ng)
    if q5:
        # the left-hand-side extent copies ng/2 rows; the last buffer row
        # keeps curx(:,my,:)
        b = b.copy()
        b[:, : ng // 2, :] = cury[1:, g.my - ng // 2: g.my, 1:]
        fold(cury, 1, g.my, ng, b1=b)
    else:
        fold(cury, 1, g.my, ng)
    fold(curz, 1, g.my, ng)
    if g.dims == 3:
        for a in cur:
            fold(a, 2, g.mz, ngz)


def apply_filter(g, cur, ntimes):
    ng, ngz = g.nghost, g.nghostz
    if g.dims == 2:
        winv = F(1.0) / F(16.0)
        wl, w0, wd = F(2.0) * winv, F(4.0) * winv, F(1.0) * winv
    else:
        winv = F(1.0) / F(64.0)
        wl, w0, wd = F(4.0) * winv, F(8.0) * winv, F(2.0) * winv
        wlz, wz, wdz = F(2.0) * winv, F(4.0) * winv, F(1.0) * winv
    for _ in range(ntimes):
        _copy(g, cur, 0, ng // 2, g.mx - (ng // 2 + 1), g.mx - ng // 2, ng // 2 + 1)
        _copy(g, cur, 1, ng // 2, g.my - (ng // 2 + 1), g.my - ng // 2, ng // 2 + 1)
        if g.dims == 3:
            _copy(g, cur, 2, ngz // 2, g.mz - (ngz // 2 + 1), g.mz - ngz // 2, ngz // 2 + 1)
        for comp, a in enumerate(cur):
            jhi = g.my - (ng // 2 + 1) + (2 if comp == 2 else 0)
            kr = range(ngz // 2 + 1, g.mz - (ngz // 2 + 1) + 1) if g.dims == 3 else range(1, 2)
            temp = {}
            for k in kr:
                for j in range(ng // 2 + 1, jhi + 1):
                    for i in range(ng // 2 + 1, g.mx - (ng // 2 + 1) + 1):
                        t = (wl * a[i - 1, j, k] + w0 * a[i, j, k] + wl * a[i + 1, j, k] + wl * a[i, j - 1, k] +
                             wl * a[i, j + 1, k] + wd * a[i - 1, j + 1, k] + wd * a[i + 1, j + 1, k] +
                             wd * a[i - 1, j - 1, k] + wd * a[i + 1, j - 1, k])
                        if g.dims == 3:
                            for kk in (k - 1, k + 1):
                                t = t + wlz * a[i - 1, j, kk] + wz * a[i, j, kk] + wlz * a[i + 1, j, kk] + \
                                    wlz * a[i, j - 1, kk] + wlz * a[i, j + 1, kk] + wdz * a[i - 1, j + 1, kk] + \
                                    wdz * a[i + 1, j + 1, kk] + wdz * a[i - 1, j - 1, kk] + wdz * a[i + 1, j - 1, kk]
                        temp[(i, j, k)] = t
            for (i, j, k), t in temp.items():
                a[i, j, k] = t


def reorder(g, parts):
    iy, iz = g.mx, (g.mx * g.my if g.dims == 3 else 0)
    keys = [int(p["x"]) + int(p["y"]) * iy + int(p["z"]) * iz for p in parts]
    order = sorted(range(len(parts)), key=lambda n: (keys[n], n))  # stable
    return parts[order]


# --- fixture generation -------------------------------------------------------
PDT = np.dtype([("x", "<f4"), ("y", "<f4"), ("z", "<f4"), ("u", "<f4"), ("v", "<f4"), ("w", "<f4"),
                ("ch", "<f4"), ("ind", "<i4"), ("proc", "<i4"), ("splitlev", "<i4")])


def random_particles(g, rng, n, spread=0.4):
    ng, ngz = g.nghost, g.nghostz
    p = np.zeros(n, PDT)
    p["x"] = rng.uniform(ng // 2 + 1, g.mx - ng // 2, n).astype(np.float32)
    p["y"] = rng.uniform(ng // 2 + 1, g.my - ng // 2, n).astype(np.float32)
    if g.dims == 3:
        p["z"] = rng.uniform(ngz // 2 + 1, g.mz - ngz // 2, n).astype(np.float32)
    else:
        p["z"] = rng.uniform(ngz // 2 + 1, ngz // 2 + 2, n).astype(np.float32)
    for k in ("u", "v", "w"):
        p[k] = (rng.standard_normal(n) * spread).astype(np.float32)
    p["u"][: n // 4] += np.float32(4.0)  # relativistic beam: crosses cells
    p["ch"] = 1.0
    p["ind"] = np.arange(1, n + 1)
    p["splitlev"] = 1
    # a few particles exactly on cell faces and half-cell points
    p["x"][-1] = np.float32(ng // 2 + 2)
    p["y"][-2] = np.float32(ng // 2 + 2.5)
    # particles about to leave through every face, so the periodic wrap
    # (and in 3D the z out-lists) are exercised
    lo = [ng // 2 + 1, ng // 2 + 1, ngz // 2 + 1]
    hi = [g.mx - ng // 2, g.my - ng // 2, (g.mz - ngz // 2) if g.dims == 3 else ngz // 2 + 2]
    for a, (k, mom) in enumerate((("x", "u"), ("y", "v"), ("z", "w"))):
        p[k][n // 4 + 2 * a] = np.float32(hi[a] - 0.05)
        p[mom][n // 4 + 2 * a] = np.float32(5.0)
        p[k][n // 4 + 2 * a + 1] = np.float32(lo[a] + 0.05)
        p[mom][n // 4 + 2 * a + 1] = np.float32(-5.0)
    return p


def main():
    rng = np.random.default_rng(20240607)
    c, corr, qm, q = 0.45, 1.025, -1.0, 3.8e-4
    for dims in (2, 3):
        for order in (1, 2, 3):
            n = 6 if dims == 3 else 10
            g = Grid(dims, order, n, n + 2, n - 1 if dims == 3 else 1)
            name = f"d{dims}o{order}"
            fl = [g.unflat(rng.standard_normal(g.mx * g.my * g.mz).astype(np.float32) * np.float32(0.05))
                  for _ in range(6)]
            parts = random_particles(g, rng, 24 if dims == 3 else 40)
            moved = mover(g, fl, parts, qm, c)
            # deposit + wrap from the moved particles
            dp = parts.copy()
            dp["x"], dp["y"], dp["z"] = moved[:, 0], moved[:, 1], moved[:, 2]
            dp["u"], dp["v"], dp["w"] = moved[:, 3], moved[:, 4], moved[:, 5]
            cur = [g.new() for _ in range(3)]
            wrapped = deposit_particles(g, cur, dp, q, c)
            dep = [g.flat(a) for a in cur]
            # field advances on the random fields
            fb = [a.copy() for a in fl]
            advance_b(g, fb, corr, c)
            fe = [a.copy() for a in fl]
            advance_e(g, fe, corr, c)
            fg = [a.copy() for a in fl[3:]]
            bc_periodic(g, fg)
            # fold and filter on random currents
            rc = [g.unflat(rng.standard_normal(g.mx * g.my * g.mz).astype(np.float32)) for _ in range(3)]
            fold = [a.copy() for a in rc]
            exchange_current(g, fold)
            foldq5 = [a.copy() for a in rc]
            exchange_current(g, foldq5, q5=True)
            filt = [a.copy() for a in fold]
            apply_filter(g, filt, 2)
            ro = reorder(g, dp)
            np.savez_compressed(
                os.path.join(HERE, f"golden_{name}.npz"),
                dims=dims, order=order, nx=g.mx - g.nghost, ny=g.my - g.nghost,
                nz=(g.mz - g.nghostz) if dims == 3 else 1, c=c, corr=corr, qm=qm, q=q,
                fields=np.stack([g.flat(a) for a in fl]), particles=parts, moved=moved,
                deposit=np.stack(dep), wrapped=wrapped,
                advance_b=np.stack([g.flat(a) for a in fb]), advance_e=np.stack([g.flat(a) for a in fe]),
                bc_b=np.stack([g.flat(a) for a in fg]), rand_cur=np.stack([g.flat(a) for a in rc]),
                fold=np.stack([g.flat(a) for a in fold]), fold_q5=np.stack([g.flat(a) for a in foldq5]),
                filter2=np.stack([g.flat(a) for a in filt]), reorder=ro)
            print("wrote", name)


if __name__ == "__main__":
    main()
