"""TEST INFRASTRUCTURE ONLY — CPU restatement of the reference's 2-D elastic
time step on the variable grid: the checker of the variable-grid elastic
GPU path (tests/test_gpu_vargrid_elastic.py).

Restates, on top of oracle/vargrid.py (layout, Dxf/Dxb/Dyf/Dyb, the
interface interpolations, CPML coefficients, density averages):

* the staggered-x y-derivatives DyfStaggeredX / DybStaggeredX
  (src/ForwardSolver/Derivatives/Derivatives.cpp:852-1011), whose taps shift
  in x by dhFactor/3 where the staggered point of the coarse layer sits at a
  different x (always zero-padded at the grid edges);
* the 4-point S-modulus average XY (src/Modelparameter/Modelparameter.cpp:
  449-533) with the vacuum rules of ModelparameterSeismic::
  calcAveragedSWaveModulus (ModelparameterSeismic.cpp:421-432);
* FD2Delastic::run with the variable-grid interpolations
  (src/ForwardSolver/ForwardSolver2Delastic.cpp:117-297) for CPML or no
  damping boundary, without a free surface.
"""
from __future__ import annotations

import numpy as np

from oracle import vargrid as vg


def _stag_rows(g: vg.VarGrid, y: int, c: int, n: int, orders, var_order: bool, forward: bool, fs: bool = False):
    """Taps [(C, Y, order, j, dh layer, image)] of one row of DyfStaggeredX / Z
    (forward) or DybStaggeredX / Z (Derivatives.cpp:852-1168): c is the row's
    coordinate along the staggered axis (x or z), n that axis' length, C the
    tap's coordinate along it. fs (backward only): DybStaggeredX /
    ZFreeSurface (Derivatives.cpp:533-704), the image coefficient
    c[order - 1 - (2 y)/f - j] subtracted where it exists (image -1: none;
    integer division as the reference's C++ evaluates it)."""
    layer = int(g.layer_y[y])
    order = orders[layer] if var_order else orders[0]
    dist = int(g.dist_y[y]) // g.dhf[layer]
    if dist == 0:
        order = 2
    elif order > dist * 2:
        order = dist * 2
    on = bool(g.on_iface_y[y])
    tr = int(g.trans_y[y])

    def iface(yy):
        return 0 <= yy < g.NY and bool(g.on_iface_y[yy])

    def trans(yy):
        return int(g.trans_y[yy])

    X = [c] * order
    out = []
    if forward:
        if on and tr == -1:
            f, dl = g.dhf[layer + 1], layer + 1
        else:
            f, dl = g.dhf[layer], layer
        if on and tr == 1 and X[0] >= f // 3:
            X[1] -= f // 3
        yq = y + (order // 2) * f
        if iface(yq) and trans(yq) == -1 and X[0] < n - f // 3:
            X[order - 1] += f // 3
        for j in range(order):
            Y = y + f * (j - order // 2 + 1)
            if 0 <= Y < g.NY:
                out.append((X[j], Y, order, j, dl, -1))
        return out
    f = g.dhf[layer]
    yq = y - (order // 2) * f
    if iface(yq) and trans(yq) == 1 and X[1] < n - f // 3:
        X[0] += f // 3
    if on and tr == -1 and X[1] >= f // 3:
        X[0] -= f // 3
    for j in range(order):
        Y = y + f * (j - order // 2)
        if on:
            if j == 0 and tr == 1:
                Y += g.dhf[layer - 1]
            if j == 1 and tr == -1:
                Y += g.dhf[layer + 1]
        img = order - 1 - (2 * y) // f - j if fs and order >= 1 + (2 * y) // f + j else -1
        if 0 <= Y < g.NY:
            out.append((X[j], Y, order, j, layer, img))
    return out


def staggered_operator(op: vg.Operators, orders, var_order: bool, forward: bool, axis: str = "x", fs: bool = False):
    """DyfStaggeredX / DybStaggeredX (axis "x") or DyfStaggeredZ /
    DybStaggeredZ (axis "z") times DT, as a CSR matrix (fs: the backward
    operators' free-surface variants). The rows of one depth y differ only at
    the edges of the staggered axis (the shifted taps are guarded by c >= f/3
    and c < n - f/3), so each (y, edge class) stencil is built once."""
    g = op.g
    n = g.NX if axis == "x" else g.NZ
    rows, cols, vals = [], [], []
    order_rows = np.argsort(g.y, kind="stable")
    bounds = np.searchsorted(g.y[order_rows], np.arange(g.NY + 1))
    for y in range(g.NY):
        r = order_rows[bounds[y]:bounds[y + 1]]
        if not len(r):
            continue
        layer = int(g.layer_y[y])
        f = g.dhf[layer] if not (g.on_iface_y[y] and g.trans_y[y] == -1 and forward) else g.dhf[layer + 1]
        cs = g.x[r] if axis == "x" else g.z[r]
        cls = (cs >= f // 3).astype(int) * 2 + (cs < n - f // 3).astype(int)
        for k in np.unique(cls):
            rr = r[cls == k]
            c_rep = int((g.x if axis == "x" else g.z)[rr[0]])
            for C, Y, o, j, dl, img in _stag_rows(g, y, c_rep, n, orders, var_order, forward, fs):
                dc = C - c_rep
                if axis == "x":
                    cols.append(g.coordinate2index(g.x[rr] + dc, Y, g.z[rr]))
                else:
                    cols.append(g.coordinate2index(g.x[rr], Y, g.z[rr] + dc))
                rows.append(rr)
                vals.append(np.full(len(rr), op._val(o, j, dl, img), dtype=op.dtype))
    return op._finish(rows, cols, vals)


def staggered_x_operator(op: vg.Operators, orders, var_order: bool, forward: bool):
    return staggered_operator(op, orders, var_order, forward, "x")


def shear_average_xy(g: vg.VarGrid, mu, dtype=np.float32):
    """calcAveragedSWaveModulus with the XY 4-point matrix
    (Modelparameter.cpp:449-533, ModelparameterSeismic.cpp:421-432): moduli
    below 1 raised to 1, their inverses averaged over the 4 points (2 at the
    bottom / right edge, 1 in the corner), the average inverted, results
    below 4 set to 0."""
    d = np.dtype(dtype).type
    mu = np.asarray(mu, dtype=dtype).copy()
    mu[mu < 1] = 1
    inv = (d(1) / mu).astype(dtype)
    f = np.array(g.dhf, dtype=np.int64)[g.layer]
    x2, y2 = g.x + f, g.y + f
    okx, oky = x2 < g.NX, y2 < g.NY
    out = np.zeros(g.N, dtype=dtype)
    q = d(0.25)
    h = d(0.5)
    full = okx & oky
    i = np.nonzero(full)[0]
    c2 = g.coordinate2index(x2[i], g.y[i], g.z[i])
    c3 = g.coordinate2index(g.x[i], y2[i], g.z[i])
    c4 = g.coordinate2index(x2[i], y2[i], g.z[i])
    s = (q * inv[i]).astype(dtype)
    s = (s + q * inv[c2]).astype(dtype)
    s = (s + q * inv[c3]).astype(dtype)
    out[i] = (s + q * inv[c4]).astype(dtype)
    b = np.nonzero(okx & ~oky)[0]          # bottom side: the point to the right
    cb = g.coordinate2index(x2[b], g.y[b], g.z[b])
    out[b] = (h * inv[cb] + h * inv[b]).astype(dtype)
    rgt = np.nonzero(~okx & oky)[0]        # right side: the point below
    cr = g.coordinate2index(g.x[rgt], y2[rgt], g.z[rgt])
    out[rgt] = (h * inv[cr] + h * inv[rgt]).astype(dtype)
    corner = np.nonzero(~okx & ~oky)[0]
    out[corner] = inv[corner]
    with np.errstate(divide="ignore"):
        av = (d(1) / out).astype(dtype)
    av[av < 4] = 0
    return av


def shear_average(g: vg.VarGrid, mu, pair: str, dtype=np.float32):
    """calcAveragedSWaveModulus with the 4-point matrix of the axis pair
    "xy", "xz" or "yz" (calc4PointAverageMatrixRow and calcAverageMatrixXY /
    XZ / YZ, Modelparameter.cpp:449-624; ModelparameterSeismic.cpp:421-432):
    the point and its neighbours f along each axis of the pair and along
    both (f the layer's dhFactor); with one axis past the grid the point and
    its neighbour along the other axis, with both past it the point alone;
    1/max(mu, 1) averaged, inverted, results below 4 set to 0."""
    d = np.dtype(dtype).type
    mu = np.asarray(mu, dtype=dtype).copy()
    mu[mu < 1] = 1
    inv = (d(1) / mu).astype(dtype)
    f = np.array(g.dhf, dtype=np.int64)[g.layer]
    c = {"x": g.x, "y": g.y, "z": g.z}
    n = {"x": g.NX, "y": g.NY, "z": g.NZ}
    a, b = pair[0], pair[1]

    def idx(sel, da, db):
        p = {k: c[k][sel].copy() for k in "xyz"}
        p[a] = p[a] + da * f[sel]
        p[b] = p[b] + db * f[sel]
        return g.coordinate2index(p["x"], p["y"], p["z"])

    oka, okb = c[a] + f < n[a], c[b] + f < n[b]
    out = np.zeros(g.N, dtype=dtype)
    q, h = d(0.25), d(0.5)
    i = np.nonzero(oka & okb)[0]
    s = (q * inv[i]).astype(dtype)
    s = (s + q * inv[idx(i, 1, 0)]).astype(dtype)
    s = (s + q * inv[idx(i, 0, 1)]).astype(dtype)
    out[i] = (s + q * inv[idx(i, 1, 1)]).astype(dtype)
    i = np.nonzero(oka & ~okb)[0]
    out[i] = (h * inv[idx(i, 1, 0)] + h * inv[i]).astype(dtype)
    i = np.nonzero(~oka & okb)[0]
    out[i] = (h * inv[idx(i, 0, 1)] + h * inv[i]).astype(dtype)
    i = np.nonzero(~oka & ~okb)[0]
    out[i] = inv[i]
    with np.errstate(divide="ignore"):
        av = (d(1) / out).astype(dtype)
    av[av < 4] = 0
    return av


def free_surface_scales(g: vg.VarGrid, M, mu, dtype=np.float32):
    """FreeSurfaceElastic::setModelparameter / init (FreeSurfaceElastic.cpp:
    11-88) on the grid's surface points (y = 0): scaleV = M - 2 mu,
    scaleH = -(M - 2 mu)^2 / M there, 0 elsewhere; fsZero 0 there, 1
    elsewhere."""
    d = np.dtype(dtype).type
    sel = (g.y == 0).astype(dtype)
    t = (M - (d(2) * mu).astype(dtype)).astype(dtype)
    scaleV = (sel * t).astype(dtype)
    t2 = ((t * t).astype(dtype) / M).astype(dtype)
    scaleH = (sel * (t2 * d(-1)).astype(dtype)).astype(dtype)
    return scaleH, scaleV, (d(1) - sel).astype(dtype)


class ElasticVarGrid2D:
    """FD2Delastic::run on a 2-D variable grid (ForwardSolver2Delastic.cpp:
    117-297), CPML or no damping boundary; with free_surface the image
    operators DybStaggeredXFreeSurface / DyfFreeSurface and the surface
    exchange (FreeSurface2Delastic.cpp:14-40)."""

    def __init__(self, g: vg.VarGrid, orders, DT: float, rho, vp, vs, cpml: dict | None,
                 src_idx, src_type, signals, rec_idx, rec_type, dtype=np.float32, var_order: bool = True,
                 edge: bool = True, var_grid: bool = True, free_surface: bool = False, damping=None):
        if g.NZ != 1:
            raise ValueError("2-D only")
        self.g, self.dtype, self.fs = g, dtype, free_surface
        self.damping = None if damping is None else np.asarray(damping, dtype=dtype)
        self.op = vg.Operators(g, orders, DT, free_surface, dtype, var_order, edge, var_grid)
        self.DyfSX = staggered_operator(self.op, orders, var_order, True, "x")
        self.DybSX = staggered_operator(self.op, orders, var_order, False, "x", free_surface)
        rho = np.asarray(rho, dtype=dtype)
        vp = np.asarray(vp, dtype=dtype)
        vs = np.asarray(vs, dtype=dtype)
        self.M = (rho * vp * vp).astype(dtype)
        self.mu = (rho * vs * vs).astype(dtype)
        self.muXY = shear_average_xy(g, self.mu, dtype)
        self.irx, self.iry = vg.inverse_density_averages(g, rho, dtype)
        if free_surface:
            self.scaleH, self.scaleV, self.fsZero = free_surface_scales(g, self.M, self.mu, dtype)
        self.cpml = cpml
        z = lambda: np.zeros(g.N, dtype=dtype)
        self.vx, self.vy, self.sxx, self.syy, self.sxy = z(), z(), z(), z(), z()
        self.psi = {k: z() for k in ("sxx_x", "sxy_y", "sxy_x", "syy_y", "vxx", "vyy", "vxy", "vyx")}
        self.src_idx = np.asarray(src_idx, np.int64)
        self.src_type = np.asarray(src_type)
        self.signals = np.asarray(signals, dtype=dtype)
        self.rec_idx = np.asarray(rec_idx, np.int64)
        self.rec_type = np.asarray(rec_type)

    def _cpml(self, upd, key, ax, half):
        if self.cpml is None:
            return upd
        af, bf, ah, bh = self.cpml[ax]
        a, b = (ah, bh) if half else (af, bf)
        ps = (self.psi[key] * b).astype(self.dtype)
        ps = (ps + (a * upd).astype(self.dtype)).astype(self.dtype)
        self.psi[key] = ps
        return (upd + ps).astype(self.dtype)

    def step(self, t: int):
        op, dt, d = self.op, self.dtype, np.dtype(self.dtype).type
        # velocities (CPML2D.cpp: sxx_x half-x, sxy_y full-y, sxy_x full-x, syy_y half-y)
        u = self._cpml(op.Dxf @ self.sxx, "sxx_x", "x", True)
        u2 = self._cpml(self.DybSX @ self.sxy, "sxy_y", "y", False)
        u = ((u + u2).astype(dt) * self.irx).astype(dt)
        self.vx = op.IStagX @ (self.vx + u).astype(dt)
        u = self._cpml(op.Dxb @ self.sxy, "sxy_x", "x", False)
        u2 = self._cpml(op.Dyf @ self.syy, "syy_y", "y", True)
        u = ((u + u2).astype(dt) * self.iry).astype(dt)
        self.vy = op.IFull @ (self.vy + u).astype(dt)
        # normal stresses
        vxx = self._cpml(op.Dxb @ self.vx, "vxx", "x", False)
        vyy = self._cpml(op.Dyb @ self.vy, "vyy", "y", False)
        u = ((vxx + vyy).astype(dt) * self.M).astype(dt)
        sxx = (self.sxx + u).astype(dt)
        syy = (self.syy + u).astype(dt)
        sxx = (sxx - (d(2.0) * (vyy * self.mu).astype(dt)).astype(dt)).astype(dt)
        syy = (syy - (d(2.0) * (vxx * self.mu).astype(dt)).astype(dt)).astype(dt)
        self.sxx = op.IFull @ sxx
        self.syy = op.IFull @ syy
        # shear stress (vxy half-y, vyx half-x)
        u = self._cpml(self.DyfSX @ self.vx, "vxy", "y", True)
        u2 = self._cpml(op.Dxf @ self.vy, "vyx", "x", True)
        u = ((u + u2).astype(dt) * self.muXY).astype(dt)
        self.sxy = op.IStagX @ (self.sxy + u).astype(dt)
        if self.fs:
            # exchangeHorizontalUpdate(vxx, vyy, Sxx), setSurfaceZero(Syy)
            self.sxx = (self.sxx + (self.scaleH * vxx).astype(dt)).astype(dt)
            self.sxx = (self.sxx - (self.scaleV * vyy).astype(dt)).astype(dt)
            self.syy = (self.syy * self.fsZero).astype(dt)
        if self.damping is not None:
            # DampingBoundary.apply(Sxx, Syy, Sxy, vX, vY)
            for k in ("sxx", "syy", "sxy", "vx", "vy"):
                setattr(self, k, (getattr(self, k) * self.damping).astype(dt))
        # sources and receivers (FDTD2Delastic.cpp:12-49)
        for s in range(len(self.src_idx)):
            i, v = self.src_idx[s], self.signals[s, t]
            if self.src_type[s] == 1:
                self.sxx[i] += v
                self.syy[i] += v
            elif self.src_type[s] == 2:
                self.vx[i] += v
            elif self.src_type[s] == 3:
                self.vy[i] += v
        out = np.zeros(len(self.rec_idx), dtype=dt)
        for r, (i, k) in enumerate(zip(self.rec_idx, self.rec_type)):
            if k == 1:
                out[r] = d((self.sxx[i] + self.syy[i]) * d(0.5))
            else:
                out[r] = (self.vx if k == 2 else self.vy)[i]
        return out

    def run(self, nt: int) -> np.ndarray:
        out = np.zeros((len(self.rec_idx), nt), dtype=self.dtype)
        for t in range(nt):
            out[:, t] = self.step(t)
        return out


class ElasticVarGrid3D:
    """FD3Delastic::run on a 3-D variable grid (ForwardSolver3Delastic.cpp:
    120-414), CPML or no damping boundary, no free surface: DybStaggeredX /
    DybStaggeredZ for the y-derivatives of sxy / syz in the velocity update,
    DyfStaggeredX / DyfStaggeredZ for those of vx / vz in the shear update,
    and the interface interpolations vx StaggeredX, vy Full, vz StaggeredZ,
    sxx / syy / szz Full, sxy StaggeredX, sxz StaggeredXZ, syz StaggeredZ
    (applied twice, as the reference does). With free_surface the image
    operators DybStaggeredX / ZFreeSurface and DyfFreeSurface and the surface
    exchange (FreeSurface3Delastic.cpp:15-47, ForwardSolver3Delastic.cpp:
    400-404)."""

    def __init__(self, g: vg.VarGrid, orders, DT: float, rho, vp, vs, cpml: dict | None,
                 src_idx, src_type, signals, rec_idx, rec_type, dtype=np.float32, var_order: bool = True,
                 edge: bool = True, var_grid: bool = True, free_surface: bool = False, damping=None):
        if g.NZ < 2:
            raise ValueError("3-D only")
        self.g, self.dtype, self.fs = g, dtype, free_surface
        self.damping = None if damping is None else np.asarray(damping, dtype=dtype)
        self.op = vg.Operators(g, orders, DT, free_surface, dtype, var_order, edge, var_grid)
        self.DyfSX = staggered_operator(self.op, orders, var_order, True, "x")
        self.DybSX = staggered_operator(self.op, orders, var_order, False, "x", free_surface)
        self.DyfSZ = staggered_operator(self.op, orders, var_order, True, "z")
        self.DybSZ = staggered_operator(self.op, orders, var_order, False, "z", free_surface)
        rho = np.asarray(rho, dtype=dtype)
        vp = np.asarray(vp, dtype=dtype)
        vs = np.asarray(vs, dtype=dtype)
        self.M = (rho * vp * vp).astype(dtype)
        self.mu = (rho * vs * vs).astype(dtype)
        self.muXY = shear_average(g, self.mu, "xy", dtype)
        self.muXZ = shear_average(g, self.mu, "xz", dtype)
        self.muYZ = shear_average(g, self.mu, "yz", dtype)
        self.irx, self.iry, self.irz = vg.inverse_density_averages(g, rho, dtype)
        if free_surface:
            self.scaleH, self.scaleV, self.fsZero = free_surface_scales(g, self.M, self.mu, dtype)
        self.cpml = cpml
        z = lambda: np.zeros(g.N, dtype=dtype)
        self.f = {k: z() for k in ("vx", "vy", "vz", "sxx", "syy", "szz", "sxy", "sxz", "syz")}
        self.psi = {k: z() for k in ("sxx_x", "sxy_y", "sxz_z", "sxy_x", "syy_y", "syz_z", "sxz_x", "syz_y", "szz_z",
                                     "vxx", "vyy", "vzz", "vxy", "vyx", "vxz", "vzx", "vyz", "vzy")}
        self.src_idx = np.asarray(src_idx, np.int64)
        self.src_type = np.asarray(src_type)
        self.signals = np.asarray(signals, dtype=dtype)
        self.rec_idx = np.asarray(rec_idx, np.int64)
        self.rec_type = np.asarray(rec_type)

    def _cpml(self, upd, key, ax, half):
        if self.cpml is None:
            return upd
        af, bf, ah, bh = self.cpml[ax]
        a, b = (ah, bh) if half else (af, bf)
        ps = (self.psi[key] * b).astype(self.dtype)
        ps = (ps + (a * upd).astype(self.dtype)).astype(self.dtype)
        self.psi[key] = ps
        return (upd + ps).astype(self.dtype)

    def _vel(self, terms, ir):
        dt = self.dtype
        u = None
        for mat, field, key, ax, half in terms:
            t = self._cpml(mat @ self.f[field], key, ax, half)
            u = t if u is None else (u + t).astype(dt)
        return (u * ir).astype(dt)

    def step(self, t: int):
        op, dt, d, F = self.op, self.dtype, np.dtype(self.dtype).type, self.f
        # velocities (CPML3D: forward derivatives take the half profiles)
        u = self._vel([(op.Dxf, "sxx", "sxx_x", "x", True), (self.DybSX, "sxy", "sxy_y", "y", False),
                       (op.Dzb, "sxz", "sxz_z", "z", False)], self.irx)
        F["vx"] = op.IStagX @ (F["vx"] + u).astype(dt)
        u = self._vel([(op.Dxb, "sxy", "sxy_x", "x", False), (op.Dyf, "syy", "syy_y", "y", True),
                       (op.Dzb, "syz", "syz_z", "z", False)], self.iry)
        F["vy"] = op.IFull @ (F["vy"] + u).astype(dt)
        u = self._vel([(op.Dxb, "sxz", "sxz_x", "x", False), (self.DybSZ, "syz", "syz_y", "y", False),
                       (op.Dzf, "szz", "szz_z", "z", True)], self.irz)
        F["vz"] = op.IStagZ @ (F["vz"] + u).astype(dt)
        # normal stresses
        vxx = self._cpml(op.Dxb @ F["vx"], "vxx", "x", False)
        vyy = self._cpml(op.Dyb @ F["vy"], "vyy", "y", False)
        vzz = self._cpml(op.Dzb @ F["vz"], "vzz", "z", False)
        u = ((((vxx + vyy).astype(dt) + vzz).astype(dt)) * self.M).astype(dt)
        sxx = (F["sxx"] + u).astype(dt)
        syy = (F["syy"] + u).astype(dt)
        szz = (F["szz"] + u).astype(dt)
        two = d(2.0)
        sxx = (sxx - (two * (((vyy + vzz).astype(dt)) * self.mu).astype(dt)).astype(dt)).astype(dt)
        syy = (syy - (two * (((vxx + vzz).astype(dt)) * self.mu).astype(dt)).astype(dt)).astype(dt)
        szz = (szz - (two * (((vxx + vyy).astype(dt)) * self.mu).astype(dt)).astype(dt)).astype(dt)
        F["sxx"], F["syy"], F["szz"] = op.IFull @ sxx, op.IFull @ syy, op.IFull @ szz
        # shear stresses
        u = self._vel([(self.DyfSX, "vx", "vxy", "y", True), (op.Dxf, "vy", "vyx", "x", True)], self.muXY)
        F["sxy"] = op.IStagX @ (F["sxy"] + u).astype(dt)
        u = self._vel([(op.Dzf, "vx", "vxz", "z", True), (op.Dxf, "vz", "vzx", "x", True)], self.muXZ)
        F["sxz"] = op.IStagXZ @ (F["sxz"] + u).astype(dt)
        u = self._vel([(op.Dzf, "vy", "vyz", "z", True), (self.DyfSZ, "vz", "vzy", "y", True)], self.muYZ)
        F["syz"] = op.IStagZ @ (op.IStagZ @ (F["syz"] + u).astype(dt))
        if self.fs:
            # setSurfaceZero(Syy), exchangeHorizontalUpdate(vxx + vzz, vyy, Sxx, Szz)
            upd = (vxx + vzz).astype(dt)
            F["syy"] = (F["syy"] * self.fsZero).astype(dt)
            tmp = (self.scaleH * upd).astype(dt)
            F["sxx"] = (F["sxx"] + tmp).astype(dt)
            F["szz"] = (F["szz"] + tmp).astype(dt)
            tmp = (self.scaleV * vyy).astype(dt)
            F["sxx"] = (F["sxx"] - tmp).astype(dt)
            F["szz"] = (F["szz"] - tmp).astype(dt)
        if self.damping is not None:
            # DampingBoundary.apply(Sxx, Syy, Szz, Sxy, Sxz, Syz, vX, vY, vZ)
            for k in ("sxx", "syy", "szz", "sxy", "sxz", "syz", "vx", "vy", "vz"):
                F[k] = (F[k] * self.damping).astype(dt)
        # sources and receivers (FDTD3Delastic.cpp:12-53)
        for k in range(len(self.src_idx)):
            i, v = self.src_idx[k], self.signals[k, t]
            if self.src_type[k] == 1:
                for c in ("sxx", "syy", "szz"):
                    F[c][i] += v
            elif self.src_type[k] in (2, 3, 4):
                F[("vx", "vy", "vz")[self.src_type[k] - 2]][i] += v
        out = np.zeros(len(self.rec_idx), dtype=dt)
        for r, (i, k) in enumerate(zip(self.rec_idx, self.rec_type)):
            if k == 1:
                out[r] = d((F["sxx"][i] + F["syy"][i] + F["szz"][i]) / d(3.0))
            else:
                out[r] = F[("vx", "vy", "vz")[k - 2]][i]
        return out

    def run(self, nt: int) -> np.ndarray:
        out = np.zeros((len(self.rec_idx), nt), dtype=self.dtype)
        for t in range(nt):
            out[:, t] = self.step(t)
        return out
