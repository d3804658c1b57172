"""TEST INFRASTRUCTURE ONLY — CPU restatement of the reference's variable
(discontinuous) grid for the acoustic equations, the checker of the GPU
variable-grid path.

Only tests and ``__graft_entry__.smoke()`` import this module. It restates, in
numpy/scipy.sparse (FP32 as the reference's float build, or FP64):

* the layered grid and its index <-> coordinate maps
  (src/Acquisition/Coordinates.cpp:35-95 gridConfig reading, :119-245 layer
  set-up, :381-397 getLayer, :455-465 locatedOnInterface, :472-481
  distToInterface, :499-513 getTransition, :603-634 mapIndex2coordinate,
  :668-698 map3Dcoordinate2index);
* the sparse FD operators on that grid (src/ForwardSolver/Derivatives/
  Derivatives.cpp:129-188 Dxf, :210-282 Dyf, :304-362 Dzf, :367-430
  DyfFreeSurface, :706-765 Dxb, :771-845 Dyb, :1177-1245 Dzb; coefficients
  :2000-2042; DT scaling FDTD2D.cpp:193-229, FDTD3D.cpp:230-300) and the
  bilinear interface interpolations (:1252-1335 InterpolationFull,
  :1356-1440 InterpolationStaggeredX, :1462-1546 InterpolationStaggeredZ);
* the density averages (src/Modelparameter/Modelparameter.cpp:336-446,
  :633-640) and the per-layer CPML coefficients (src/ForwardSolver/
  BoundaryCondition/CPML.cpp:38-95, CPML2DAcoustic.cpp:105-210,
  CPML3DAcoustic.cpp);
* the acoustic time step with those operators (src/ForwardSolver/
  ForwardSolver2Dacoustic.cpp:91-190, ForwardSolver3Dacoustic.cpp:91-230).

Every operator row is assembled by the reference's own per-row rule. Rows
whose rule depends on the same inputs (the coordinate along the axis, the
layer and whether the row lies on an interface) share one stencil, which is
then broadcast to all of them, so the 3-D CI grid (about 10^6 points)
assembles in seconds.
"""
from __future__ import annotations

import math

import numpy as np
import scipy.sparse as sp

# Derivatives.cpp:2000-2042 (the Stencil1D values of each order)
FD_VALUES = {
    2: (-1.0, 1.0),
    4: (1.0 / 24.0, -9.0 / 8.0, 9.0 / 8.0, -1.0 / 24.0),
    6: (-3.0 / 640.0, 25.0 / 384.0, -75.0 / 64.0, 75.0 / 64.0, -25.0 / 384.0, 3.0 / 640.0),
    8: (5.0 / 7168.0, -49.0 / 5120.0, 245.0 / 3072.0, -1225.0 / 1024.0,
        1225.0 / 1024.0, -245.0 / 3072.0, 49.0 / 5120.0, -5.0 / 7168.0),
    10: (-8756999275442633.0 / 73786976294838206464.0, 8142668969129685.0 / 4611686018427387904.0,
         -567.0 / 40960.0, 735.0 / 8192.0, -19845.0 / 16384.0, 19845.0 / 16384.0, -735.0 / 8192.0,
         567.0 / 40960.0, -8142668969129685.0 / 4611686018427387904.0,
         8756999275442633.0 / 73786976294838206464.0),
    12: (6448335830095439.0 / 295147905179352825856.0, -1655620175512543.0 / 4611686018427387904.0,
         6842103786556949.0 / 2305843009213693952.0, -628618285389933.0 / 36028797018963968.0,
         436540475965291.0 / 4503599627370496.0, -2750204998582123.0 / 2251799813685248.0,
         2750204998582123.0 / 2251799813685248.0, -436540475965291.0 / 4503599627370496.0,
         628618285389933.0 / 36028797018963968.0, -6842103786556949.0 / 2305843009213693952.0,
         1655620175512543.0 / 4611686018427387904.0, -6448335830095439.0 / 295147905179352825856.0),
}


def cdiv(a: int, b: int) -> int:
    """C integer division (truncation toward zero)."""
    q = abs(a) // abs(b)
    return q if (a >= 0) == (b > 0) else -q


def cmod(a: int, b: int) -> int:
    """C remainder (sign of the dividend)."""
    return a - b * cdiv(a, b)


def read_grid_config(path: str):
    """gridConfigurationFilename columns: interface y, dhFactor, FD order
    (Coordinates.cpp:52-63, Derivatives.cpp:1663-1672)."""
    rows = []
    with open(path) as f:
        for line in f:
            s = line.strip()
            if not s or s.startswith("#"):
                continue
            rows.append([int(float(v)) for v in s.split()[:3]])
    iface = [r[0] for r in rows]
    dhf = [r[1] for r in rows]
    order = [r[2] for r in rows] if all(len(r) > 2 for r in rows) else None
    return iface, dhf, order


class VarGrid:
    """Coordinates<ValueType> of a variable grid (Coordinates.cpp:35-245)."""

    def __init__(self, NX: int, NY: int, NZ: int, DH: float, interfaces, dh_factors):
        iface = list(interfaces)
        if iface[0] != 0:
            raise ValueError("First interface must by at y=0")
        iface = iface[1:]
        dhf = list(dh_factors)
        for i in range(1, len(iface)):
            if iface[i] <= iface[i - 1]:
                raise ValueError("interface coordinates must increase")
        for i in range(1, len(dhf)):
            if dhf[i] not in (dhf[i - 1] * 3, dhf[i - 1] // 3, dhf[i - 1]) or (dhf[i] == dhf[i - 1] // 3 and dhf[i - 1] % 3):
                raise ValueError("Only gridspacing changes with factor 3 are allowed")
        nl = len(dhf)
        if len(iface) != nl - 1:
            raise ValueError("number of interfaces doesn't match to the number of different grid spacings")
        iface = [-1] + iface + [NY - 1]
        dhmax = max(dhf)
        for f in dhf:
            k = round(math.log(f) / math.log(3))
            if 3 ** k != f:
                raise ValueError("incompatible dhFactor, dhFactor must be 3^n")
        NXmax, NZmax = NX, NZ
        if dhmax != 1:
            while NXmax != (NXmax // dhmax) * dhmax + 1 + dhmax // 2:
                NXmax -= 1
            while NZ != 1 and NZmax != (NZmax // dhmax) * dhmax + 1 + dhmax // 2:
                NZmax -= 1
            NX, NZ = NXmax, NZmax
            layer = 0
            while layer < 1:
                layer += 1
                test = (iface[layer] - iface[layer - 1] - 1) / dhf[layer - 1]
                if math.floor(test) != test:
                    iface[layer] -= 1
                    layer -= 1
            layer = 1
            while layer < nl:
                layer += 1
                test = (iface[layer] - iface[layer - 1]) / dhf[layer - 1]
                if math.floor(test) != test:
                    iface[layer] -= 1
                    layer -= 1
        NY = iface[nl] + 1
        start = [0] * nl
        end = [0] * nl
        trans = [0] * nl
        for l in range(nl - 1):
            if dhf[l] < dhf[l + 1]:
                trans[l] = 1
                end[l] = iface[l + 1]
                start[l + 1] = iface[l + 1] + dhf[l + 1]
            elif dhf[l] > dhf[l + 1]:
                trans[l] = -1
                end[l] = iface[l + 1] - dhf[l]
                start[l + 1] = iface[l + 1]
            else:
                trans[l] = 0
                end[l] = iface[l + 1] - dhf[l]
                start[l + 1] = iface[l + 1]
        trans[nl - 1] = 0
        end[nl - 1] = iface[nl]
        vnx, vny, vnz = [], [], []
        for l in range(nl):
            ny = (end[l] - start[l]) // dhf[l] + 1
            nx = NXmax // dhf[l]
            nz = NZmax // dhf[l]
            if dhf[l] > 1:
                nx += 1
                nz += 1
            vnx.append(nx); vny.append(ny); vnz.append(nz)
        self.NX, self.NY, self.NZ, self.DH = NX, NY, NZ, DH
        self.nl, self.dhf, self.iface, self.start, self.end, self.trans = nl, dhf, iface, start, end, trans
        self.vnx, self.vny, self.vnz = vnx, vny, vnz
        self.npl = [vnx[l] * vny[l] * vnz[l] for l in range(nl)]
        self.offset = np.concatenate([[0], np.cumsum(self.npl)]).astype(np.int64)
        self.N = int(self.offset[-1])
        # getLayer / locatedOnInterface / getTransition / distToInterface depend on y only
        ys = range(NY)
        self.layer_y = np.array([self._get_layer(y) for y in ys], dtype=np.int64)
        self.on_iface_y = np.array([y in iface[:nl] for y in ys], dtype=bool)
        self.trans_y = np.array([self._get_transition(y) for y in ys], dtype=np.int64)
        self.dist_y = np.array([self._dist_to_interface(y) for y in ys], dtype=np.int64)
        # coordinates of every index (mapIndex2coordinate)
        X, Y, Z = [], [], []
        for l in range(nl):
            f = dhf[l]
            yy, zz, xx = np.meshgrid(np.arange(vny[l]), np.arange(vnz[l]), np.arange(vnx[l]), indexing="ij")
            X.append(xx.ravel() * f); Z.append(zz.ravel() * f); Y.append(yy.ravel() * f + start[l])
        self.x = np.concatenate(X).astype(np.int64)
        self.y = np.concatenate(Y).astype(np.int64)
        self.z = np.concatenate(Z).astype(np.int64)
        self.layer = self.layer_y[self.y]
        self.on_iface = self.on_iface_y[self.y]

    # Coordinates.cpp:381-397
    def _get_layer(self, y: int) -> int:
        layer = 0
        while layer < self.nl:
            if self.iface[layer] < y < self.iface[layer + 1]:
                break
            if y == self.iface[layer + 1]:
                if self.trans[layer] > 0:
                    layer += 1
                break
            layer += 1
        return layer

    def _get_transition(self, y: int) -> int:
        if y not in self.iface[:self.nl]:
            return 0
        t = 0
        for l in range(self.nl):
            if y == self.iface[l + 1]:
                t = self.trans[l]
        return t

    def _dist_to_interface(self, y: int) -> int:
        d = self.NY
        for i in self.iface[1:-1]:
            d = min(d, abs(y - i))
        return d

    def coordinate2index(self, X, Y, Z):
        """map3Dcoordinate2index (Coordinates.cpp:668-698), vectorised."""
        X = np.asarray(X, dtype=np.int64); Y = np.asarray(Y, dtype=np.int64); Z = np.asarray(Z, dtype=np.int64)
        X, Y, Z = np.broadcast_arrays(X, Y, Z)
        if (X < 0).any() or (X >= self.NX).any() or (Y < 0).any() or (Y >= self.NY).any() or (Z < 0).any() or (Z >= self.NZ).any():
            raise IndexError("Could not map from coordinate to index!")
        out = np.full(X.shape, -1, dtype=np.int64)
        done = np.zeros(X.shape, dtype=bool)
        for l in range(self.nl):
            m = (~done) & (Y >= self.start[l]) & (Y <= self.end[l])
            f = self.dhf[l]
            out[m] = (X[m] // f + (Z[m] // f) * self.vnx[l] + ((Y[m] - self.start[l]) // f) * self.vnx[l] * self.vnz[l]
                      + self.offset[l])
            done |= m
        if not done.all():
            raise IndexError("coordinate between the layers of the variable grid")
        return out

    def dh_of_layer(self, l: int, dtype) -> float:
        d = np.dtype(dtype).type
        return d(d(self.DH) * d(self.dhf[l]))


# --------------------------------------------------------------------------
# per-row stencils (positions along the axis, coefficient index, order)
# --------------------------------------------------------------------------
def _row_dxf(c: int, f: int, on_iface: bool, order: int, n: int, backward: bool, edge: bool = True):
    """Derivatives.cpp:149-184 (Dxf) and :726-761 (Dxb), for x or z. Returns
    [(position, order, j)] in push order. edge=False: taps outside the grid
    are dropped at full order (zero padding) instead of lowering the order."""
    out = []
    j = 0
    while j < order:
        if not edge:
            sh = (-(f // 3) if not backward else f // 3) if on_iface else 0
            P = c + sh + f * (j - order // 2 + (0 if backward else 1))
            if 0 <= P < n:
                out.append((P, order, j))
            j += 1
            continue
        sh = (-(f // 3) if not backward else f // 3) if on_iface else 0
        if not backward:
            P = c + sh + f * (j - order // 2 + 1)
            Pmin = c + sh + f * (-order // 2 + 1)
            Pmax = c + sh + f * (order // 2)
        else:
            P = c + sh + f * (j - order // 2)
            Pmin = c + sh + f * (-order // 2)
            Pmax = c + sh + f * (order // 2 - 1)
        if Pmin < 0:
            order += 2 * Pmin
            if backward and order == 0:
                order = 2
                c += 1
            j -= 1
        elif Pmax >= n:
            order -= 2 * (Pmax - n + 1)
            if not backward and order == 0:
                order = 2
                c -= 1
            j -= 1
        else:
            out.append((P, order, j))
        j += 1
    return out


def _row_dyf(g: VarGrid, y: int, orders, var_order: bool, fs: bool, edge: bool = True, var_grid: bool = True):
    """Derivatives.cpp:227-276 (Dyf) / :380-425 (DyfFreeSurface). Returns
    [(Y, order, j, image_j or -1)] and the DH layer."""
    layer = int(g.layer_y[y])
    order = orders[layer] if var_order else orders[0]
    dist = int(g.dist_y[y]) // g.dhf[layer]
    if var_grid and dist == 0:
        order = 2
    elif var_grid and order > dist * 2:
        order = dist * 2
    if g.on_iface_y[y] and g.trans_y[y] == -1:
        f = g.dhf[layer + 1]
        dl = layer + 1
    else:
        f = g.dhf[layer]
        dl = layer
    out = []
    if fs:
        for j in range(order):
            Y = y + f * (j - order // 2 + 1)
            img = -1
            if order >= 2 + (2 * y) // f + j:
                img = order - 2 - (2 * y) // f - j
            if 0 <= Y < g.NY:
                out.append((Y, order, j, img))
        return out, dl
    j = 0
    while j < order:
        Y = y + f * (j - order // 2 + 1)
        if not edge:
            if 0 <= Y < g.NY:
                out.append((Y, order, j, -1))
            j += 1
            continue
        Ymin = y + f * (-order // 2 + 1)
        Ymax = y + f * (order // 2)
        if Ymin < 0:
            order += 2 * Ymin
            j -= 1
        elif Ymax >= g.NY:
            order -= 2 * (Ymax - g.NY + 1)
            if order == 0:
                order = 2
                y -= 1
            j -= 1
        else:
            out.append((Y, order, j, -1))
        j += 1
    return out, dl


def _row_dyb(g: VarGrid, y: int, orders, var_order: bool, edge: bool = True, var_grid: bool = True):
    """Derivatives.cpp:790-840 (Dyb). Returns [(Y, order, j, DH layer)]."""
    layer = int(g.layer_y[y])
    f = g.dhf[layer]
    order = orders[layer] if var_order else orders[0]
    dist = int(g.dist_y[y]) // g.dhf[layer]
    if var_grid and dist == 0:
        order = 2
    elif var_grid and order > dist * 2:
        order = dist * 2
    out = []
    j = 0
    while j < order:
        Y = y + f * (j - order // 2)
        Ymin = y + f * (-order // 2)
        Ymax = y + f * (order // 2 - 1)
        # the interface tests see the current (possibly shifted) row
        on = bool(g.on_iface_y[y]) if 0 <= y < g.NY else False
        tr = int(g.trans_y[y]) if on else 0
        if on:
            if j == 0 and tr == 1:
                Y += g.dhf[layer - 1]
            if j == 1 and tr == -1:
                Y += g.dhf[layer + 1]
        if not edge:
            if 0 <= Y < g.NY:
                out.append((Y, order, j, int(g.layer_y[y])))
            j += 1
            continue
        if Ymin < 0:
            order += 2 * Ymin
            if order == 0:
                order = 2
                y += 1
            j -= 1
        elif Ymax >= g.NY:
            order -= 2 * (Ymax - g.NY + 1)
            j -= 1
        else:
            out.append((Y, order, j, int(g.layer_y[y])))
        j += 1
    return out


class Operators:
    """The acoustic operator set of one variable grid, DT folded in."""

    def __init__(self, g: VarGrid, orders, DT: float, free_surface: bool, dtype=np.float32, var_order: bool = True,
                 edge: bool = True, var_grid: bool = True):
        self.g, self.dtype, self.edge, self.var_grid = g, dtype, edge, var_grid
        d = np.dtype(dtype).type
        self.fdv = {k: np.array(v, dtype=dtype) for k, v in FD_VALUES.items()}
        self.DT = d(DT)
        is3d = g.NZ > 1
        self.Dxf = self._axis_op(orders, var_order, "x", backward=False)
        self.Dxb = self._axis_op(orders, var_order, "x", backward=True)
        self.Dyf = self._dy(orders, var_order, fs=bool(free_surface))
        self.Dyb = self._dyb(orders, var_order)
        if is3d:
            self.Dzf = self._axis_op(orders, var_order, "z", backward=False)
            self.Dzb = self._axis_op(orders, var_order, "z", backward=True)
        if var_grid:
            self.IFull = self._interp("full")
            self.IStagX = self._interp("x")
            if is3d:
                self.IStagZ = self._interp("z")
                self.IStagXZ = self._interp("xz")
        else:   # variable FD orders on a regular grid: no interpolation
            self.IFull = self.IStagX = self.IStagZ = self.IStagXZ = sp.identity(g.N, dtype=dtype, format="csr")

    def _val(self, order: int, j: int, dl: int, img: int = -1):
        """coefficient / DH (ValueType), then * DT (FDTD2D.cpp:212-215)."""
        d = np.dtype(self.dtype).type
        c = self.fdv[order][j]
        if img >= 0:
            c = d(c - self.fdv[order][img])
        v = d(c / self.g.dh_of_layer(dl, self.dtype))
        return d(v * self.DT)

    def _finish(self, rows, cols, vals):
        n = self.g.N
        rows = np.concatenate(rows) if rows else np.zeros(0, np.int64)
        cols = np.concatenate(cols) if cols else np.zeros(0, np.int64)
        vals = np.concatenate(vals).astype(self.dtype) if vals else np.zeros(0, self.dtype)
        return sp.csr_matrix((vals, (rows, cols)), shape=(n, n), dtype=self.dtype)

    def _axis_op(self, orders, var_order, axis, backward):
        g = self.g
        c_all = g.x if axis == "x" else g.z
        n = g.NX if axis == "x" else g.NZ
        keys = np.stack([c_all, g.layer, g.on_iface.astype(np.int64)], axis=1)
        uniq, inv = np.unique(keys, axis=0, return_inverse=True)
        inv = inv.ravel()
        order_rows = np.argsort(inv, kind="stable")
        bounds = np.searchsorted(inv[order_rows], np.arange(len(uniq) + 1))
        rows, cols, vals = [], [], []
        for k, (c, layer, on) in enumerate(uniq):
            r = order_rows[bounds[k]:bounds[k + 1]]
            f = g.dhf[layer]
            order = orders[layer] if var_order else orders[0]
            for P, o, j in _row_dxf(int(c), f, bool(on), order, n, backward, self.edge):
                if axis == "x":
                    col = g.coordinate2index(P, g.y[r], g.z[r])
                else:
                    col = g.coordinate2index(g.x[r], g.y[r], P)
                rows.append(r); cols.append(col)
                vals.append(np.full(len(r), self._val(o, j, int(layer)), dtype=self.dtype))
        return self._finish(rows, cols, vals)

    def _group_by_y(self):
        g = self.g
        order_rows = np.argsort(g.y, kind="stable")
        bounds = np.searchsorted(g.y[order_rows], np.arange(g.NY + 1))
        for y in range(g.NY):
            r = order_rows[bounds[y]:bounds[y + 1]]
            if len(r):
                yield y, r

    def _dy(self, orders, var_order, fs):
        g = self.g
        rows, cols, vals = [], [], []
        for y, r in self._group_by_y():
            taps, dl = _row_dyf(g, y, orders, var_order, fs, self.edge, self.var_grid)
            for Y, o, j, img in taps:
                rows.append(r); cols.append(g.coordinate2index(g.x[r], Y, g.z[r]))
                vals.append(np.full(len(r), self._val(o, j, dl, img), dtype=self.dtype))
        return self._finish(rows, cols, vals)

    def _dyb(self, orders, var_order):
        g = self.g
        rows, cols, vals = [], [], []
        for y, r in self._group_by_y():
            for Y, o, j, dl in _row_dyb(g, y, orders, var_order, self.edge, self.var_grid):
                rows.append(r); cols.append(g.coordinate2index(g.x[r], Y, g.z[r]))
                vals.append(np.full(len(r), self._val(o, j, dl), dtype=self.dtype))
        return self._finish(rows, cols, vals)

    def _interp(self, kind):
        """Derivatives.cpp:1252-1335 / 1356-1440 / 1462-1546 / 1568-1661
        (full, staggered x, staggered z, staggered xz): identity off the
        interfaces, bilinear from the coarse-aligned points on them."""
        g = self.g
        d = np.dtype(self.dtype).type
        rows, cols, vals = [], [], []
        off = np.nonzero(~g.on_iface)[0]
        rows.append(off); cols.append(off); vals.append(np.ones(len(off), dtype=self.dtype))
        on = np.nonzero(g.on_iface)[0]
        x, y, z = g.x[on], g.y[on], g.z[on]
        dhf = np.array(g.dhf, dtype=np.int64)
        layer = g.layer[on]
        f = dhf[layer]
        tr = g.trans_y[y]
        ff = f.copy()
        ff[tr == 1] = dhf[layer[tr == 1] - 1]
        ff[tr == -1] = dhf[np.minimum(layer[tr == -1] + 1, g.nl - 1)]
        den = (d(1) / (f * f).astype(self.dtype)).astype(self.dtype)
        cm = lambda a, b: np.fmod(a, b)          # C remainder (sign of the dividend)
        T = np.ones(len(on), dtype=bool)
        if kind == "full":
            mx, mz = cm(x, f), cm(z, f)
            pts = [(T, x - mx, z - mz, (f - mx) * (f - mz)),
                   (x + 2 * ff < g.NX, x + f - mx, z - mz, mx * (f - mz)),
                   (z + 2 * ff < g.NZ, x - mx, z + f - mz, (f - mx) * mz),
                   ((x + 2 * ff < g.NX) & (z + 2 * ff < g.NZ), x + f - mx, z + f - mz, mx * mz)]
        elif kind == "x":
            mx, mz = cm(x - f // 2, f), cm(z, f)
            pts = [(x >= mx, x - mx, z - mz, (f - mx) * (f - mz)),
                   (x + ff < g.NX, x + f - mx, z - mz, mx * (f - mz)),
                   ((x >= mx) & (z + 2 * ff < g.NZ), x - mx, z + f - mz, (f - mx) * mz),
                   ((x + ff < g.NX) & (z + 2 * ff < g.NZ), x + f - mx, z + f - mz, mx * mz)]
        elif kind == "z":
            mx, mz = cm(x, f), cm(z - f // 2, f)
            pts = [(z >= mz, x - mx, z - mz, (f - mx) * (f - mz)),
                   (x + 2 * ff < g.NX, x + f - mx, z - mz, mx * (f - mz)),
                   ((x >= mx) & (z + ff < g.NZ), x - mx, z + f - mz, (f - mx) * mz),
                   ((x + 2 * ff < g.NX) & (z + ff < g.NZ), x + f - mx, z + f - mz, mx * mz)]
        else:
            mx, mz = cm(x - f // 2, f), cm(z - f // 2, f)
            pts = [((x >= mx) & (z >= mz), x - mx, z - mz, (f - mx) * (f - mz)),
                   (x + ff < g.NX, x + f - mx, z - mz, mx * (f - mz)),
                   ((x >= mx) & (z + ff < g.NZ), x - mx, z + f - mz, (f - mx) * mz),
                   ((x + ff < g.NX) & (z + ff < g.NZ), x + f - mx, z + f - mz, mx * mz)]
        for ok, X, Z, w in pts:
            rows.append(on[ok]); cols.append(g.coordinate2index(X[ok], y[ok], Z[ok]))
            vals.append((w[ok].astype(self.dtype) * den[ok]).astype(self.dtype))
        return self._finish(rows, cols, vals)


# --------------------------------------------------------------------------
# model averages and CPML coefficients
# --------------------------------------------------------------------------
def density_partners(g: VarGrid):
    """The averaging partner of every point per axis (x, y[, z]) of
    calcAverageMatrixX/Y/Z (Modelparameter.cpp:336-446): (ok, col) with ok
    false where the point is averaged with itself alone."""
    out = []
    axes = ["x", "y"] + (["z"] if g.NZ > 1 else [])
    f_row = np.array(g.dhf, dtype=np.int64)[g.layer]
    for ax in axes:
        if ax == "x":
            X = g.x + f_row
            ok = X < g.NX
            col = np.where(ok, 0, 0)
            col[ok] = g.coordinate2index(X[ok], g.y[ok], g.z[ok])
        elif ax == "z":
            Z = g.z + f_row
            ok = Z < g.NZ
            col = np.zeros(g.N, np.int64)
            col[ok] = g.coordinate2index(g.x[ok], g.y[ok], Z[ok])
        else:
            step = f_row.copy()
            t0 = g.on_iface & (g.trans_y[g.y] == 0)
            nxt = np.minimum(g.layer + 1, g.nl - 1)
            step[t0] = np.array(g.dhf, dtype=np.int64)[nxt[t0]]
            Y = g.y + step
            ok = Y < g.NY
            col = np.zeros(g.N, np.int64)
            col[ok] = g.coordinate2index(g.x[ok], Y[ok], g.z[ok])
        out.append((ok, col))
    return out


def inverse_density_averages(g: VarGrid, rho: np.ndarray, dtype=np.float32):
    """calcAverageMatrixX/Y/Z (Modelparameter.cpp:336-446) applied to rho,
    then 1/avg with invalid -> 0 (calcInverseAveragedParameter :633-640)."""
    d = np.dtype(dtype).type
    rho = rho.astype(dtype)
    half = d(0.5)
    out = []
    for ok, col in density_partners(g):
        avg = np.where(ok, (half * rho + half * rho[col]).astype(dtype), rho).astype(dtype)
        with np.errstate(divide="ignore", invalid="ignore"):
            inv = (d(1) / avg).astype(dtype)
        inv[~np.isfinite(inv)] = 0
        out.append(inv)
    return out


def cpml_profile(width: int, npower: float, fc: float, vmax: float, DT: float, DH: float, shift: bool, dtype):
    """CPML::calcCoeffCPML (CPML.cpp:38-64) in the value type."""
    d = np.dtype(dtype).type
    a = np.zeros(width, dtype=dtype)
    b = np.zeros(width, dtype=dtype)
    sh = d(0.5) if shift else d(0)
    f64 = np.float64
    # the C++ expressions promote to double wherever a double literal enters
    alpha_max = d(2.0 * math.pi * (f64(d(fc)) / 2.0))
    num = d(d(-(d(npower) + d(1))) * d(vmax))
    num = d(num * d(np.log(d(0.0008))))
    d0 = d(f64(num) / (2.0 * width * f64(d(DH))))
    for i in range(width):
        pn = d(d(d(width - i) - sh) / d(width))
        dd = d(d0 * d(np.power(pn, d(npower))))
        ap = d(f64(alpha_max) * (1.0 - f64(pn)))
        b[i] = d(np.exp(d(d(-(d(dd + ap))) * d(DT))))
        a[i] = d(f64(dd) * (f64(b[i]) - 1.0) / f64(d(dd + ap))) if abs(dd) > 1.0e-6 else d(0)
    return a, b


def cpml_coefficients(g: VarGrid, BW: int, npower: float, fc: float, vmax: float, DT: float,
                      free_surface: bool, dtype=np.float32):
    """Per-point CPML coefficient vectors (CPML2DAcoustic.cpp:140-205 and the
    3-D counterpart), zero outside the absorbing frame. Returns
    {axis: (a_full, b_full, a_half, b_half)}."""
    prof = []
    for l in range(g.nl):
        w = int(math.ceil(np.float32(BW) / g.dhf[l]))
        dh = g.dh_of_layer(l, dtype)
        prof.append((w,) + cpml_profile(w, npower, fc, vmax, DT, dh, False, dtype)
                    + cpml_profile(w, npower, fc, vmax, DT, dh, True, dtype))
    out = {}
    axes = ["x", "y"] + (["z"] if g.NZ > 1 else [])
    f_row = np.array(g.dhf, dtype=np.int64)[g.layer]
    for ax in axes:
        c = {"x": g.x, "y": g.y, "z": g.z}[ax]
        n = {"x": g.NX, "y": g.NY, "z": g.NZ}[ax]
        gd = np.minimum(c, n - 1 - c)
        dist = gd // f_row
        coord = c // f_row
        af, bf, ah, bh = (np.zeros(g.N, dtype=dtype) for _ in range(4))
        for l in range(g.nl):
            w, a, b, a2, b2 = prof[l]
            m = (g.layer == l) & (dist < w)
            lo = m & (coord < w)
            hi = m & ~(coord < w)
            if ax == "y" and free_surface:
                lo = lo & False
            dl = dist[lo]
            af[lo], bf[lo], ah[lo], bh[lo] = a[dl], b[dl], a2[dl], b2[dl]
            dh_ = dist[hi]
            af[hi], bf[hi], ah[hi], bh[hi] = a2[dh_], b2[dh_], a[dh_], b[dh_]
        out[ax] = (af, bf, ah, bh)
    return out


# --------------------------------------------------------------------------
# ABS on the variable grid
# --------------------------------------------------------------------------
def abs_damping(g: VarGrid, BW: int, damping_coeff: float, free_surface: bool, dtype=np.float32):
    """ABS2D::init / ABS3D::init (ABS2D.cpp:110-180, ABS3D.cpp:154-220) per
    point of the grid at its fine-grid coordinates (Coordinates::edgeDistance,
    Coordinates.cpp:734-760): coeff[j] = exp(-a^2 (w - j)^2),
    a = sqrt(-ln(1 - DampingCoeff/100) / w^2), at the smallest edge distance
    below w (with a free surface the top rows take the x (and z) distance
    only); 1 elsewhere."""
    d = np.dtype(dtype).type
    w = int(BW)
    amp = d(1) - d(damping_coeff) / d(100)
    a = np.sqrt(d(-np.log(amp)) / d(w * w)).astype(dtype)
    j = np.arange(w)
    coeff = np.exp(-(a * a * ((w - j) * (w - j)).astype(dtype)).astype(dtype)).astype(dtype)
    dx = np.minimum(g.x, g.NX - 1 - g.x)
    dy = np.minimum(g.y, g.NY - 1 - g.y)
    dz = np.minimum(g.z, g.NZ - 1 - g.z)
    is3d = g.NZ > 1
    m = np.minimum(dx, dy)
    if is3d:
        m = np.minimum(m, dz)
    out = np.ones(g.N, dtype=dtype)
    if not free_surface:
        sel = m < w
        out[sel] = coeff[m[sel]]
        return out
    top = g.y < w
    xz = np.where(dx < dz, dx, dz) if is3d else dx
    sel_top = top & ((dx < w) | (dz < w)) if is3d else top & (dx < w)
    out[sel_top] = coeff[xz[sel_top]]
    sel = ~top & (m < w)
    out[sel] = coeff[m[sel]]
    return out


# --------------------------------------------------------------------------
# the acoustic time loop
# --------------------------------------------------------------------------
class AcousticVarGrid:
    """FD2Dacoustic / FD3Dacoustic::run on a variable grid, CPML, ABS
    (`damping`: abs_damping's per-point factors) or no damping boundary,
    mirror free surface (FreeSurface=1) or none."""

    def __init__(self, g: VarGrid, orders, DT: float, rho, vp, free_surface: int, cpml: dict | None,
                 src_idx, src_type, signals, rec_idx, rec_type, dtype=np.float32, var_order: bool = True,
                 edge: bool = True, var_grid: bool = True, damping=None):
        self.g, self.dtype = g, dtype
        self.damping = None if damping is None else np.asarray(damping, dtype=dtype)
        d = np.dtype(dtype).type
        self.op = Operators(g, orders, DT, free_surface == 1, dtype, var_order, edge, var_grid)
        self.is3d = g.NZ > 1
        rho = np.asarray(rho, dtype=dtype); vp = np.asarray(vp, dtype=dtype)
        self.M = (rho * vp * vp).astype(dtype)
        inv = inverse_density_averages(g, rho, dtype)
        self.irx, self.iry = inv[0], inv[1]
        self.irz = inv[2] if self.is3d else None
        self.cpml = cpml
        self.fs = free_surface == 1
        self.surface = (g.y != 0).astype(dtype)
        n = g.N
        z = lambda: np.zeros(n, dtype=dtype)
        self.p, self.vx, self.vy = z(), z(), z()
        self.vz = z() if self.is3d else None
        self.psi = {k: z() for k in ("p_x", "p_y", "p_z", "vxx", "vyy", "vzz")}
        self.src_idx = np.asarray(src_idx, np.int64); self.src_type = np.asarray(src_type)
        self.signals = np.asarray(signals, dtype=dtype)
        self.rec_idx = np.asarray(rec_idx, np.int64); self.rec_type = np.asarray(rec_type)
        self.d = d

    def _cpml(self, upd, key, ax, half):
        if self.cpml is None:
            return upd
        af, bf, ah, bh = self.cpml[ax]
        a, b = (ah, bh) if half else (af, bf)
        ps = (self.psi[key] * b).astype(self.dtype)
        ps = (ps + a * upd).astype(self.dtype)
        self.psi[key] = ps
        return (upd + ps).astype(self.dtype)

    def step(self, t: int):
        op, dt = self.op, self.dtype
        upd = self._cpml(op.Dxf @ self.p, "p_x", "x", True)
        self.vx = (self.vx + (upd * self.irx).astype(dt)).astype(dt)
        self.vx = op.IStagX @ self.vx
        upd = self._cpml(op.Dyf @ self.p, "p_y", "y", True)
        self.vy = (self.vy + (upd * self.iry).astype(dt)).astype(dt)
        self.vy = op.IFull @ self.vy
        if self.is3d:
            upd = self._cpml(op.Dzf @ self.p, "p_z", "z", True)
            self.vz = (self.vz + (upd * self.irz).astype(dt)).astype(dt)
            self.vz = op.IStagZ @ self.vz
        upd = self._cpml(op.Dxb @ self.vx, "vxx", "x", False)
        u2 = self._cpml(op.Dyb @ self.vy, "vyy", "y", False)
        upd = (upd + u2).astype(dt)
        if self.is3d:
            u2 = self._cpml(op.Dzb @ self.vz, "vzz", "z", False)
            upd = (upd + u2).astype(dt)
        upd = (upd * self.M).astype(dt)
        self.p = (self.p + upd).astype(dt)
        if self.damping is not None:
            # DampingBoundary.apply(p, vX, vY[, vZ]) before the interpolation
            self.p = (self.p * self.damping).astype(dt)
            self.vx = (self.vx * self.damping).astype(dt)
            self.vy = (self.vy * self.damping).astype(dt)
            if self.is3d:
                self.vz = (self.vz * self.damping).astype(dt)
        self.p = op.IFull @ self.p
        if self.fs:
            self.p = (self.p * self.surface).astype(dt)
        for s in range(len(self.src_idx)):
            if self.src_type[s] == 1:
                self.p[self.src_idx[s]] += self.signals[s, t]
            elif self.src_type[s] == 2:
                self.vx[self.src_idx[s]] += self.signals[s, t]
            elif self.src_type[s] == 3:
                self.vy[self.src_idx[s]] += self.signals[s, t]
            elif self.src_type[s] == 4 and self.is3d:
                self.vz[self.src_idx[s]] += self.signals[s, t]
        fields = {1: self.p, 2: self.vx, 3: self.vy, 4: self.vz}
        return np.array([fields[int(k)][i] for i, k in zip(self.rec_idx, self.rec_type)], dtype=dt)

    def run(self, nt: int) -> np.ndarray:
        out = np.zeros((len(self.rec_idx), nt), dtype=self.dtype)
        for t in range(nt):
            out[:, t] = self.step(t)
        return out
