"""Discrete adjoints of the acoustic and elastic variable-grid steps
(oracle, test infrastructure only: used by tests/ as the checker, never by
the library).

The forward step is AcousticVarGrid.step (oracle/vargrid.py), the
restatement of FD2Dacoustic / FD3Dacoustic::run on a variable grid
(ForwardSolver2Dacoustic.cpp:91-194, ForwardSolver3Dacoustic.cpp:91-233) with
the interface interpolations of Derivatives.cpp:1177-1546, the CPML of
CPML.cpp:84-95, the ABS taper of ABS2D.cpp:14-50 / ABS3D.cpp:15-100 and the
free-surface zero of FreeSurface.cpp:14-19. Every operator of that step is a
scipy sparse matrix or a per-point factor, so the adjoint step applies the
transposes in reverse order. The misfit is J = 1/2 sum (d - d_obs)^2 over
receivers and steps; the gradient runs through M = rho vp^2
(ModelparameterSeismic.cpp:131-136) and the inverse density averages of
Modelparameter.cpp:336-446, 633-640 (averaging partners per axis)."""
import numpy as np

from oracle.vargrid import AcousticVarGrid, VarGrid, density_partners

_PSI = ("p_x", "p_y", "p_z", "vxx", "vyy", "vzz")


def _state(f: AcousticVarGrid):
    s = dict(p=f.p.copy(), vx=f.vx.copy(), vy=f.vy.copy(), vz=None if f.vz is None else f.vz.copy())
    s.update({k: v.copy() for k, v in f.psi.items()})
    return s


def adjoint_gradient(g: VarGrid, orders, DT, rho, vp, free_surface, cpml, src_idx, src_type, signals, rec_idx, rec_type,
                     dobs, damping=None, var_order=True, edge=True, var_grid=True):
    """Returns (J, dJ/dvp, dJ/drho) of the acoustic variable-grid run in FP64."""
    rho = np.asarray(rho, np.float64)
    vp = np.asarray(vp, np.float64)
    f = AcousticVarGrid(g, orders, DT, rho, vp, free_surface, cpml, src_idx, src_type, np.asarray(signals, np.float64),
                        rec_idx, rec_type, dtype=np.float64, var_order=var_order, edge=edge, var_grid=var_grid,
                        damping=damping)
    nt = np.asarray(signals).shape[1]
    states, seis = [], np.zeros((len(rec_idx), nt))
    for t in range(nt):
        states.append(_state(f))
        seis[:, t] = f.step(t)
    res = seis - np.asarray(dobs, np.float64)
    J = 0.5 * float(np.sum(res * res))

    op, is3d = f.op, f.is3d
    axes = ("x", "y", "z") if is3d else ("x", "y")
    D = {"x": (op.Dxf, op.Dxb, op.IStagX, f.irx, "vx", "p_x", "vxx"),
         "y": (op.Dyf, op.Dyb, op.IFull, f.iry, "vy", "p_y", "vyy")}
    if is3d:
        D["z"] = (op.Dzf, op.Dzb, op.IStagZ, f.irz, "vz", "p_z", "vzz")
    n = g.N
    lam = {k: np.zeros(n) for k in ("p", "vx", "vy") + (("vz",) if is3d else ()) + _PSI}
    gM = np.zeros(n)
    gir = {a: np.zeros(n) for a in axes}
    dmp = None if damping is None else np.asarray(damping, np.float64)
    surface = (g.y != 0).astype(np.float64)
    fields = {1: "p", 2: "vx", 3: "vy", 4: "vz"}
    for t in range(nt - 1, -1, -1):
        S = states[t]
        # the receivers read the state after step t
        for r, (i, k) in enumerate(zip(rec_idx, rec_type)):
            lam[fields[int(k)]][i] += res[r, t]
        # re-formed forward intermediates of step t
        gx, v2, h = {}, {}, {}
        for a in axes:
            Df, Db, I, ir, vk, pk, qk = D[a]
            u = Df @ S["p"]
            if cpml is not None:
                af, bf, ah, bh = cpml[a]
                u = u + (S[pk] * bh + ah * u)
            gx[a] = u
            v2[a] = I @ (S[vk] + u * ir)
        d = np.zeros(n)
        for a in axes:
            Df, Db, I, ir, vk, pk, qk = D[a]
            u = Db @ v2[a]
            if cpml is not None:
                af, bf, ah, bh = cpml[a]
                u = u + (S[qk] * bf + af * u)
            d += u
        # adjoint of the step, last operation first
        lp = lam["p"] * surface if f.fs else lam["p"]
        lp = op.IFull.T @ lp
        lv2 = {}
        for a in axes:
            lv2[a] = lam[D[a][4]].copy()
        if dmp is not None:
            lp = dmp * lp
            for a in axes:
                lv2[a] = dmp * lv2[a]
        gM += lp * d
        ld = f.M.astype(np.float64) * lp
        new = {"p": lp.copy()}
        for a in axes:
            Df, Db, I, ir, vk, pk, qk = D[a]
            ldx = ld
            if cpml is not None:
                af, bf, ah, bh = cpml[a]
                tot = lam[qk] + ld
                ldx = ld + af * tot
                new[qk] = bf * tot
            lv2[a] = lv2[a] + Db.T @ ldx
        for a in axes:
            Df, Db, I, ir, vk, pk, qk = D[a]
            lv1 = I.T @ lv2[a]
            new[vk] = lv1
            lg = ir * lv1
            gir[a] += lv1 * gx[a]
            lu = lg
            if cpml is not None:
                af, bf, ah, bh = cpml[a]
                tot = lam[pk] + lg
                lu = lg + ah * tot
                new[pk] = bh * tot
            new["p"] = new["p"] + Df.T @ lu
        for k in lam:
            lam[k] = new.get(k, np.zeros(n))

    M = rho * vp * vp
    gvp = gM * 2.0 * rho * vp
    grho = gM * vp * vp
    for a, (ok, col) in zip(axes, density_partners(g)):
        avg = np.where(ok, 0.5 * rho + 0.5 * rho[col], rho)
        ir = 1.0 / avg
        w = -gir[a] * ir * ir
        grho += np.where(ok, 0.5 * w, w)
        np.add.at(grho, col[ok], 0.5 * w[ok])
    del M
    return J, gvp, grho


def _shear_xy_terms(g: VarGrid):
    """The points and weights of every point's XY 4-point average
    (shear_average_xy in oracle/vargrid_elastic.py, Modelparameter.cpp:
    449-533): a list of (rows, partner columns, weight)."""
    f = np.array(g.dhf, dtype=np.int64)[g.layer]
    x2, y2 = g.x + f, g.y + f
    okx, oky = x2 < g.NX, y2 < g.NY
    out = []
    i = np.nonzero(okx & oky)[0]
    for c in (i, g.coordinate2index(x2[i], g.y[i], g.z[i]), g.coordinate2index(g.x[i], y2[i], g.z[i]),
              g.coordinate2index(x2[i], y2[i], g.z[i])):
        out.append((i, np.asarray(c, np.int64), 0.25))
    b = np.nonzero(okx & ~oky)[0]
    out += [(b, b, 0.5), (b, np.asarray(g.coordinate2index(x2[b], g.y[b], g.z[b]), np.int64), 0.5)]
    r = np.nonzero(~okx & oky)[0]
    out += [(r, r, 0.5), (r, np.asarray(g.coordinate2index(g.x[r], y2[r], g.z[r]), np.int64), 0.5)]
    c = np.nonzero(~okx & ~oky)[0]
    out.append((c, c, 1.0))
    return out


def elastic_adjoint_gradient_2d(g: VarGrid, orders, DT, rho, vp, vs, cpml, src_idx, src_type, signals, rec_idx, rec_type,
                                dobs, damping=None, free_surface=False, var_order=True, edge=True, var_grid=True):
    """(J, dJ/dvp, dJ/dvs, dJ/drho) of the 2-D elastic variable-grid run
    (ElasticVarGrid2D, FD2Delastic::run ForwardSolver2Delastic.cpp:117-297)
    in FP64: the transposes of its sparse step in reverse order; the chain
    rule through M = rho vp^2, mu = rho vs^2, the inverse density averages,
    the XY shear average of 1/max(mu, 1) and the free-surface scales
    scaleV = M - 2 mu, scaleH = -(M - 2 mu)^2 / M (FreeSurfaceElastic.cpp:11-47)."""
    from oracle.vargrid_elastic import ElasticVarGrid2D
    rho = np.asarray(rho, np.float64)
    vp = np.asarray(vp, np.float64)
    vs = np.asarray(vs, np.float64)
    f = ElasticVarGrid2D(g, orders, DT, rho, vp, vs, cpml, src_idx, src_type, np.asarray(signals, np.float64), rec_idx,
                         rec_type, dtype=np.float64, var_order=var_order, edge=edge, var_grid=var_grid,
                         free_surface=free_surface, damping=damping)
    nt = np.asarray(signals).shape[1]
    names = ("vx", "vy", "sxx", "syy", "sxy")
    states, seis = [], np.zeros((len(rec_idx), nt))
    for t in range(nt):
        st = {k: getattr(f, k).copy() for k in names}
        st.update({"psi_" + k: v.copy() for k, v in f.psi.items()})
        states.append(st)
        seis[:, t] = f.step(t)
    res = seis - np.asarray(dobs, np.float64)
    J = 0.5 * float(np.sum(res * res))

    op, n = f.op, g.N
    cp = cpml

    def term(D, u, psi, ax, half):
        d = D @ u
        if cp is not None:
            af, bf, ah, bh = cp[ax]
            a, b = (ah, bh) if half else (af, bf)
            d = d + (psi * b + a * d)
        return d

    def term_t(ld, lpsi, ax, half):
        if cp is None:
            return ld, np.zeros(n)
        af, bf, ah, bh = cp[ax]
        a, b = (ah, bh) if half else (af, bf)
        tot = lpsi + ld
        return ld + a * tot, b * tot

    lam = {k: np.zeros(n) for k in names}
    lpsi = {k: np.zeros(n) for k in f.psi}
    gM, gmu, gmuXY, girx, giry, gsH, gsV = (np.zeros(n) for _ in range(7))
    dmp = np.ones(n) if damping is None else np.asarray(damping, np.float64)
    M, mu, muXY = f.M, f.mu, f.muXY
    for t in range(nt - 1, -1, -1):
        S = states[t]
        for r, (i, k) in enumerate(zip(rec_idx, rec_type)):
            if k == 1:
                lam["sxx"][i] += 0.5 * res[r, t]
                lam["syy"][i] += 0.5 * res[r, t]
            else:
                lam["vx" if k == 2 else "vy"][i] += res[r, t]
        # forward intermediates of step t
        gvx = term(op.Dxf, S["sxx"], S["psi_sxx_x"], "x", True) + term(f.DybSX, S["sxy"], S["psi_sxy_y"], "y", False)
        vx2 = op.IStagX @ (S["vx"] + gvx * f.irx)
        gvy = term(op.Dxb, S["sxy"], S["psi_sxy_x"], "x", False) + term(op.Dyf, S["syy"], S["psi_syy_y"], "y", True)
        vy2 = op.IFull @ (S["vy"] + gvy * f.iry)
        vxx = term(op.Dxb, vx2, S["psi_vxx"], "x", False)
        vyy = term(op.Dyb, vy2, S["psi_vyy"], "y", False)
        ush = term(f.DyfSX, vx2, S["psi_vxy"], "y", True) + term(op.Dxf, vy2, S["psi_vyx"], "x", True)
        # the step's adjoint, last operation first: ABS taper, free surface
        l = {k: dmp * lam[k] for k in names}
        lvxx, lvyy = np.zeros(n), np.zeros(n)
        if free_surface:
            gsH += l["sxx"] * vxx
            gsV -= l["sxx"] * vyy
            lvxx += f.scaleH * l["sxx"]
            lvyy -= f.scaleV * l["sxx"]
            l["syy"] = l["syy"] * f.fsZero
        new = {}
        newpsi = {}
        # shear stress
        ls1 = op.IStagX.T @ l["sxy"]
        new["sxy"] = ls1.copy()
        gmuXY += ls1 * ush
        lu = muXY * ls1
        ld, newpsi["vxy"] = term_t(lu, lpsi["vxy"], "y", True)
        lvx2 = l["vx"] + f.DyfSX.T @ ld
        ld, newpsi["vyx"] = term_t(lu, lpsi["vyx"], "x", True)
        lvy2 = l["vy"] + op.Dxf.T @ ld
        # normal stresses
        lx1 = op.IFull.T @ l["sxx"]
        ly1 = op.IFull.T @ l["syy"]
        new["sxx"], new["syy"] = lx1.copy(), ly1.copy()
        lu = lx1 + ly1
        gM += lu * (vxx + vyy)
        gmu -= 2.0 * (vyy * lx1 + vxx * ly1)
        lvxx += M * lu - 2.0 * mu * ly1
        lvyy += M * lu - 2.0 * mu * lx1
        ld, newpsi["vxx"] = term_t(lvxx, lpsi["vxx"], "x", False)
        lvx2 = lvx2 + op.Dxb.T @ ld
        ld, newpsi["vyy"] = term_t(lvyy, lpsi["vyy"], "y", False)
        lvy2 = lvy2 + op.Dyb.T @ ld
        # vy
        lv1 = op.IFull.T @ lvy2
        new["vy"] = lv1
        lg = f.iry * lv1
        giry += lv1 * gvy
        ld, newpsi["sxy_x"] = term_t(lg, lpsi["sxy_x"], "x", False)
        new["sxy"] += op.Dxb.T @ ld
        ld, newpsi["syy_y"] = term_t(lg, lpsi["syy_y"], "y", True)
        new["syy"] += op.Dyf.T @ ld
        # vx
        lv1 = op.IStagX.T @ lvx2
        new["vx"] = lv1
        lg = f.irx * lv1
        girx += lv1 * gvx
        ld, newpsi["sxx_x"] = term_t(lg, lpsi["sxx_x"], "x", True)
        new["sxx"] += op.Dxf.T @ ld
        ld, newpsi["sxy_y"] = term_t(lg, lpsi["sxy_y"], "y", False)
        new["sxy"] += f.DybSX.T @ ld
        lam, lpsi = new, newpsi

    # chain rule: free-surface scales (surface points only), shear average
    if free_surface:
        sel = (g.y == 0).astype(np.float64)
        tt = M - 2.0 * mu
        gM += sel * (gsV + gsH * (-2.0 * tt / M + tt * tt / (M * M)))
        gmu += sel * (-2.0 * gsV + gsH * 4.0 * tt / M)
    ok = muXY >= 4
    for rows, cols, w in _shear_xy_terms(g):
        m = mu[cols]
        dd = np.where(ok[rows] & (m > 1), gmuXY[rows] * muXY[rows] ** 2 * w / (m * m), 0.0)
        np.add.at(gmu, cols, dd)
    gvp = gM * 2.0 * rho * vp
    gvs = gmu * 2.0 * rho * vs
    grho = gM * vp * vp + gmu * vs * vs
    for gir, (okp, col) in zip((girx, giry), density_partners(g)):
        avg = np.where(okp, 0.5 * rho + 0.5 * rho[col], rho)
        ir = 1.0 / avg
        w = -gir * ir * ir
        grho += np.where(okp, 0.5 * w, w)
        np.add.at(grho, col[okp], 0.5 * w[okp])
    return J, gvp, gvs, grho


def _shear_terms(g: VarGrid, pair: str):
    """The points and weights of every point's 4-point average of the axis
    pair (shear_average in oracle/vargrid_elastic.py, Modelparameter.cpp:
    449-624): a list of (rows, partner columns, weight)."""
    f = np.array(g.dhf, dtype=np.int64)[g.layer]
    c = {"x": g.x, "y": g.y, "z": g.z}
    n = {"x": g.NX, "y": g.NY, "z": g.NZ}
    a, b = pair[0], pair[1]

    def idx(sel, da, db):
        p = {k: c[k][sel].copy() for k in "xyz"}
        p[a] = p[a] + da * f[sel]
        p[b] = p[b] + db * f[sel]
        return np.asarray(g.coordinate2index(p["x"], p["y"], p["z"]), np.int64)

    oka, okb = c[a] + f < n[a], c[b] + f < n[b]
    out = []
    i = np.nonzero(oka & okb)[0]
    out += [(i, i, 0.25), (i, idx(i, 1, 0), 0.25), (i, idx(i, 0, 1), 0.25), (i, idx(i, 1, 1), 0.25)]
    i = np.nonzero(oka & ~okb)[0]
    out += [(i, i, 0.5), (i, idx(i, 1, 0), 0.5)]
    i = np.nonzero(~oka & okb)[0]
    out += [(i, i, 0.5), (i, idx(i, 0, 1), 0.5)]
    i = np.nonzero(~oka & ~okb)[0]
    out.append((i, i, 1.0))
    return out


def elastic_adjoint_gradient_3d(g: VarGrid, orders, DT, rho, vp, vs, cpml, src_idx, src_type, signals, rec_idx, rec_type,
                                dobs, damping=None, free_surface=False, var_order=True, edge=True, var_grid=True):
    """(J, dJ/dvp, dJ/dvs, dJ/drho) of the 3-D elastic variable-grid run
    (ElasticVarGrid3D, FD3Delastic::run ForwardSolver3Delastic.cpp:120-414)
    in FP64, as elastic_adjoint_gradient_2d with the z terms, the XZ and YZ
    shear averages, the twice-applied StaggeredZ interpolation of syz and the
    surface exchange of sxx and szz with vxx + vzz (FreeSurface3Delastic.cpp:
    15-47)."""
    from oracle.vargrid_elastic import ElasticVarGrid3D
    rho = np.asarray(rho, np.float64)
    vp = np.asarray(vp, np.float64)
    vs = np.asarray(vs, np.float64)
    f = ElasticVarGrid3D(g, orders, DT, rho, vp, vs, cpml, src_idx, src_type, np.asarray(signals, np.float64), rec_idx,
                         rec_type, dtype=np.float64, var_order=var_order, edge=edge, var_grid=var_grid,
                         free_surface=free_surface, damping=damping)
    nt = np.asarray(signals).shape[1]
    states, seis = [], np.zeros((len(rec_idx), nt))
    for t in range(nt):
        st = {k: v.copy() for k, v in f.f.items()}
        st.update({"psi_" + k: v.copy() for k, v in f.psi.items()})
        states.append(st)
        seis[:, t] = f.step(t)
    res = seis - np.asarray(dobs, np.float64)
    J = 0.5 * float(np.sum(res * res))

    op, n, cp = f.op, g.N, cpml
    IStagZ2 = op.IStagZ @ op.IStagZ
    vel = {"vx": ([(op.Dxf, "sxx", "sxx_x", "x", True), (f.DybSX, "sxy", "sxy_y", "y", False),
                   (op.Dzb, "sxz", "sxz_z", "z", False)], f.irx, op.IStagX),
           "vy": ([(op.Dxb, "sxy", "sxy_x", "x", False), (op.Dyf, "syy", "syy_y", "y", True),
                   (op.Dzb, "syz", "syz_z", "z", False)], f.iry, op.IFull),
           "vz": ([(op.Dxb, "sxz", "sxz_x", "x", False), (f.DybSZ, "syz", "syz_y", "y", False),
                   (op.Dzf, "szz", "szz_z", "z", True)], f.irz, op.IStagZ)}
    shear = {"sxy": ([(f.DyfSX, "vx", "vxy", "y", True), (op.Dxf, "vy", "vyx", "x", True)], f.muXY, op.IStagX),
             "sxz": ([(op.Dzf, "vx", "vxz", "z", True), (op.Dxf, "vz", "vzx", "x", True)], f.muXZ, op.IStagXZ),
             "syz": ([(op.Dzf, "vy", "vyz", "z", True), (f.DyfSZ, "vz", "vzy", "y", True)], f.muYZ, IStagZ2)}
    normal = {"vx": (op.Dxb, "vxx", "x"), "vy": (op.Dyb, "vyy", "y"), "vz": (op.Dzb, "vzz", "z")}

    def term(D, u, psi, ax, half):
        d = D @ u
        if cp is not None:
            af, bf, ah, bh = cp[ax]
            a, b = (ah, bh) if half else (af, bf)
            d = d + (psi * b + a * d)
        return d

    def term_t(ld, lpsi, ax, half):
        if cp is None:
            return ld, np.zeros(n)
        af, bf, ah, bh = cp[ax]
        a, b = (ah, bh) if half else (af, bf)
        tot = lpsi + ld
        return ld + a * tot, b * tot

    names = list(f.f)
    lam = {k: np.zeros(n) for k in names}
    lpsi = {k: np.zeros(n) for k in f.psi}
    gM, gmu, girx, giry, girz, gsH, gsV = (np.zeros(n) for _ in range(7))
    gmuS = {k: np.zeros(n) for k in shear}
    gir = {"vx": girx, "vy": giry, "vz": girz}
    dmp = np.ones(n) if damping is None else np.asarray(damping, np.float64)
    M, mu = f.M, f.mu
    for t in range(nt - 1, -1, -1):
        S = states[t]
        for r, (i, k) in enumerate(zip(rec_idx, rec_type)):
            if k == 1:
                for c in ("sxx", "syy", "szz"):
                    lam[c][i] += res[r, t] / 3.0
            else:
                lam[("vx", "vy", "vz")[k - 2]][i] += res[r, t]
        gv, v2 = {}, {}
        for k, (terms, ir, I) in vel.items():
            gv[k] = sum(term(D, S[fld], S["psi_" + q], ax, half) for D, fld, q, ax, half in terms)
            v2[k] = I @ (S[k] + gv[k] * ir)
        e = {k: term(D, v2[k], S["psi_" + q], ax, False) for k, (D, q, ax) in normal.items()}
        ush = {k: sum(term(D, v2[fld], S["psi_" + q], ax, half) for D, fld, q, ax, half in terms)
               for k, (terms, m, I) in shear.items()}
        l = {k: dmp * lam[k] for k in names}
        lnorm = {k: np.zeros(n) for k in normal}
        if free_surface:
            ls = l["sxx"] + l["szz"]
            gsH += ls * (e["vx"] + e["vz"])
            gsV -= ls * e["vy"]
            lnorm["vx"] += f.scaleH * ls
            lnorm["vz"] += f.scaleH * ls
            lnorm["vy"] -= f.scaleV * ls
            l["syy"] = l["syy"] * f.fsZero
        new, newpsi = {}, {}
        lv2 = {k: l[k].copy() for k in ("vx", "vy", "vz")}
        for k, (terms, m, I) in shear.items():
            l1 = I.T @ l[k]
            new[k] = l1.copy()
            gmuS[k] += l1 * ush[k]
            lu = m * l1
            for D, fld, q, ax, half in terms:
                ld, newpsi[q] = term_t(lu, lpsi[q], ax, half)
                lv2[fld] = lv2[fld] + D.T @ ld
        l1 = {c: op.IFull.T @ l[c] for c in ("sxx", "syy", "szz")}
        for c in l1:
            new[c] = l1[c].copy()
        lsum = l1["sxx"] + l1["syy"] + l1["szz"]
        ex, ey, ez = e["vx"], e["vy"], e["vz"]
        gM += lsum * (ex + ey + ez)
        gmu -= 2.0 * ((ey + ez) * l1["sxx"] + (ex + ez) * l1["syy"] + (ex + ey) * l1["szz"])
        lnorm["vx"] += M * lsum - 2.0 * mu * (l1["syy"] + l1["szz"])
        lnorm["vy"] += M * lsum - 2.0 * mu * (l1["sxx"] + l1["szz"])
        lnorm["vz"] += M * lsum - 2.0 * mu * (l1["sxx"] + l1["syy"])
        for k, (D, q, ax) in normal.items():
            ld, newpsi[q] = term_t(lnorm[k], lpsi[q], ax, False)
            lv2[k] = lv2[k] + D.T @ ld
        for k, (terms, ir, I) in vel.items():
            lv1 = I.T @ lv2[k]
            new[k] = lv1
            lg = ir * lv1
            gir[k] += lv1 * gv[k]
            for D, fld, q, ax, half in terms:
                ld, newpsi[q] = term_t(lg, lpsi[q], ax, half)
                new[fld] = new[fld] + D.T @ ld
        lam, lpsi = new, newpsi

    if free_surface:
        sel = (g.y == 0).astype(np.float64)
        tt = M - 2.0 * mu
        gM += sel * (gsV + gsH * (-2.0 * tt / M + tt * tt / (M * M)))
        gmu += sel * (-2.0 * gsV + gsH * 4.0 * tt / M)
    for k, pair in (("sxy", "xy"), ("sxz", "xz"), ("syz", "yz")):
        m = shear[k][1]
        ok = m >= 4
        for rows, cols, w in _shear_terms(g, pair):
            mm = mu[cols]
            dd = np.where(ok[rows] & (mm > 1), gmuS[k][rows] * m[rows] ** 2 * w / (mm * mm), 0.0)
            np.add.at(gmu, cols, dd)
    gvp = gM * 2.0 * rho * vp
    gvs = gmu * 2.0 * rho * vs
    grho = gM * vp * vp + gmu * vs * vs
    for gr, (okp, col) in zip((girx, giry, girz), density_partners(g)):
        avg = np.where(okp, 0.5 * rho + 0.5 * rho[col], rho)
        ir = 1.0 / avg
        w = -gr * ir * ir
        grho += np.where(okp, 0.5 * w, w)
        np.add.at(grho, col[okp], 0.5 * w[okp])
    return J, gvp, gvs, grho
