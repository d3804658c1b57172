"""Discrete adjoint of the acoustic variable-grid step (oracle, test
infrastructure only: used by tests/ as the checker, never by the library).

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
