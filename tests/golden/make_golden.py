"""Generate the golden fixtures under tests/golden/ (committed).

The reference (Julia + ParallelStencil) cannot run in this container, so the
fixtures come from a second, independent restatement of the reference kernels
written here in numpy's array-slice form -- the closest Python analogue of the
reference's own `@all/@inn/@d_xi/@av_*` expressions.  The C++ oracle is
checked against these fixtures; the two restatements share no code.

Run:  python tests/golden/make_golden.py   (writes tests/golden/*.npz)
Sources restated (all paths relative to the reference repository):
  Dimensionless/kernels_HT3D.jl:73-154, Dimensionless/HydroThermal3D_Alban_v6.jl:84-159,
  tools/Weno5_Routines.jl:5-276, tools/Weno5_Routines_v2.jl:1-347,
  Dimensional/kernels_HT3D_dimensional.jl:40-363, Dimensional/HydroThermal3D_v18.jl:29-39,432-477.
"""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def F(a):
    return np.asfortranarray(a)


# ----------------------------------------------------------------- macros
def d_xi(A): return A[1:, 1:-1, 1:-1] - A[:-1, 1:-1, 1:-1]
def d_yi(A): return A[1:-1, 1:, 1:-1] - A[1:-1, :-1, 1:-1]
def d_zi(A): return A[1:-1, 1:-1, 1:] - A[1:-1, 1:-1, :-1]
def d_xa(A): return A[1:] - A[:-1]
def d_ya(A): return A[:, 1:] - A[:, :-1]
def d_za(A): return A[:, :, 1:] - A[:, :, :-1]
def inn(A): return A[1:-1, 1:-1, 1:-1]
def av_yza(A): return (A[:, :-1, :-1] + A[:, 1:, :-1] + A[:, :-1, 1:] + A[:, 1:, 1:]) * 0.25
def av_xza(A): return (A[:-1, :, :-1] + A[1:, :, :-1] + A[:-1, :, 1:] + A[1:, :, 1:]) * 0.25
def av_xya(A): return (A[:-1, :-1, :] + A[1:, :-1, :] + A[:-1, 1:, :] + A[1:, 1:, :]) * 0.25
def av_yi(A): return (A[1:-1, :-1, 1:-1] + A[1:-1, 1:, 1:-1]) * 0.5


def av(A):
    return (A[:-1, :-1, :-1] + A[1:, :-1, :-1] + A[:-1, 1:, :-1] + A[1:, 1:, :-1] +
            A[:-1, :-1, 1:] + A[1:, :-1, 1:] + A[:-1, 1:, 1:] + A[1:, 1:, 1:]) * 0.125


# ------------------------------------------------------- dimensionless kernels
def compute_flux(kx, ky, kz, A, _dx, _dy, _dz):
    return F(-kx * (_dx * d_xi(A))), F(-ky * (_dy * d_yi(A))), F(-kz * (_dz * d_zi(A)))


def residual_transient(T, R, qx, qy, qz, _dt, _dx, _dy, _dz):
    return F(R + _dt * inn(T) + _dx * d_xa(qx) + _dy * d_ya(qy) + _dz * d_za(qz))


def residual_diffusion(R, qx, qy, qz, _dx, _dy, _dz):
    return F(R + _dx * d_xa(qx) + _dy * d_ya(qy) + _dz * d_za(qz))


def face_bcs(X, types, vals):
    """Six-face ghost rules with pre-launch snapshot reads (see oracle header)."""
    S = X.copy()
    X = X.copy(order="F")
    n1, n2, n3 = X.shape

    def r(f, inner):
        return inner if types[f] == 0 else 2.0 * vals[f] - inner
    # evaluate rule by rule in the reference order; later rules overwrite
    X[0, :, :] = r(0, S[1, :, :])
    X[-1, :, :] = r(1, S[-2, :, :])
    X[:, 0, :] = r(2, S[:, 1, :])
    X[:, -1, :] = r(3, S[:, -2, :])
    X[:, :, 0] = r(4, S[:, :, 1])
    X[:, :, -1] = r(5, S[:, :, -2])
    return X


def gershgorin(rhoC, kx, ky, kz, transient, dt, dx, dy, dz):
    kW, kE, kS, kN, kB, kF = kx[:-1], kx[1:], ky[:, :-1], ky[:, 1:], kz[:, :, :-1], kz[:, :, 1:]
    diag = ((kB / dz + kF / dz) / dz + (kN / dy + kS / dy) / dy + (kE / dx + kW / dx) / dx + rhoC * transient / dt)
    G = (np.abs(kE / dx ** 2) + np.abs(kW / dx ** 2) + np.abs(kN / dy ** 2) + np.abs(kS / dy ** 2) +
         np.abs(kB / dz ** 2) + np.abs(kF / dz ** 2) + np.abs(diag))
    return F(G / diag), F(diag)


def dyrel_dimless(X, R, kx, ky, kz, cX, dx, dy, dz, types, vals, niter, cfl=0.99, cfact=0.5, ratio=500.0, nitout=1000):
    """n fixed DYREL iterations (Dimensional/HydroThermal3D_v18.jl:432-477 with the
    dimensionless residual).  Returns X, F, F0, (lmin, h1, h2)."""
    X = X.copy(order="F")
    _dx, _dy, _dz = 1 / dx, 1 / dy, 1 / dz
    G, PC = gershgorin(np.ones_like(R), kx, ky, kz, 1.0 if cX else 0.0, 1 / cX if cX else 1.0, dx, dy, dz)
    lmax = G.max()
    lmin = lmax / ratio
    dtau = 2.0 / np.sqrt(lmax) * cfl
    c = 2.0 * np.sqrt(lmin) * cfact
    h1, h2 = (2 - c * dtau) / (2 + c * dtau), 2 * dtau / (2 + c * dtau)
    Fc = np.zeros_like(R)
    F0 = np.zeros_like(R)
    for it in range(1, niter + 1):
        check = it % nitout == 0 or it <= 2
        Fit = Fc.copy()
        X = face_bcs(X, types, vals)
        qx, qy, qz = compute_flux(kx, ky, kz, X, _dx, _dy, _dz)
        if cX:
            Fc = residual_transient(X, R, qx, qy, qz, cX, _dx, _dy, _dz)
        else:
            Fc = residual_diffusion(R, qx, qy, qz, _dx, _dy, _dz)
        Fc = F(Fc / PC)
        F0 = F(h1 * F0 + h2 * Fc)
        X[1:-1, 1:-1, 1:-1] = inn(X) - dtau * F0
        if check and it > 1:
            d = dtau * F0
            lmin = abs(np.sum(-d * (Fc - Fit))) / abs(np.sum(d * d))
            c = 2.0 * np.sqrt(lmin) * cfact
            h1, h2 = (2 - c * dtau) / (2 + c * dtau), 2 * dtau / (2 + c * dtau)
    return X, Fc, F0, np.array([lmin, h1, h2, lmax, dtau])


# ------------------------------------------------------------------ WENO5
def weno_flux(v1, v2, v3, v4, v5):
    p1 = v1 / 3.0 - 7.0 / 6.0 * v2 + 11.0 / 6.0 * v3
    p2 = -v2 / 6.0 + 5.0 / 6.0 * v3 + v4 / 3.0
    p3 = v3 / 3.0 + 5.0 / 6.0 * v4 - v5 / 6.0
    maxV = np.maximum(np.maximum(np.maximum(np.maximum(v1 ** 2, v2 ** 2), v3 ** 2), v4 ** 2), v5 ** 2)
    e = 1e-99 + 1e-6 * maxV
    w1 = 13.0 / 12.0 * (v1 - 2.0 * v2 + v3) ** 2 + 1.0 / 4.0 * (v1 - 4.0 * v2 + 3.0 * v3) ** 2
    w2 = 13.0 / 12.0 * (v2 - 2.0 * v3 + v4) ** 2 + 1.0 / 4.0 * (v2 - v4) ** 2
    w3 = 13.0 / 12.0 * (v3 - 2.0 * v4 + v5) ** 2 + 1.0 / 4.0 * (3.0 * v3 - 4.0 * v4 + v5) ** 2
    w1 = 0.1 / (w1 + e) ** 2
    w2 = 0.6 / (w2 + e) ** 2
    w3 = 0.3 / (w3 + e) ** 2
    w = w1 + w2 + w3
    return (w1 / w) * p1 + (w2 / w) * p2 + (w3 / w) * p3


def exxx_fill(Fc, axis, tL, vL, tR, vR):
    """Boundaries_*_Weno5! on an inner (n^3) field -> the parts of exxx the sweep reads."""
    n = Fc.shape
    X = np.zeros(tuple(s + 6 for s in n), order="F")
    X[3:-3, 3:-3, 3:-3] = Fc
    A = np.moveaxis(Fc, axis, 0)
    Xa = np.moveaxis(X, axis, 0)
    m = A.shape[0]
    lat = (slice(3, -3), slice(3, -3))
    for side, t, v in ((0, tL, vL), (1, tR, vR)):
        if side == 0:
            src = A[m - 3:m] if t == 2 else A[2::-1]
            dst = Xa[0:3]
        else:
            src = A[0:3] if t == 2 else A[m - 1:m - 4:-1] if m >= 4 else A[::-1][:3]
            dst = Xa[m + 3:m + 6]
        val = 2 * v - src if t == 1 else src
        dst[(slice(None),) + lat] = val
    return X


def weno_L(X, axis, h, V, quirk):
    """-(Vp dF- + Vm dF+) pieces of Advect! on an exxx array: returns (Vp*dFm + Vm*dFp)."""
    Xa = np.moveaxis(X, axis, 0)[:, 3:-3, 3:-3]
    m = Xa.shape[0] - 6

    def x(o):
        return Xa[3 + o:3 + o + m]
    m5 = h * (x(2) - x(-1)) if quirk else h * (x(2) - x(1))
    dFm = weno_flux(h * (x(-2) - x(-3)), h * (x(-1) - x(-2)), h * (x(0) - x(-1)), h * (x(1) - x(0)), m5)
    dFp = weno_flux(h * (x(3) - x(2)), h * (x(2) - x(1)), h * (x(1) - x(0)), h * (x(0) - x(-1)), h * (x(-1) - x(-2)))
    Va = np.moveaxis(V, axis, 0)
    Vm = np.where(Va[:-1] < 0, Va[:-1], 0.0)
    Vp = np.where(Va[1:] > 0, Va[1:], 0.0)
    return np.moveaxis(Vp * dFm + Vm * dFp, 0, axis)


def advect_weno5(T_ex, V, dt, h, types, vals, quirk):
    """AdvectWithWeno5 (v1, quirk=False) / AdvectWithWeno5_v2 (quirk=True)."""
    T = T_ex.copy(order="F")
    Tc = inn(T).copy(order="F")
    for a in range(3):
        Told = Tc.copy()
        for _ in range(2):
            X = exxx_fill(Tc, a, types[2 * a], vals[2 * a], types[2 * a + 1], vals[2 * a + 1])
            Tc = F(Tc - dt * weno_L(X, a, h[a], V[a], quirk))
        Tc = F((1.0 / 2.0) * Tc + (1.0 - 1.0 / 2.0) * Told)
    T[1:-1, 1:-1, 1:-1] = Tc
    return T


# ---------------------------------------------------------------- material laws
def rhof_C(T_C, p):
    return (1006 + (7.424e-7 * p) + (-0.3922 * T_C) + (-4.441e-15 * p ** 2) + (4.547e-9 * p * T_C) +
            (-0.003774 * T_C ** 2) + (1.451e-23 * p ** 3) + (-1.793e-17 * p ** 2 * T_C) + (7.485e-12 * p * T_C ** 2) +
            (2.955e-6 * T_C ** 3) + (-1.463e-32 * p ** 4) + (1.361e-26 * p ** 3 * T_C) +
            (4.018e-21 * (p ** 2) * (T_C ** 2)) + (-7.372e-15 * p * T_C ** 3) + (5.698e-11 * T_C ** 4))


def drhodP_C(T_C, p):
    return (-7.372e-15 * T_C ** 3 + 8.036e-21 * T_C ** 2 * p + 7.485e-12 * T_C ** 2 + 4.083e-26 * T_C * p ** 2 -
            3.586e-17 * T_C * p + 4.547e-9 * T_C - 5.852e-32 * p ** 3 + 4.353e-23 * p ** 2 - 8.882e-15 * p + 7.424e-7)


def main():
    rng = np.random.default_rng(20240607)
    nx, ny, nz = 7, 6, 5
    ex = (nx + 2, ny + 2, nz + 2)
    fx, fy, fz, v = (nx + 1, ny, nz), (nx, ny + 1, nz), (nx, ny, nz + 1), (nx + 1, ny + 1, nz + 1)
    U = lambda s, lo=0.5, hi=1.5: F(rng.uniform(lo, hi, size=s))
    d = {}
    d["dims"] = np.array([nx, ny, nz])
    d["dx"], d["dy"], d["dz"] = np.array(1 / nx), np.array(0.8 / ny), np.array(1.2 / nz)
    dx, dy, dz = float(d["dx"]), float(d["dy"]), float(d["dz"])
    _dx, _dy, _dz = 1 / dx, 1 / dy, 1 / dz
    T, P = U(ex), U(ex, -1, 1)
    kx, ky, kz, kv = U(fx), U(fy), U(fz), U(v)
    R = U((nx, ny, nz), -1, 1)
    d.update(T=T, P=P, kx=kx, ky=ky, kz=kz, kv=kv, R=R)
    qx, qy, qz = compute_flux(kx, ky, kz, T, _dx, _dy, _dz)
    d.update(qx=qx, qy=qy, qz=qz)
    _dt = 3.7
    d["_dt"] = np.array(_dt)
    d["F_transient"] = residual_transient(T, R, qx, qy, qz, _dt, _dx, _dy, _dz)
    d["F_diffusion"] = residual_diffusion(R, qx, qy, qz, _dx, _dy, _dz)
    d["Ty"] = F(av_yi(T))
    d["kx_v"], d["ky_v"], d["kz_v"] = F(av_yza(kv)), F(av_xza(kv)), F(av_xya(kv))
    Ra = 123.0
    d["Ra"] = np.array(Ra)
    d["Rp"] = F(Ra * _dy * (ky[:, 1:] * d["Ty"][:, 1:] - ky[:, :-1] * d["Ty"][:, :-1]))
    d["Vx"] = F(-kx * _dx * d_xi(P))
    d["Vy"] = F(-ky * (_dy * d_yi(P) - Ra * d["Ty"]))
    d["Vz"] = F(-kz * _dz * d_zi(P))
    types, vals = [0, 0, 1, 1, 0, 1], [0.0, 0.0, 1.0, -0.5, 0.0, 2.0]
    d["bc_types"], d["bc_vals"] = np.array(types), np.array(vals)
    d["T_bc"] = face_bcs(T, types, vals)
    d["ktc_v2c"] = F(av(kv))
    G, D = gershgorin(U((nx, ny, nz)), kx, ky, kz, 1.0, 0.3, dx, dy, dz)
    d["rhoC"] = U((nx, ny, nz))
    d["G"], d["D"] = gershgorin(d["rhoC"], kx, ky, kz, 1.0, 0.3, dx, dy, dz)
    # DYREL iterations (thermal with cX = _dt, Darcy with cX = 0)
    X, Fc, F0, sc = dyrel_dimless(T, R, kx, ky, kz, _dt, dx, dy, dz, types, vals, 7, nitout=3)
    d.update(dyrel_T_X=X, dyrel_T_F=Fc, dyrel_T_F0=F0, dyrel_T_sc=sc)
    X, Fc, F0, sc = dyrel_dimless(P, R, kx, ky, kz, 0.0, dx, dy, dz, [0] * 6, [0.0] * 6, 7, nitout=3)
    d.update(dyrel_P_X=X, dyrel_P_F=Fc, dyrel_P_F0=F0, dyrel_P_sc=sc)
    # WENO5 (v1 textbook stencil, v2 quirk); need n >= 3 per axis
    Vx, Vy, Vz = U(fx, -1, 1), U(fy, -1, 1), U(fz, -1, 1)
    d.update(wVx=Vx, wVy=Vy, wVz=Vz)
    wt, wv = [0, 0, 1, 1, 2, 2], [0.0, 0.0, 1.0, 0.0, 0.0, 0.0]
    d["weno_types"], d["weno_vals"] = np.array(wt), np.array(wv)
    d["weno_dt"] = np.array(0.01)
    d["weno_v1"] = advect_weno5(T, (Vx, Vy, Vz), 0.01, (_dx, _dy, _dz), wt, wv, False)
    d["weno_v2"] = advect_weno5(T, (Vx, Vy, Vz), 0.01, (_dx, _dy, _dz), wt, wv, True)
    # material laws on a grid of (T_C, p)
    Tg, pg = np.meshgrid(np.linspace(10, 700, 7), np.linspace(1e5, 3e8, 5), indexing="ij")
    d["law_T"], d["law_p"] = F(Tg), F(pg)
    d["rhof"], d["drhodp"] = F(rhof_C(Tg, pg)), F(drhodP_C(Tg, pg))
    np.savez_compressed(os.path.join(HERE, "dimless_small.npz"), **d)
    print("wrote", os.path.join(HERE, "dimless_small.npz"))


if __name__ == "__main__":
    main()
