"""Host-side mirror of the reference's ParallelStencil kernel interface.

Every function here has the name of the reference kernel it replaces (without
the trailing ``!``; ``ρ``/``ϕ`` spelled ``Rho``/``Phi``), takes the same
arguments in the same order, mutates its output arrays in place and returns
``None`` -- so a driver line ``@parallel ComputeFlux!(qx, qy, qz, kx, ky, kz,
A, _dx, _dy, _dz)`` becomes ``ComputeFlux(ctx, qx, qy, qz, kx, ky, kz, A, _dx,
_dy, _dz)``.  Arrays are CUDA float64 torch tensors in the reference's
column-major layout (see :func:`zeros`); grid sizes are inferred from the
array shapes exactly like ParallelStencil infers its launch range.

Errors: a bad shape/dtype raises ``ValueError`` before anything is launched; a
non-zero status from libht3d raises :class:`Ht3dError`.
"""
import ctypes

import torch

from . import _lib
from . import abi


class Ht3dError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"libht3d status {status} ({msg})")
        self.status = status


class Context:
    """Owns one ht3d_ctx (one CUDA stream; scratch memory).

    stream: the cudaStream_t (int handle, e.g. torch.cuda.Stream().cuda_stream)
    the library launches on; None gives the context a private non-blocking
    stream.  Issue the torch work that produces a call's inputs on the same
    stream (``with torch.cuda.stream(s)``), or synchronize it first: a private
    stream is not ordered after torch's.  Calls are synchronous by default."""

    def __init__(self, device=0, stream=None, sync=True):
        self.lib = _lib.load()
        self.ptr = ctypes.c_void_p()
        s = 0 if stream is None else int(stream)
        st = self.lib.ht3d_ctx_create(ctypes.byref(self.ptr), int(device), s)
        if st != abi.OK:
            raise Ht3dError(st, self.lib.ht3d_status_string(st).decode())
        self.device = device
        self.stream = s  # the stream handle the context was created on (0: a private stream)
        if not sync:
            self.lib.ht3d_ctx_set_sync(self.ptr, 0)

    def check(self, st):
        if st != abi.OK:
            msg = self.lib.ht3d_status_string(st).decode()
            detail = self.lib.ht3d_ctx_last_error(self.ptr).decode()
            raise Ht3dError(st, f"{msg}: {detail}" if detail else msg)

    def call(self, name, *args):
        self.check(getattr(self.lib, name)(self.ptr, *args))

    def synchronize(self):
        self.check(self.lib.ht3d_ctx_synchronize(self.ptr))

    @property
    def launches(self):
        return int(self.lib.ht3d_ctx_launch_count(self.ptr))

    def set_tuning(self, key, value):
        self.check(self.lib.ht3d_ctx_set_tuning(self.ptr, int(key), int(value)))

    def inner_timing(self, reset=False):
        """(ms, launches) of the mixed solver's event-timed inner-iteration runs."""
        ms, nl = ctypes.c_double(), ctypes.c_ulonglong()
        self.check(self.lib.ht3d_ctx_inner_timing(self.ptr, ctypes.byref(ms), ctypes.byref(nl), int(bool(reset))))
        return ms.value, nl.value

    def close(self):
        if self.ptr:
            self.lib.ht3d_ctx_destroy(self.ptr)
            self.ptr = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# --------------------------------------------------------------- arrays
def zeros(n1, n2, n3=1, dtype=torch.float64, device="cuda"):
    """@zeros(n1,n2,n3): column-major (x fastest) tensor of shape (n1,n2,n3)."""
    return torch.zeros((n3, n2, n1), dtype=dtype, device=device).permute(2, 1, 0)


def ones(n1, n2, n3=1, dtype=torch.float64, device="cuda"):
    return torch.ones((n3, n2, n1), dtype=dtype, device=device).permute(2, 1, 0)


def from_numpy(a, device="cuda"):
    """Copy a numpy array (any order) into a column-major device tensor."""
    import numpy as np
    a = np.asarray(a, dtype=np.float64)
    if a.ndim == 2:  # column-major 2-D (e.g. the immersed-surface weights wN)
        t = torch.zeros((a.shape[1], a.shape[0]), dtype=torch.float64, device=device).t()
        t.copy_(torch.from_numpy(np.ascontiguousarray(a.T)).t())
        return t
    t = zeros(*a.shape, device=device)
    t.copy_(torch.from_numpy(np.ascontiguousarray(a.transpose(2, 1, 0))).permute(2, 1, 0))
    return t


def to_numpy(t):
    """Device tensor (3-D, or 2-D like wN) -> Fortran-ordered numpy array of the same shape."""
    import numpy as np
    if t.dim() == 2:
        return np.asfortranarray(t.detach().t().contiguous().cpu().numpy().T)
    return np.asfortranarray(t.detach().permute(2, 1, 0).contiguous().cpu().numpy().transpose(2, 1, 0))


def _ptr(t, shape=None, name="array", dtype=torch.float64):
    if not isinstance(t, torch.Tensor):
        raise ValueError(f"{name}: expected a torch tensor")
    if t.dtype != dtype or not t.is_cuda:
        raise ValueError(f"{name}: expected a CUDA {dtype} tensor, got {t.dtype} on {t.device}")
    if t.dim() == 2:
        n1, n2 = t.shape
        ok = t.stride() == (1, n1)
        s = (n1, n2)
    else:
        n1, n2, n3 = t.shape
        ok = t.stride() == (1, n1, n1 * n2)
        s = (n1, n2, n3)
    if not ok:
        raise ValueError(f"{name}: expected a column-major (x fastest) contiguous tensor (use hydrothermal3d_gb300.zeros)")
    if shape is not None and tuple(shape) != s:
        raise ValueError(f"{name}: shape {s} does not match the staggering {tuple(shape)}")
    return t.data_ptr()


def _cells_ex(A, name="A"):
    if A.dim() != 3:
        raise ValueError(f"{name}: expected a 3-D ghosted array")
    nx, ny, nz = (int(s) - 2 for s in A.shape)
    return nx, ny, nz


def _cells(A):
    return tuple(int(s) for s in A.shape)


def _shapes(nx, ny, nz):
    return dict(c=(nx, ny, nz), ex=(nx + 2, ny + 2, nz + 2), fx=(nx + 1, ny, nz), fy=(nx, ny + 1, nz),
                fz=(nx, ny, nz + 1), v=(nx + 1, ny + 1, nz + 1), xxx=(nx + 6, ny + 6, nz + 6))


def _numel(t):
    return int(t.numel())


# ------------------------------------------------- dimensionless kernels
def Init_vel(ctx, Vx, Vy, Vz, kx, ky, kz, Pc_ex, Ty, Ra, _dx, _dy, _dz):
    nx, ny, nz = _cells_ex(Pc_ex, "Pc_ex"); S = _shapes(nx, ny, nz)
    ctx.call("ht3d_Init_vel", _ptr(Vx, S["fx"], "Vx"), _ptr(Vy, S["fy"], "Vy"), _ptr(Vz, S["fz"], "Vz"),
             _ptr(kx, S["fx"], "kx"), _ptr(ky, S["fy"], "ky"), _ptr(kz, S["fz"], "kz"), _ptr(Pc_ex, S["ex"]),
             _ptr(Ty, S["fy"], "Ty"), Ra, _dx, _dy, _dz, nx, ny, nz)


def InitDarcy(ctx, Ty, kx, ky, kz, Tc_ex, kfv, _dt):
    nx, ny, nz = _cells_ex(Tc_ex, "Tc_ex"); S = _shapes(nx, ny, nz)
    ctx.call("ht3d_InitDarcy", _ptr(Ty, S["fy"], "Ty"), _ptr(kx, S["fx"], "kx"), _ptr(ky, S["fy"], "ky"),
             _ptr(kz, S["fz"], "kz"), _ptr(Tc_ex, S["ex"]), _ptr(kfv, S["v"], "kfv"), _dt, nx, ny, nz)


def Compute_Rp(ctx, Rp, ky, Ty, Ra, _dy):
    nx, ny, nz = _cells(Rp); S = _shapes(nx, ny, nz)
    ctx.call("ht3d_Compute_Rp", _ptr(Rp, S["c"], "Rp"), _ptr(ky, S["fy"], "ky"), _ptr(Ty, S["fy"], "Ty"), Ra, _dy,
             nx, ny, nz)


def InitThermal(ctx, Rt, kx, ky, kz, Tc_ex, ktv, _dt):
    nx, ny, nz = _cells_ex(Tc_ex, "Tc_ex"); S = _shapes(nx, ny, nz)
    ctx.call("ht3d_InitThermal", _ptr(Rt, S["c"], "Rt"), _ptr(kx, S["fx"], "kx"), _ptr(ky, S["fy"], "ky"),
             _ptr(kz, S["fz"], "kz"), _ptr(Tc_ex, S["ex"]), _ptr(ktv, S["v"], "ktv"), _dt, nx, ny, nz)


def ComputeFlux(ctx, qx, qy, qz, kx, ky, kz, A, _dx, _dy, _dz):
    nx, ny, nz = _cells_ex(A); S = _shapes(nx, ny, nz)
    ctx.call("ht3d_ComputeFlux", _ptr(qx, S["fx"], "qx"), _ptr(qy, S["fy"], "qy"), _ptr(qz, S["fz"], "qz"),
             _ptr(kx, S["fx"], "kx"), _ptr(ky, S["fy"], "ky"), _ptr(kz, S["fz"], "kz"), _ptr(A, S["ex"]), _dx, _dy,
             _dz, nx, ny, nz)


def UpdateT(ctx, F, T, R, qx, qy, qz, _dt, dtau, _dx, _dy, _dz):
    nx, ny, nz = _cells(F); S = _shapes(nx, ny, nz)
    ctx.call("ht3d_UpdateT", _ptr(F, S["c"], "F"), _ptr(T, S["ex"], "T"), _ptr(R, S["c"], "R"),
             _ptr(qx, S["fx"], "qx"), _ptr(qy, S["fy"], "qy"), _ptr(qz, S["fz"], "qz"), _dt, dtau, _dx, _dy, _dz,
             nx, ny, nz)


def ResidualDiffusion(ctx, F, R, qx, qy, qz, _dx, _dy, _dz):
    nx, ny, nz = _cells(F); S = _shapes(nx, ny, nz)
    ctx.call("ht3d_ResidualDiffusion", _ptr(F, S["c"], "F"), _ptr(R, S["c"], "R"), _ptr(qx, S["fx"], "qx"),
             _ptr(qy, S["fy"], "qy"), _ptr(qz, S["fz"], "qz"), _dx, _dy, _dz, nx, ny, nz)


def ResidualDiffusionTransient(ctx, F, T, R, qx, qy, qz, _dt, _dx, _dy, _dz):
    nx, ny, nz = _cells(F); S = _shapes(nx, ny, nz)
    ctx.call("ht3d_ResidualDiffusionTransient", _ptr(F, S["c"], "F"), _ptr(T, S["ex"], "T"), _ptr(R, S["c"], "R"),
             _ptr(qx, S["fx"], "qx"), _ptr(qy, S["fy"], "qy"), _ptr(qz, S["fz"], "qz"), _dt, _dx, _dy, _dz,
             nx, ny, nz)


def UpdateP(ctx, F0, P, F, dampx, dtau):
    nx, ny, nz = _cells(F); S = _shapes(nx, ny, nz)
    ctx.call("ht3d_UpdateP", _ptr(F0, S["c"], "F0"), _ptr(P, S["ex"], "P"), _ptr(F, S["c"], "F"), dampx, dtau,
             nx, ny, nz)


DampedUpdate = UpdateP


def DYRELUpdate(ctx, F0, X, F, h1, h2, dtau):
    nx, ny, nz = _cells(F); S = _shapes(nx, ny, nz)
    ctx.call("ht3d_DYRELUpdate", _ptr(F0, S["c"], "F0"), _ptr(X, S["ex"], "X"), _ptr(F, S["c"], "F"), h1, h2, dtau,
             nx, ny, nz)


def SetPressureBCs(ctx, Pc_ex, Pbot, Ptop):
    nx, ny, nz = _cells_ex(Pc_ex, "Pc_ex")
    ctx.call("ht3d_SetPressureBCs", _ptr(Pc_ex), Pbot, Ptop, nx, ny, nz)


def SetFaceBCs(ctx, X_ex, bc_type6, bc_val6):
    nx, ny, nz = _cells_ex(X_ex, "X_ex")
    ctx.call("ht3d_SetFaceBCs", _ptr(X_ex), abi.int6(*bc_type6), abi.dbl6(*bc_val6), nx, ny, nz)


def KillNorthSouthFluxes(ctx, Ty):
    nx, ny1, nz = _cells(Ty)
    ctx.call("ht3d_KillNorthSouthFluxes", _ptr(Ty), nx, ny1 - 1, nz)


def ResetA(ctx, A, B):
    if A.numel() != B.numel():
        raise ValueError("ResetA: arrays differ in size")
    ctx.call("ht3d_ResetA", _ptr(A, None, "A"), _ptr(B, None, "B"), _numel(A))


def Cpy_inn_to_all(ctx, A, B):
    nx, ny, nz = _cells(A); S = _shapes(nx, ny, nz)
    ctx.call("ht3d_Cpy_inn_to_all", _ptr(A, S["c"], "A"), _ptr(B, S["ex"], "B"), nx, ny, nz)


def Cpy_all_to_inn(ctx, A, B):
    nx, ny, nz = _cells(B); S = _shapes(nx, ny, nz)
    ctx.call("ht3d_Cpy_all_to_inn", _ptr(A, S["ex"], "A"), _ptr(B, S["c"], "B"), nx, ny, nz)


def ArrayEqualArray(ctx, A, B):
    if A.shape != B.shape:
        raise ValueError("ArrayEqualArray: shapes differ")
    ctx.call("ht3d_ArrayEqualArray", _ptr(A, None, "A"), _ptr(B, None, "B"), _numel(A))


def Multiply(ctx, a, b, c):
    if not (a.shape == b.shape == c.shape):
        raise ValueError("Multiply: shapes differ")
    ctx.call("ht3d_Multiply", _ptr(a), _ptr(b), _ptr(c), _numel(a))


# ------------------------------------------------------ DYREL support
def GershgorinPoisson(ctx, G, D, rhoC_eff, kx, ky, kz, transient, dt, dx, dy, dz):
    nx, ny, nz = _cells(G); S = _shapes(nx, ny, nz)
    ctx.call("ht3d_GershgorinPoisson", _ptr(G, S["c"], "G"), _ptr(D, S["c"], "D"), _ptr(rhoC_eff, S["c"], "rhoC"),
             _ptr(kx, S["fx"], "kx"), _ptr(ky, S["fy"], "ky"), _ptr(kz, S["fz"], "kz"), transient, dt, dx, dy, dz,
             nx, ny, nz)


def GershgorinHydro(ctx, G, phidrhodP, kx, ky, kz, transient, dt, dx, dy, dz):
    nx, ny, nz = _cells(G); S = _shapes(nx, ny, nz)
    ctx.call("ht3d_GershgorinHydro", _ptr(G, S["c"], "G"), _ptr(phidrhodP, S["c"]), _ptr(kx, S["fx"], "kx"),
             _ptr(ky, S["fy"], "ky"), _ptr(kz, S["fz"], "kz"), transient, dt, dx, dy, dz, nx, ny, nz)


def SwapDYREL(ctx, Xc, Yc, X0c_ex, Y0c):
    nx, ny, nz = _cells(Xc); S = _shapes(nx, ny, nz)
    ctx.call("ht3d_SwapDYREL", _ptr(Xc, S["c"]), _ptr(Yc, S["c"]), _ptr(X0c_ex, S["ex"]), _ptr(Y0c, S["c"]),
             nx, ny, nz)


def RayleighQuotientNumerator(ctx, G, Fc0, Fcit, Fc, dtau):
    ctx.call("ht3d_RayleighQuotientNumerator", _ptr(G), _ptr(Fc0), _ptr(Fcit), _ptr(Fc), dtau, _numel(G))


def RayleighQuotientDenominator(ctx, G, Fc0, dtau):
    ctx.call("ht3d_RayleighQuotientDenominator", _ptr(G), _ptr(Fc0), dtau, _numel(G))


# ------------------------------------------------------ reductions
def _reduce(ctx, a, op):
    out = ctypes.c_double()
    ctx.call("ht3d_reduce", _ptr(a), _numel(a), op, ctypes.byref(out))
    return out.value


def sum_g(ctx, a):
    return _reduce(ctx, a, abi.RED_SUM)


def maximum_g(ctx, a):
    return _reduce(ctx, a, abi.RED_MAX)


def minimum_g(ctx, a):
    return _reduce(ctx, a, abi.RED_MIN)


def mean_g(ctx, a):
    return _reduce(ctx, a, abi.RED_SUM) / a.numel()


def mean_abs_g(ctx, a):
    """mean_g(abs.(a)) -- Dimensional/HydroThermal3D_v18.jl:460."""
    return _reduce(ctx, a, abi.RED_SUM_ABS) / a.numel()


def maximum_abs_g(ctx, a):
    return _reduce(ctx, a, abi.RED_MAX_ABS)


# ------------------------------------------------------ WENO5
def VPlusMinus(ctx, Vm, Vp, V, axis):
    nx, ny, nz = _cells(Vm)
    ctx.call("ht3d_VPlusMinus", _ptr(Vm), _ptr(Vp), _ptr(V), axis, nx, ny, nz)


def VxPlusMinus(ctx, Vxm, Vxp, Vx):
    VPlusMinus(ctx, Vxm, Vxp, Vx, 0)


def VyPlusMinus(ctx, Vym, Vyp, Vy):
    VPlusMinus(ctx, Vym, Vyp, Vy, 1)


def VzPlusMinus(ctx, Vzm, Vzp, Vz):
    VPlusMinus(ctx, Vzm, Vzp, Vz, 2)


def dFdx_Weno5(ctx, dFdxi, V1, V2, V3, V4, V5):
    ctx.call("ht3d_dFdx_Weno5", _ptr(dFdxi), _ptr(V1), _ptr(V2), _ptr(V3), _ptr(V4), _ptr(V5), _numel(dFdxi))


def Gradients_Weno5(ctx, v1, v2, v3, v4, v5, Fc_exxx, axis, sign, _dx, _dy, _dz):
    nx, ny, nz = _cells(v1); S = _shapes(nx, ny, nz)
    ctx.call("ht3d_Gradients_Weno5", _ptr(v1), _ptr(v2), _ptr(v3), _ptr(v4), _ptr(v5), _ptr(Fc_exxx, S["xxx"]),
             axis, sign, _dx, _dy, _dz, nx, ny, nz)


def Boundaries_Weno5(ctx, Fc_exxx, Fc, axis, type_L, val_L, type_R, val_R):
    nx, ny, nz = (int(s) - 6 for s in Fc_exxx.shape)
    ghosted = 1 if tuple(Fc.shape) == (nx + 2, ny + 2, nz + 2) else 0
    ctx.call("ht3d_Boundaries_Weno5", _ptr(Fc_exxx), _ptr(Fc), axis, type_L, val_L, type_R, val_R, ghosted,
             nx, ny, nz)


def Advect_v1(ctx, Fc, Vxp, dTdxm, Vxm, dTdxp, dt):
    ctx.call("ht3d_Advect_v1", _ptr(Fc), _ptr(Vxp), _ptr(dTdxm), _ptr(Vxm), _ptr(dTdxp), dt, _numel(Fc))


def TimeAveraging_v1(ctx, Fc, Fold, order):
    ctx.call("ht3d_TimeAveraging_v1", _ptr(Fc), _ptr(Fold), order, _numel(Fc))


def Advect_v2(ctx, Fc_ex, X, V, axis, dt, _dx, _dy, _dz, quirk=1):
    nx, ny, nz = _cells_ex(Fc_ex, "Fc")
    ctx.call("ht3d_Advect_v2", _ptr(Fc_ex), _ptr(X), _ptr(V), axis, dt, _dx, _dy, _dz, quirk, nx, ny, nz)


def TimeAveraging_v2(ctx, Fc_ex, Fold, order):
    nx, ny, nz = _cells(Fold)
    ctx.call("ht3d_TimeAveraging_v2", _ptr(Fc_ex), _ptr(Fold), order, nx, ny, nz)


def weno5_advect(ctx, Tc_ex, Vx, Vy, Vz, dt, _dx, _dy, _dz, bc_type6, bc_val6, variant=abi.WENO_V1,
                 precision=abi.FP64):
    nx, ny, nz = _cells_ex(Tc_ex, "Tc_ex"); S = _shapes(nx, ny, nz)
    ctx.call("ht3d_weno5_advect", _ptr(Tc_ex, S["ex"]), _ptr(Vx, S["fx"]), _ptr(Vy, S["fy"]), _ptr(Vz, S["fz"]), dt,
             _dx, _dy, _dz, abi.int6(*bc_type6), abi.dbl6(*bc_val6), variant, precision, nx, ny, nz)


def weno5_advect_f32(ctx, Tc_ex, Vx, Vy, Vz, dt, _dx, _dy, _dz, bc_type6, bc_val6, variant=abi.WENO_V1):
    """FP32 fused sweep (float32 fields of the same shapes)."""
    nx, ny, nz = _cells_ex(Tc_ex, "Tc_ex"); S = _shapes(nx, ny, nz)
    f = torch.float32
    ctx.call("ht3d_weno5_advect_f32", _ptr(Tc_ex, S["ex"], "Tc_ex", f), _ptr(Vx, S["fx"], "Vx", f),
             _ptr(Vy, S["fy"], "Vy", f), _ptr(Vz, S["fz"], "Vz", f), dt, _dx, _dy, _dz, abi.int6(*bc_type6),
             abi.dbl6(*bc_val6), variant, nx, ny, nz)


# ------------------------------------------------------ fused solver / step
def dyrel_solve_dimless(ctx, X_ex, R, kx, ky, kz, cX, dx, dy, dz, bc_type6, bc_val6, params, F, F0,
                        precision=abi.FP64, n_iter_fixed=0):
    nx, ny, nz = _cells_ex(X_ex, "X_ex"); S = _shapes(nx, ny, nz)
    st = abi.DyrelStats()
    ctx.call("ht3d_dyrel_solve_dimless", _ptr(X_ex, S["ex"]), _ptr(R, S["c"], "R"), _ptr(kx, S["fx"], "kx"),
             _ptr(ky, S["fy"], "ky"), _ptr(kz, S["fz"], "kz"), cX, dx, dy, dz, abi.int6(*bc_type6),
             abi.dbl6(*bc_val6), ctypes.byref(params), n_iter_fixed, _ptr(F, S["c"], "F"), _ptr(F0, S["c"], "F0"),
             precision, ctypes.byref(st), nx, ny, nz)
    return st


def step_hrl(ctx, Tc_ex, Pc_ex, ktv, kfv, Vx, Vy, Vz, params, precision=abi.FP64):
    nx, ny, nz = _cells_ex(Tc_ex, "Tc_ex"); S = _shapes(nx, ny, nz)
    st_t, st_d = abi.DyrelStats(), abi.DyrelStats()
    ctx.call("ht3d_step_hrl", _ptr(Tc_ex, S["ex"]), _ptr(Pc_ex, S["ex"]), _ptr(ktv, S["v"]), _ptr(kfv, S["v"]),
             _ptr(Vx, S["fx"]), _ptr(Vy, S["fy"]), _ptr(Vz, S["fz"]), ctypes.byref(params), ctypes.byref(st_t),
             ctypes.byref(st_d), precision, nx, ny, nz)
    return st_t, st_d


class Member:
    """One ensemble member: device fields (torch, column-major FP64) and its
    host HrlParams; step statistics land in st_thermal / st_darcy."""

    def __init__(self, Tc_ex, Pc_ex, ktv, kfv, Vx, Vy, Vz, params):
        self.Tc_ex, self.Pc_ex, self.ktv, self.kfv = Tc_ex, Pc_ex, ktv, kfv
        self.Vx, self.Vy, self.Vz = Vx, Vy, Vz
        self.params = params
        self.st_thermal, self.st_darcy = abi.DyrelStats(), abi.DyrelStats()
        self.status = abi.OK


def SetInitialConditions_Khaled(ctx, phc_ex, phv, wN, case, Tc_ex, Pc_ex):
    """Device SetInitialConditions_Khaled; `case` is v18.khaled_case()'s dict."""
    nx, ny, nz = case["nx"], case["ny"], case["nz"]
    S = _shapes(nx, ny, nz)
    ctx.call("ht3d_SetInitialConditions_Khaled", _ptr(phc_ex, S["ex"], "phc_ex"), _ptr(phv, S["v"], "phv"),
             _ptr(wN, (nx + 2, nz + 2), "wN"), ctypes.byref(case["geom"]), _ptr(Tc_ex, S["ex"], "Tc_ex"),
             _ptr(Pc_ex, S["ex"], "Pc_ex"), case["Tbot"], case["Ttop"], case["Pbot"], case["Ptop"], case["xmin"],
             case["ymin"], case["zmin"], case["xmax"], case["ymax"], case["zmax"], case["L"], nx, ny, nz)


def ensemble_step(ctx, members, precision=abi.MIXED):
    """One time step of every member (ht3d_ensemble_step); returns the statuses.
    Raises on the first failing member like step_hrl does."""
    arr = (abi.Instance * len(members))()
    for rec, m in zip(arr, members):
        nx, ny, nz = _cells_ex(m.Tc_ex, "Tc_ex"); S = _shapes(nx, ny, nz)
        rec.Tc_ex, rec.Pc_ex = _ptr(m.Tc_ex, S["ex"], "Tc_ex"), _ptr(m.Pc_ex, S["ex"], "Pc_ex")
        rec.ktv, rec.kfv = _ptr(m.ktv, S["v"], "ktv"), _ptr(m.kfv, S["v"], "kfv")
        rec.Vx, rec.Vy, rec.Vz = _ptr(m.Vx, S["fx"], "Vx"), _ptr(m.Vy, S["fy"], "Vy"), _ptr(m.Vz, S["fz"], "Vz")
        rec.params = ctypes.pointer(m.params)
        rec.st_thermal, rec.st_darcy = ctypes.pointer(m.st_thermal), ctypes.pointer(m.st_darcy)
        rec.nx, rec.ny, rec.nz = nx, ny, nz
    st = ctx.lib.ht3d_ensemble_step(ctx.ptr, arr, len(members), precision)
    for rec, m in zip(arr, members):
        m.status = rec.status
    ctx.check(st)
    return [m.status for m in members]


# ------------------------------------------------------ dimensional kernels
def ComputeThermalConductivity(ctx, ktv, Tce, phv, phi0, scale_kt, scale_T):
    nx, ny, nz = _cells_ex(Tce, "Tce"); S = _shapes(nx, ny, nz)
    ctx.call("ht3d_ComputeThermalConductivity", _ptr(ktv, S["v"]), _ptr(Tce, S["ex"]), _ptr(phv, S["v"]), phi0,
             scale_kt, scale_T, nx, ny, nz)


def ComputeHydroConductivity(ctx, kfv, Tce, Pce, phv, ymin, dy, k_fact, delta, scale_sigma, scale_T, scale_L,
                             scale_t, scale_eta, mode, kmul=None):
    nx, ny, nz = _cells_ex(Tce, "Tce"); S = _shapes(nx, ny, nz)
    ctx.call("ht3d_ComputeHydroConductivity", _ptr(kfv, S["v"]), _ptr(Tce, S["ex"]), _ptr(Pce, S["ex"]),
             _ptr(phv, S["v"]), ymin, dy, k_fact, delta, scale_sigma, scale_T, scale_L, scale_t, scale_eta, mode,
             None if kmul is None else _ptr(kmul, S["v"]), nx, ny, nz)


def ComputeFluidDensity(ctx, rhofv, Tce, Pce, phv, scale_sigma, scale_T, scale_rho):
    nx, ny, nz = _cells_ex(Tce, "Tce"); S = _shapes(nx, ny, nz)
    ctx.call("ht3d_ComputeFluidDensity", _ptr(rhofv, S["v"]), _ptr(Tce, S["ex"]), _ptr(Pce, S["ex"]),
             _ptr(phv, S["v"]), scale_sigma, scale_T, scale_rho, nx, ny, nz)


def SmoothConductivityV2C(ctx, ktc, ktv):
    nx, ny, nz = _cells(ktc)
    ctx.call("ht3d_SmoothConductivityV2C", _ptr(ktc), _ptr(ktv, (nx + 1, ny + 1, nz + 1)), nx, ny, nz)


def SmoothConductivityC2V(ctx, ktv, ktc):
    nx, ny, nz = _cells(ktc)
    ctx.call("ht3d_SmoothConductivityC2V", _ptr(ktv, (nx + 1, ny + 1, nz + 1)), _ptr(ktc), nx, ny, nz)


def InitConductivity(ctx, kx, ky, kz, ktv):
    nx, ny, nz = (int(s) - 1 for s in ktv.shape); S = _shapes(nx, ny, nz)
    ctx.call("ht3d_InitConductivity", _ptr(kx, S["fx"]), _ptr(ky, S["fy"]), _ptr(kz, S["fz"]), _ptr(ktv), nx, ny, nz)


def ComputeRhoCeffective(ctx, rhoC_eff, Tc_ex, Pc_ex, phc_ex, phi_i, sca_T, sca_sigma, sca_C, sca_rho):
    nx, ny, nz = _cells(rhoC_eff); S = _shapes(nx, ny, nz)
    ctx.call("ht3d_ComputeRhoCeffective", _ptr(rhoC_eff), _ptr(Tc_ex, S["ex"]), _ptr(Pc_ex, S["ex"]),
             _ptr(phc_ex, S["ex"]), phi_i, sca_T, sca_sigma, sca_C, sca_rho, nx, ny, nz)


def ResidualTemperatureLinearised(ctx, F, Tc_ex, Tc_old, rhoC_eff, phc_ex, PC, qx, qy, qz, Qt, transient, _dt, _dx,
                                  _dy, _dz):
    nx, ny, nz = _cells(F); S = _shapes(nx, ny, nz)
    ctx.call("ht3d_ResidualTemperatureLinearised", _ptr(F), _ptr(Tc_ex, S["ex"]), _ptr(Tc_old, S["c"]),
             _ptr(rhoC_eff, S["c"]), _ptr(phc_ex, S["ex"]), _ptr(PC, S["c"]), _ptr(qx, S["fx"]), _ptr(qy, S["fy"]),
             _ptr(qz, S["fz"]), Qt, transient, _dt, _dx, _dy, _dz, nx, ny, nz)


def SetTemperatureBCs(ctx, Tc_ex, ky, wN, phc_ex, qyS, _dy, kS, TS, TN, y_plateau=0.0, a2=0.0, b2=0.0, dTdy=0.0,
                      dx=0.0, dy=0.0, sticky_air=0, sca_T=1.0, sca_kT=1.0, phi_i=0.0):
    nx, ny, nz = _cells_ex(Tc_ex, "Tc_ex"); S = _shapes(nx, ny, nz)
    ctx.call("ht3d_SetTemperatureBCs", _ptr(Tc_ex), _ptr(ky, S["fy"]), _ptr(wN, (nx + 2, nz + 2)),
             _ptr(phc_ex, S["ex"]), qyS, _dy, kS, TS, TN, y_plateau, a2, b2, dTdy, dx, dy, int(sticky_air), sca_T,
             sca_kT, phi_i, nx, ny, nz)


def SetPressureBCs_dim(ctx, Pc_ex, wN, phc_ex, PS, PN, y_plateau=0.0, a2=0.0, b2=0.0, rhof=0.0, g=0.0, dx=0.0,
                       dy=0.0, sticky_air=0):
    nx, ny, nz = _cells_ex(Pc_ex, "Pc_ex"); S = _shapes(nx, ny, nz)
    ctx.call("ht3d_SetPressureBCs_dim", _ptr(Pc_ex), _ptr(wN, (nx + 2, nz + 2)), _ptr(phc_ex, S["ex"]), PS, PN,
             y_plateau, a2, b2, rhof, g, dx, dy, int(sticky_air), nx, ny, nz)


def _phirhof(name, ctx, out, T, P, phc_ex, phi_i, scale_rho, scale_T, scale_sigma):
    nx, ny, nz = _cells(out); S = _shapes(nx, ny, nz)
    ctx.call(name, _ptr(out), _ptr(T), _ptr(P), _ptr(phc_ex, S["ex"]), phi_i, scale_rho, scale_T, scale_sigma,
             nx, ny, nz)


def PhiRhof(ctx, phirhofc, Tc_ex, Pc_ex, phc_ex, phi_i, scale_rho, scale_T, scale_sigma):
    _phirhof("ht3d_PhiRhof", ctx, phirhofc, Tc_ex, Pc_ex, phc_ex, phi_i, scale_rho, scale_T, scale_sigma)


def PhiRhofOld(ctx, phirhofc, Tc0, Pc0, phc_ex, phi_i, scale_rho, scale_T, scale_sigma):
    _phirhof("ht3d_PhiRhofOld", ctx, phirhofc, Tc0, Pc0, phc_ex, phi_i, scale_rho, scale_T, scale_sigma)


def PhiDrhodP(ctx, phidrhodP, Tc_ex, Pc_ex, phc_ex, phi_i, scale_rho, scale_T, scale_sigma):
    _phirhof("ht3d_PhiDrhodP", ctx, phidrhodP, Tc_ex, Pc_ex, phc_ex, phi_i, scale_rho, scale_T, scale_sigma)


def ComputeDarcyFlux(ctx, qx, qy, qz, rhofv, kx, ky, kz, Pf, g, _dx, _dy, _dz):
    nx, ny, nz = _cells_ex(Pf, "Pf"); S = _shapes(nx, ny, nz)
    ctx.call("ht3d_ComputeDarcyFlux", _ptr(qx, S["fx"]), _ptr(qy, S["fy"]), _ptr(qz, S["fz"]), _ptr(rhofv, S["v"]),
             _ptr(kx, S["fx"]), _ptr(ky, S["fy"]), _ptr(kz, S["fz"]), _ptr(Pf, S["ex"]), g, _dx, _dy, _dz, nx, ny, nz)


def ResidualFluidPressure(ctx, F, phc_ex, phirhofc, phirhofc0, PC, qx, qy, qz, transient, _dt, _dx, _dy, _dz):
    nx, ny, nz = _cells(F); S = _shapes(nx, ny, nz)
    ctx.call("ht3d_ResidualFluidPressure", _ptr(F), _ptr(phc_ex, S["ex"]), _ptr(phirhofc, S["c"]),
             _ptr(phirhofc0, S["c"]), _ptr(PC, S["c"]), _ptr(qx, S["fx"]), _ptr(qy, S["fy"]), _ptr(qz, S["fz"]),
             transient, _dt, _dx, _dy, _dz, nx, ny, nz)


def Init_vel_dim(ctx, Vx, Vy, Vz, qx, qy, qz, rhofv):
    nx, ny, nz = (int(s) - 1 for s in rhofv.shape); S = _shapes(nx, ny, nz)
    ctx.call("ht3d_Init_vel_dim", _ptr(Vx, S["fx"]), _ptr(Vy, S["fy"]), _ptr(Vz, S["fz"]), _ptr(qx, S["fx"]),
             _ptr(qy, S["fy"]), _ptr(qz, S["fz"]), _ptr(rhofv, S["v"]), nx, ny, nz)


def material_law(ctx, which, a, b=None):
    out = torch.empty_like(a)
    ctx.call("ht3d_material_law", which, _ptr(a), None if b is None else _ptr(b), _ptr(out), _numel(a))
    return out


def step_v18(ctx, Tc_ex, Pc_ex, phc_ex, phv, wN, kmul, Vx, Vy, Vz, params):
    nx, ny, nz = _cells_ex(Tc_ex, "Tc_ex"); S = _shapes(nx, ny, nz)
    st_t, st_d = abi.DyrelStats(), abi.DyrelStats()
    ctx.call("ht3d_step_v18", _ptr(Tc_ex, S["ex"]), _ptr(Pc_ex, S["ex"]), _ptr(phc_ex, S["ex"]), _ptr(phv, S["v"]),
             _ptr(wN, (nx + 2, nz + 2)), None if kmul is None else _ptr(kmul, S["v"]), _ptr(Vx, S["fx"]),
             _ptr(Vy, S["fy"]), _ptr(Vz, S["fz"]), ctypes.byref(params), ctypes.byref(st_t), ctypes.byref(st_d),
             nx, ny, nz)
    return st_t, st_d


# ------------------------------------------------------ output diagnostics
# Dimensional/kernels_HT3D_postprocessing.jl: X is a cell array (nx, ny, nz);
# phc_ex, Tc_ex, Pc_ex are ghosted; Vx/Vy/Vz are face arrays.
def Phase(ctx, X, phc_ex):
    nx, ny, nz = _cells(X); S = _shapes(nx, ny, nz)
    ctx.call("ht3d_Phase", _ptr(X, S["c"], "X"), _ptr(phc_ex, S["ex"], "phc_ex"), nx, ny, nz)


def Pressure(ctx, X, Pc_ex, phc_ex, scale_sigma):
    nx, ny, nz = _cells(X); S = _shapes(nx, ny, nz)
    ctx.call("ht3d_Pressure", _ptr(X, S["c"], "X"), _ptr(Pc_ex, S["ex"], "Pc_ex"), _ptr(phc_ex, S["ex"], "phc_ex"),
             scale_sigma, nx, ny, nz)


def Temperature(ctx, X, Tc_ex, phc_ex, scale_T):
    nx, ny, nz = _cells(X); S = _shapes(nx, ny, nz)
    ctx.call("ht3d_Temperature", _ptr(X, S["c"], "X"), _ptr(Tc_ex, S["ex"], "Tc_ex"), _ptr(phc_ex, S["ex"], "phc_ex"),
             scale_T, nx, ny, nz)


def Velocity(ctx, X, Y, Z, Vx, Vy, Vz, phc_ex, scale_V):
    nx, ny, nz = _cells(X); S = _shapes(nx, ny, nz)
    ctx.call("ht3d_Velocity", _ptr(X, S["c"], "X"), _ptr(Y, S["c"], "Y"), _ptr(Z, S["c"], "Z"),
             _ptr(Vx, S["fx"], "Vx"), _ptr(Vy, S["fy"], "Vy"), _ptr(Vz, S["fz"], "Vz"),
             _ptr(phc_ex, S["ex"], "phc_ex"), scale_V, nx, ny, nz)


def EffectiveThermalConductivity(ctx, X, Tc_ex, phi0, phc_ex, scale_T):
    nx, ny, nz = _cells(X); S = _shapes(nx, ny, nz)
    ctx.call("ht3d_EffectiveThermalConductivity", _ptr(X, S["c"], "X"), _ptr(Tc_ex, S["ex"], "Tc_ex"), phi0,
             _ptr(phc_ex, S["ex"], "phc_ex"), scale_T, nx, ny, nz)


def EffectiveHeatCapacity(ctx, Ceff, Tc_ex, Pc_ex, phc_ex, phi_i, sca_T, sca_sigma, sca_C, sca_rho):
    nx, ny, nz = _cells(Ceff); S = _shapes(nx, ny, nz)
    ctx.call("ht3d_EffectiveHeatCapacity", _ptr(Ceff, S["c"], "Ceff"), _ptr(Tc_ex, S["ex"], "Tc_ex"),
             None if Pc_ex is None else _ptr(Pc_ex, S["ex"], "Pc_ex"), _ptr(phc_ex, S["ex"], "phc_ex"), phi_i, sca_T,
             sca_sigma, sca_C, sca_rho, nx, ny, nz)


def Permeability(ctx, X, k_fact, ymin, dy, phc_ex, delta, scale_L):
    nx, ny, nz = _cells(X); S = _shapes(nx, ny, nz)
    ctx.call("ht3d_Permeability", _ptr(X, S["c"], "X"), k_fact, ymin, dy, _ptr(phc_ex, S["ex"], "phc_ex"), delta,
             scale_L, nx, ny, nz)


def FluidDensity(ctx, X, Tc_ex, Pc_ex, phc_ex, scale_T, scale_sigma):
    nx, ny, nz = _cells(X); S = _shapes(nx, ny, nz)
    ctx.call("ht3d_FluidDensity", _ptr(X, S["c"], "X"), _ptr(Tc_ex, S["ex"], "Tc_ex"), _ptr(Pc_ex, S["ex"], "Pc_ex"),
             _ptr(phc_ex, S["ex"], "phc_ex"), scale_T, scale_sigma, nx, ny, nz)


def Viscosity(ctx, X, Tc_ex, phc_ex, scale_T):
    nx, ny, nz = _cells(X); S = _shapes(nx, ny, nz)
    ctx.call("ht3d_Viscosity", _ptr(X, S["c"], "X"), _ptr(Tc_ex, S["ex"], "Tc_ex"), _ptr(phc_ex, S["ex"], "phc_ex"),
             scale_T, nx, ny, nz)


def Peclet(ctx, X, Tc_ex, Pc_ex, Vx, Vy, Vz, phc_ex, phi0, scale_T, scale_sigma, scale_V, scale_L):
    nx, ny, nz = _cells(X); S = _shapes(nx, ny, nz)
    ctx.call("ht3d_Peclet", _ptr(X, S["c"], "X"), _ptr(Tc_ex, S["ex"], "Tc_ex"), _ptr(Pc_ex, S["ex"], "Pc_ex"),
             _ptr(Vx, S["fx"], "Vx"), _ptr(Vy, S["fy"], "Vy"), _ptr(Vz, S["fz"], "Vz"),
             _ptr(phc_ex, S["ex"], "phc_ex"), phi0, scale_T, scale_sigma, scale_V, scale_L, nx, ny, nz)


def postprocess_fields(ctx, out, Tc_ex, Pc_ex, Vx, Vy, Vz, phc_ex, **params):
    """Every diagnostic named in `out` (a dict field name -> cell tensor, field
    names as abi.POST_FIELDS) in one pass; `params` are abi.PostParams fields."""
    nx, ny, nz = _cells_ex(phc_ex, "phc_ex"); S = _shapes(nx, ny, nz)
    f = abi.PostFields()
    for name, t in out.items():
        if name not in abi.POST_FIELDS:
            raise ValueError(f"unknown diagnostic {name!r}")
        setattr(f, name, _ptr(t, S["c"], name))
    p = abi.PostParams(**{k: float(v) for k, v in params.items()})
    opt = lambda t, shape, name: None if t is None else _ptr(t, shape, name)
    ctx.call("ht3d_postprocess_fields", ctypes.byref(f), opt(Tc_ex, S["ex"], "Tc_ex"), opt(Pc_ex, S["ex"], "Pc_ex"),
             opt(Vx, S["fx"], "Vx"), opt(Vy, S["fy"], "Vy"), opt(Vz, S["fz"], "Vz"), _ptr(phc_ex, S["ex"], "phc_ex"),
             ctypes.byref(p), nx, ny, nz)


def Nusselt(ctx, qy, Lx, Lz):
    """Nu = sum(qy[:,end,:]) / (Lx*Lz) / (nx*nz) of the (nx, ny+1, nz) y-flux."""
    nx, ny1, nz = _cells(qy)
    out = ctypes.c_double()
    ctx.call("ht3d_Nusselt", _ptr(qy, (nx, ny1, nz), "qy"), Lx, Lz, nx, ny1 - 1, nz, ctypes.byref(out))
    return out.value


# ------------------------------------------------------ output and restart files
def write_vtr(path, xc, yc, zc, fields):
    """vtk_grid(path, xc, yc, zc) + vtkfile[name] = array (v18.jl:664-686).

    fields: dict name -> (nx, ny, nz) array, or a tuple of three for a vector
    field; numpy arrays or device tensors (copied to the host).  Returns the
    file name written (".vtr" appended)."""
    import numpy as np
    lib = _lib.load()
    host = lambda a: np.asfortranarray(to_numpy(a) if isinstance(a, torch.Tensor) else a, dtype=np.float64)
    xc, yc, zc = (np.ascontiguousarray(np.asarray(c, dtype=np.float64).ravel()) for c in (xc, yc, zc))
    n = (xc.size, yc.size, zc.size)
    names, ncomp, arrs = [], [], []
    for name, v in fields.items():
        comps = v if isinstance(v, (tuple, list)) else (v,)
        if len(comps) not in (1, 3):
            raise ValueError(f"{name}: a field has 1 or 3 components")
        for a in comps:
            a = host(a)
            if a.shape != n:
                raise ValueError(f"{name}: shape {a.shape} does not match the coordinates {n}")
            arrs.append(a)
        names.append(name.encode())
        ncomp.append(len(comps))
    c_names = (ctypes.c_char_p * max(1, len(names)))(*names)
    c_ncomp = (ctypes.c_int * max(1, len(ncomp)))(*ncomp)
    c_data = (ctypes.c_void_p * max(1, len(arrs)))(*[a.ctypes.data for a in arrs])
    st = lib.ht3d_write_vtr(str(path).encode(), xc.ctypes.data, yc.ctypes.data, zc.ctypes.data, *n, len(names),
                            c_names, c_ncomp, c_data)
    if st != abi.OK:
        raise Ht3dError(st, lib.ht3d_status_string(st).decode())
    p = str(path)
    return p if p.endswith(".vtr") else p + ".vtr"


def _h5(path):
    return str(path).endswith(".h5")


def breakpoint_write(ctx, path, Tc_ex, Pc_ex, time, dt):
    """Restart state Tc_ex, Pc_ex, time, dt to a file (v18.jl:579-588): the
    reference's HDF5 format when the path ends in .h5 (ht3d_breakpoint_write_h5),
    else the library's raw format (ht3d_breakpoint_write)."""
    nx, ny, nz = _cells_ex(Tc_ex, "Tc_ex"); S = _shapes(nx, ny, nz)
    ctx.call("ht3d_breakpoint_write_h5" if _h5(path) else "ht3d_breakpoint_write", str(path).encode(),
             _ptr(Tc_ex, S["ex"], "Tc_ex"), _ptr(Pc_ex, S["ex"], "Pc_ex"), float(time), float(dt), nx, ny, nz)


def breakpoint_read(ctx, path, Tc_ex, Pc_ex):
    """Fill Tc_ex, Pc_ex from a restart file (v18.jl:384-395), HDF5 when the
    path ends in .h5, else raw; returns (time, dt)."""
    nx, ny, nz = _cells_ex(Tc_ex, "Tc_ex"); S = _shapes(nx, ny, nz)
    t, d = ctypes.c_double(), ctypes.c_double()
    ctx.call("ht3d_breakpoint_read_h5" if _h5(path) else "ht3d_breakpoint_read", str(path).encode(),
             _ptr(Tc_ex, S["ex"], "Tc_ex"), _ptr(Pc_ex, S["ex"], "Pc_ex"), ctypes.byref(t), ctypes.byref(d), nx, ny,
             nz)
    return t.value, d.value
