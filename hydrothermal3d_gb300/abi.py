"""ctypes mirrors of the parameter structs and constants of include/ht3d.h."""
import ctypes

OK = 0
ERR_ARG, ERR_CUDA, ERR_NAN, ERR_DIVERGED, ERR_MAXITER, ERR_TIMEOUT, ERR_NOMEM, ERR_SCRATCH, ERR_IO = 1, 2, 3, 4, 5, 6, 7, 8, 9
FP64, MIXED = 0, 1
BC_NEUMANN, BC_DIRICHLET, BC_PERIODIC = 0, 1, 2
WENO_V1, WENO_V2_REF, WENO_V2_FIXED = 0, 1, 2
RED_SUM, RED_SUM_ABS, RED_MAX, RED_MIN, RED_MAX_ABS = 0, 1, 2, 3, 4
TUNE_DYREL_VARIANT = 1
TUNE_MIXED_REFRESH = 2
TUNE_TIME_INNER = 3
TUNE_ENS_BLOCK = 4
TUNE_ENS_GRAPH = 5
TUNE_TEMPORAL = 6
TUNE_WAIT_TEST = 7
TUNE_ENS_TILE = 8
DYREL_ZMARCH, DYREL_CELL = 1, 2


class DyrelParams(ctypes.Structure):
    """ht3d_dyrel_params: DYREL controls of Dimensional/HydroThermal3D_v18.jl:292-303,433-439."""
    _fields_ = [
        ("tol_abs", ctypes.c_double),
        ("tol_rel", ctypes.c_double),
        ("nitmax", ctypes.c_int),
        ("nitout", ctypes.c_int),
        ("cfl", ctypes.c_double),
        ("cfact", ctypes.c_double),
        ("lmin_ratio", ctypes.c_double),
        ("norm_scale", ctypes.c_double),
    ]

    @classmethod
    def reference(cls, tol=1e-8, nitmax=10000, nitout=1000, norm_scale=1.0):
        """The reference's values: CFL 0.99, cfact 0.5, lambda_min = lambda_max/500."""
        return cls(tol_abs=tol, tol_rel=tol, nitmax=nitmax, nitout=nitout, cfl=0.99, cfact=0.5, lmin_ratio=500.0,
                   norm_scale=norm_scale)


class DyrelStats(ctypes.Structure):
    _fields_ = [
        ("iters", ctypes.c_int),
        ("converged", ctypes.c_int),
        ("status", ctypes.c_int),
        ("checks", ctypes.c_int),
        ("nF_abs", ctypes.c_double),
        ("nF_rel", ctypes.c_double),
        ("nF_ini", ctypes.c_double),
        ("lambda_min", ctypes.c_double),
        ("lambda_max", ctypes.c_double),
        ("h1", ctypes.c_double),
        ("h2", ctypes.c_double),
        ("dtau", ctypes.c_double),
    ]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


Int6 = ctypes.c_int * 6
Dbl6 = ctypes.c_double * 6


class HrlParams(ctypes.Structure):
    """ht3d_hrl_params: one time step of the dimensionless HRL model."""
    _fields_ = [
        ("Ra", ctypes.c_double),
        ("dx", ctypes.c_double),
        ("dy", ctypes.c_double),
        ("dz", ctypes.c_double),
        ("dt", ctypes.c_double),
        ("Tbot", ctypes.c_double),
        ("Ttop", ctypes.c_double),
        ("thermal_bc", Int6),
        ("thermal_val", Dbl6),
        ("darcy_bc", Int6),
        ("darcy_val", Dbl6),
        ("weno_bc", Int6),
        ("weno_val", Dbl6),
        ("weno_variant", ctypes.c_int),
        ("kill_ns", ctypes.c_int),
        ("dt_adapt", ctypes.c_int),
        ("advection", ctypes.c_int),
        ("dt_fact", ctypes.c_double),
        ("thermal", DyrelParams),
        ("darcy", DyrelParams),
        ("dt_max", ctypes.c_double),
    ]


class KhaledGeom(ctypes.Structure):
    """ht3d_khaled_geom: the detachment-fault geometry (lines y = a x + b)."""
    _fields_ = [
        ("y_plateau", ctypes.c_double),
        ("surf_a1", ctypes.c_double),
        ("surf_b1", ctypes.c_double),
        ("fault", (ctypes.c_double * 6) * 4),
    ]


class PostParams(ctypes.Structure):
    """ht3d_post_params: scales and constants of the output diagnostics."""
    _fields_ = [(f, ctypes.c_double) for f in (
        "phi0", "scale_T", "scale_sigma", "scale_V", "scale_L", "k_fact", "ymin", "dy", "delta")]


POST_FIELDS = ("phase", "pressure", "temperature", "vx", "vy", "vz", "k_thermal", "heat_capacity", "permeability",
               "density", "viscosity", "peclet")


class PostFields(ctypes.Structure):
    """ht3d_post_fields: device output pointers of ht3d_postprocess_fields (NULL skips a field)."""
    _fields_ = [(f, ctypes.c_void_p) for f in POST_FIELDS]


class Instance(ctypes.Structure):
    """ht3d_instance: one member of an ensemble (the arguments of one ht3d_step_hrl)."""
    _fields_ = [
        ("Tc_ex", ctypes.c_void_p),
        ("Pc_ex", ctypes.c_void_p),
        ("ktv", ctypes.c_void_p),
        ("kfv", ctypes.c_void_p),
        ("Vx", ctypes.c_void_p),
        ("Vy", ctypes.c_void_p),
        ("Vz", ctypes.c_void_p),
        ("params", ctypes.POINTER(HrlParams)),
        ("st_thermal", ctypes.POINTER(DyrelStats)),
        ("st_darcy", ctypes.POINTER(DyrelStats)),
        ("nx", ctypes.c_int),
        ("ny", ctypes.c_int),
        ("nz", ctypes.c_int),
        ("status", ctypes.c_int),
    ]


def int6(*v):
    return Int6(*v)


def dbl6(*v):
    return Dbl6(*[float(x) for x in v])


class V18Params(ctypes.Structure):
    """ht3d_v18_params: one time step of the dimensional model (Dimensional/HydroThermal3D_v18.jl)."""
    _fields_ = [(f, ctypes.c_double) for f in (
        "dx", "dy", "dz", "ymin", "dt", "time", "phi_i", "k_fact", "delta", "g", "Qt", "qyS", "Ttop", "Tbot", "Ptop",
        "Pbot", "T_pluton", "C_adv", "sc_T", "sc_L", "sc_t", "sc_eta", "sc_sigma", "sc_rho", "sc_C", "sc_kt")] + [
        (f, ctypes.c_int) for f in ("it", "thermal", "hydro", "advection", "dt_constant", "weno_variant")] + [
        ("thermal_dyrel", DyrelParams), ("darcy_dyrel", DyrelParams), ("n_adv", ctypes.c_int), ("pad_", ctypes.c_int)]
