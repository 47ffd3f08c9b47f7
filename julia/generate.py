"""Generates julia/HT3D.jl, the Julia binding of libht3d.so, from include/ht3d.h.

    python julia/generate.py            # rewrites julia/HT3D.jl

Three layers are written:
  * `HT3D.C`: one function per prototype of the header, same name, same
    arguments, a plain `ccall` whose argument types follow the C types (device
    arrays as `CuPtr`, host arrays as `Ptr`, structs by `Ref`);
  * the parameter structs, mirrored field by field from the ctypes mirror
    (hydrothermal3d_gb300/abi.py) with their sizes checked against the
    library at load time;
  * drop-in `Kernel!(args...)` wrappers under the reference's kernel names
    (`ComputeFlux!`, `ϕρf`, `Gradients_minus_x_Weno5!`, ...), taking the
    reference's arguments in the reference's order, inferring nx, ny, nz from
    the array shapes, checking every array's staggering and throwing
    `Ht3dError` on a non-zero status, so a driver line
    `@parallel ComputeFlux!(qx, qy, qz, kx, ky, kz, Tc_ex, _dx, _dy, _dz)`
    becomes `HT3D.ComputeFlux!(qx, qy, qz, kx, ky, kz, Tc_ex, _dx, _dy, _dz)`;
    plus wrappers of the fused entry points (`step_hrl!`, `step_v18!`, ...).

The array staggering of every wrapper is read from the Python mirror
(hydrothermal3d_gb300/api.py: the `_ptr(name, S["key"])` of each call), so the
two host mirrors check the same shapes.  tests/test_julia_binding.py parses the
generated file and checks it against the header and abi.py.
"""
import ast
import ctypes
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
HEADER = os.path.join(ROOT, "include", "ht3d.h")
API = os.path.join(ROOT, "hydrothermal3d_gb300", "api.py")
OUT = os.path.join(HERE, "HT3D.jl")
sys.path.insert(0, ROOT)

# ----------------------------------------------------------------- header
_PROTO = re.compile(r"^\s*([A-Za-z_][A-Za-z0-9_ ]*?\**)\s*\b(ht3d_[A-Za-z0-9_]+)\s*\(([^;]*?)\)\s*;", re.M | re.S)


def _strip_comments(src):
    src = re.sub(r"/\*.*?\*/", " ", src, flags=re.S)
    return re.sub(r"//[^\n]*", " ", src)


def parse_header(path=HEADER):
    """[(ret, name, [(ctype, pname)])] in header order."""
    with open(path) as f:
        src = _strip_comments(f.read())
    out = []
    for m in _PROTO.finditer(src):
        ret = " ".join(m.group(1).split()).replace(" *", "*")
        params = []
        for q in (x.strip() for x in m.group(3).split(",")):
            q = " ".join(q.split())
            if not q or q == "void":
                continue
            q = q.replace(" *", "*").replace("* ", "* ")
            mm = re.match(r"^(.*?[\s\*])([A-Za-z_][A-Za-z0-9_]*)$", q)
            ctype, pname = " ".join(mm.group(1).split()).replace(" *", "*"), mm.group(2)
            params.append((ctype, pname))
        out.append((ret, m.group(2), params))
    return out


# double* parameters that are host memory (everything else double*/float* is a device array)
HOST_DOUBLE = {("ht3d_reduce", "out"), ("ht3d_ctx_inner_timing", "ms"), ("ht3d_Nusselt", "Nu"),
               ("ht3d_breakpoint_read", "time"), ("ht3d_breakpoint_read", "dt"), ("ht3d_write_vtr", "x"),
               ("ht3d_write_vtr", "y"), ("ht3d_write_vtr", "z")}
STRUCTS = {"ht3d_dyrel_params": "DyrelParams", "ht3d_dyrel_stats": "DyrelStats", "ht3d_hrl_params": "HrlParams",
           "ht3d_v18_params": "V18Params", "ht3d_khaled_geom": "KhaledGeom", "ht3d_post_params": "PostParams",
           "ht3d_post_fields": "PostFields", "ht3d_instance": "Instance"}


def julia_type(fn, ctype, pname):
    """Julia ccall type of one C parameter."""
    base = ctype.replace("const ", "").strip()
    if base == "ht3d_ctx*":
        return "Ptr{Cvoid}"
    if base == "ht3d_ctx**":
        return "Ref{Ptr{Cvoid}}"
    if base == "ht3d_instance*":
        return "Ptr{Instance}"
    for c, j in STRUCTS.items():
        if base == c + "*":
            return f"Ref{{{j}}}"
    if base == "double*":
        if (fn, pname) in HOST_DOUBLE or pname == "bc_val6":
            return "Ptr{Cdouble}"
        return "CuPtr{Cdouble}"
    if base == "float*":
        return "CuPtr{Cfloat}"
    if base == "int*":
        return "Ptr{Cint}"
    if base == "unsigned long long*":
        return "Ptr{Culonglong}"
    if base == "void*":
        return "Ptr{Cvoid}"
    if base == "char*":
        return "Cstring"
    if base == "char* const*":
        return "Ptr{Cstring}"
    if base == "double* const*":
        return "Ptr{Ptr{Cdouble}}"
    return {"double": "Cdouble", "int": "Cint", "long long": "Clonglong",
            "unsigned long long": "Culonglong"}[base]


def julia_ret(ret):
    return {"int": "Cint", "const char*": "Cstring", "unsigned long long": "Culonglong", "double": "Cdouble"}[ret]


# ----------------------------------------------------------------- structs (from abi.py)
def struct_defs():
    from hydrothermal3d_gb300 import abi

    def jt(t):
        if t is ctypes.c_double:
            return "Cdouble"
        if t is ctypes.c_int:
            return "Cint"
        if t is ctypes.c_void_p:
            return "CuPtr{Cdouble}"
        if isinstance(t, type) and issubclass(t, ctypes.Array):
            return f"NTuple{{{t._length_}, {jt(t._type_)}}}"
        if isinstance(t, type) and issubclass(t, ctypes._Pointer):
            return f"Ptr{{{t._type_.__name__}}}"
        if isinstance(t, type) and issubclass(t, ctypes.Structure):
            return t.__name__
        raise TypeError(t)

    order = ["DyrelParams", "DyrelStats", "HrlParams", "V18Params", "KhaledGeom", "PostParams", "PostFields",
             "Instance"]
    cname = {v: k for k, v in STRUCTS.items()}
    out = []
    for name in order:
        cls = getattr(abi, name)
        out.append(f"# {cname[name]} (include/ht3d.h)")
        out.append(f"Base.@kwdef struct {name}")
        for f, t in cls._fields_:
            j = jt(t)
            if j == "Cdouble":
                d = "0.0"
            elif j == "Cint":
                d = "Cint(0)"
            elif j.startswith("NTuple"):
                d = f"ntuple(_ -> {'Cint(0)' if 'Cint' in j.split(',')[-1] else '0.0'}, {t._length_})"
                if "NTuple" in j[7:]:
                    d = f"ntuple(_ -> ntuple(_ -> 0.0, {t._type_._length_}), {t._length_})"
            elif j.startswith("Ptr"):
                d = f"{j}(C_NULL)"
            elif j.startswith("CuPtr"):
                d = f"{j}(0)"
            else:
                d = f"{j}()"
            out.append(f"    {f}::{j} = {d}")
        out.append("end")
        out.append("")
    return "\n".join(out)


# ----------------------------------------------------------------- staggering (from api.py)
SHAPE = {"c": "(nx, ny, nz)", "ex": "(nx + 2, ny + 2, nz + 2)", "fx": "(nx + 1, ny, nz)", "fy": "(nx, ny + 1, nz)",
         "fz": "(nx, ny, nz + 1)", "v": "(nx + 1, ny + 1, nz + 1)", "xxx": "(nx + 6, ny + 6, nz + 6)",
         "wN": "(nx + 2, nz + 2)"}


def api_shapes():
    """{c_name: {param: staggering key}} from api.py's _ptr(name, S["key"]) calls."""
    tree = ast.parse(open(API).read())
    res = {}
    for node in ast.walk(tree):
        if not (isinstance(node, ast.Call) and isinstance(node.func, ast.Attribute) and node.func.attr == "call"):
            continue
        if not node.args or not isinstance(node.args[0], ast.Constant):
            continue
        cname = node.args[0].value
        m = res.setdefault(cname, {})
        for a in node.args[1:]:
            if isinstance(a, ast.Call) and getattr(a.func, "id", "") == "_ptr" and len(a.args) >= 2:
                nm = a.args[0]
                sh = a.args[1]
                if isinstance(nm, ast.Name) and isinstance(sh, ast.Subscript) and isinstance(sh.slice, ast.Constant):
                    m[nm.id] = sh.slice.value
                elif isinstance(nm, ast.Name) and isinstance(sh, ast.Tuple):
                    m[nm.id] = "wN"
    return res


# ----------------------------------------------------------------- drop-in wrappers
# (julia name, C entry point, grid (array, staggering) or ("n", array), fixed C args,
#  argument renames C -> reference, keyword args, reference citation)
GRID_N = "n"
K = [
    # Dimensionless/kernels_HT3D.jl, Dimensionless/HydroThermal3D_Alban_v6.jl, tools/Macros.jl
    ("Init_vel!", "ht3d_Init_vel", ("Pc_ex", "ex"), {}, "Dimensionless/kernels_HT3D.jl:73-80"),
    ("InitDarcy!", "ht3d_InitDarcy", ("Tc_ex", "ex"), {}, "Dimensionless/kernels_HT3D.jl:82-90"),
    ("Compute_Rp!", "ht3d_Compute_Rp", ("Rp", "c"), {}, "Dimensionless/kernels_HT3D.jl:92-97"),
    ("InitThermal!", "ht3d_InitThermal", ("Tc_ex", "ex"), {}, "Dimensionless/kernels_HT3D.jl:99-107"),
    ("ComputeFlux!", "ht3d_ComputeFlux", ("A", "ex"), {},
     "Dimensionless/kernels_HT3D.jl:109-117, Dimensional/kernels_HT3D_dimensional.jl:140-146"),
    ("UpdateT!", "ht3d_UpdateT", ("F", "c"), {}, "Dimensionless/kernels_HT3D.jl:119-126"),
    ("ResidualDiffusion!", "ht3d_ResidualDiffusion", ("F", "c"), {}, "Dimensionless/kernels_HT3D.jl:128-134"),
    ("ResidualDiffusionTransient!", "ht3d_ResidualDiffusionTransient", ("F", "c"), {},
     "Dimensionless/HydroThermal3D_Alban_v6.jl:84-90"),
    ("UpdateP!", "ht3d_UpdateP", ("F", "c"), {}, "Dimensionless/kernels_HT3D.jl:136-142"),
    ("DampedUpdate!", "ht3d_UpdateP", ("F", "c"), {}, "Dimensional/kernels_HT3D_dimensional.jl:316-320"),
    ("DYRELUpdate!", "ht3d_DYRELUpdate", ("F", "c"), {}, "Dimensional/kernels_HT3D_dimensional.jl:322-326"),
    ("SetPressureBCs!", "ht3d_SetPressureBCs", ("Pc_ex", "ex"), {}, "Dimensionless/kernels_HT3D.jl:144-154"),
    ("SetFaceBCs!", "ht3d_SetFaceBCs", ("X_ex", "ex"), {},
     "the face rules of Dimensionless/HydroThermal3D_Alban_v6.jl:108-130 (faces W,E,S,N,B,F)"),
    ("KillNorthSouthFluxes!", "ht3d_KillNorthSouthFluxes", ("Ty", "fy"), {},
     "Dimensionless/HydroThermal3D_Alban_v6.jl:153-159"),
    ("ResetA!", "ht3d_ResetA", (GRID_N, "A"), {}, "tools/Macros.jl:171-177"),
    ("Cpy_inn_to_all!", "ht3d_Cpy_inn_to_all", ("A", "c"), {}, "tools/Macros.jl:187-192"),
    ("Cpy_all_to_inn!", "ht3d_Cpy_all_to_inn", ("B", "c"), {}, "tools/Macros.jl:194-199"),
    ("ArrayEqualArray!", "ht3d_ArrayEqualArray", (GRID_N, "A"), {}, "tools/Weno5_Routines.jl:271-276"),
    # Dimensional/kernels_HT3D_dimensional.jl
    ("Multiply", "ht3d_Multiply", (GRID_N, "a"), {}, "Dimensional/kernels_HT3D_dimensional.jl:106-109"),
    ("InitThermal!", "ht3d_Cpy_inn_to_all", ("A", "c"), {}, "Dimensional/kernels_HT3D_dimensional.jl:128-131"),
    ("InitDarcy!", "ht3d_ArrayEqualArray", (GRID_N, "A"), {}, "Dimensional/kernels_HT3D_dimensional.jl:261-264"),
    ("GershgorinPoisson!", "ht3d_GershgorinPoisson", ("G", "c"), {}, "Dimensional/kernels_HT3D_dimensional.jl:207-221"),
    ("GershgorinHydro!", "ht3d_GershgorinHydro", ("G", "c"), {}, "Dimensional/kernels_HT3D_dimensional.jl:335-347"),
    ("SwapDYREL!", "ht3d_SwapDYREL", ("Xc", "c"), {}, "Dimensional/kernels_HT3D_dimensional.jl:122-126"),
    ("RayleighQuotientNumerator!", "ht3d_RayleighQuotientNumerator", (GRID_N, "G"), {},
     "Dimensional/kernels_HT3D_dimensional.jl:349-355"),
    ("RayleighQuotientDenominator!", "ht3d_RayleighQuotientDenominator", (GRID_N, "G"), {},
     "Dimensional/kernels_HT3D_dimensional.jl:357-363"),
    ("ComputeThermalConductivity", "ht3d_ComputeThermalConductivity", ("ktv", "v"), {},
     "Dimensional/kernels_HT3D_dimensional.jl:40-50"),
    ("ComputeHydroConductivity", "ht3d_ComputeHydroConductivity", ("kfv", "v"), {},
     "Dimensional/kernels_HT3D_dimensional.jl:52-86"),
    ("ComputeFluidDensity", "ht3d_ComputeFluidDensity", ("rhofv", "v"), {},
     "Dimensional/kernels_HT3D_dimensional.jl:88-104"),
    ("SmoothConductivityV2C", "ht3d_SmoothConductivityV2C", ("ktc", "c"), {},
     "Dimensional/kernels_HT3D_dimensional.jl:111-114"),
    ("SmoothConductivityC2V", "ht3d_SmoothConductivityC2V", ("ktc", "c"), {},
     "Dimensional/kernels_HT3D_dimensional.jl:116-119"),
    ("InitConductivity!", "ht3d_InitConductivity", ("ktv", "v"), {}, "Dimensional/kernels_HT3D_dimensional.jl:133-138"),
    ("ComputeρCeffective!", "ht3d_ComputeRhoCeffective", ("rhoC_eff", "c"), {},
     "Dimensional/kernels_HT3D_dimensional.jl:148-160"),
    ("ResidualTemperatureLinearised!", "ht3d_ResidualTemperatureLinearised", ("F", "c"), {},
     "Dimensional/kernels_HT3D_dimensional.jl:162-181"),
    ("SetTemperatureBCs!", "ht3d_SetTemperatureBCs", ("Tc_ex", "ex"), {},
     "Dimensional/kernels_HT3D_dimensional.jl:183-205"),
    ("SetPressureBCs!", "ht3d_SetPressureBCs_dim", ("Pc_ex", "ex"), {},
     "Dimensional/kernels_HT3D_dimensional.jl:291-314"),
    ("ϕρf", "ht3d_PhiRhof", ("phirhofc", "c"), {}, "Dimensional/kernels_HT3D_dimensional.jl:225-235"),
    ("ϕρf_old", "ht3d_PhiRhofOld", ("phirhofc", "c"), {}, "Dimensional/kernels_HT3D_dimensional.jl:237-247"),
    ("ϕdρdP!", "ht3d_PhiDrhodP", ("phidrhodP", "c"), {}, "Dimensional/kernels_HT3D_dimensional.jl:249-259"),
    ("ComputeDarcyFlux!", "ht3d_ComputeDarcyFlux", ("Pf", "ex"), {}, "Dimensional/kernels_HT3D_dimensional.jl:266-272"),
    ("ResidualFluidPressure!", "ht3d_ResidualFluidPressure", ("F", "c"), {},
     "Dimensional/kernels_HT3D_dimensional.jl:274-289"),
    ("Init_vel!", "ht3d_Init_vel_dim", ("rhofv", "v"), {}, "Dimensional/kernels_HT3D_dimensional.jl:328-333"),
    # tools/Weno5_Routines.jl (v1)
    ("VxPlusMinus!", "ht3d_VPlusMinus", ("Vm", "c"), {"axis": "0"}, "tools/Weno5_Routines.jl:5-16"),
    ("VyPlusMinus!", "ht3d_VPlusMinus", ("Vm", "c"), {"axis": "1"}, "tools/Weno5_Routines.jl:18-29"),
    ("VzPlusMinus!", "ht3d_VPlusMinus", ("Vm", "c"), {"axis": "2"}, "tools/Weno5_Routines.jl:31-42"),
    ("dFdx_Weno5!", "ht3d_dFdx_Weno5", (GRID_N, "dFdxi"), {}, "tools/Weno5_Routines.jl:44-68"),
    ("Gradients_minus_x_Weno5!", "ht3d_Gradients_Weno5", ("v1", "c"), {"axis": "0", "sign": "-1"},
     "tools/Weno5_Routines.jl:70-78"),
    ("Gradients_plus_x_Weno5!", "ht3d_Gradients_Weno5", ("v1", "c"), {"axis": "0", "sign": "1"},
     "tools/Weno5_Routines.jl:80-88"),
    ("Gradients_minus_y_Weno5!", "ht3d_Gradients_Weno5", ("v1", "c"), {"axis": "1", "sign": "-1"},
     "tools/Weno5_Routines.jl:90-98"),
    ("Gradients_plus_y_Weno5!", "ht3d_Gradients_Weno5", ("v1", "c"), {"axis": "1", "sign": "1"},
     "tools/Weno5_Routines.jl:100-108"),
    ("Gradients_minus_z_Weno5!", "ht3d_Gradients_Weno5", ("v1", "c"), {"axis": "2", "sign": "-1"},
     "tools/Weno5_Routines.jl:110-118"),
    ("Gradients_plus_z_Weno5!", "ht3d_Gradients_Weno5", ("v1", "c"), {"axis": "2", "sign": "1"},
     "tools/Weno5_Routines.jl:120-128"),
    # v1 (Fc n^3) and v2 (Fc ghosted, tools/Weno5_Routines_v2.jl:221-347) told apart by Fc's shape
    ("Boundaries_x_Weno5!", "ht3d_Boundaries_Weno5", ("Fc_exxx", "xxx"),
     {"axis": "0", "fc_ghosted": "Cint(size(Fc) == (nx + 2, ny + 2, nz + 2))"},
     "tools/Weno5_Routines.jl:130-170, tools/Weno5_Routines_v2.jl:221-262"),
    ("Boundaries_y_Weno5!", "ht3d_Boundaries_Weno5", ("Fc_exxx", "xxx"),
     {"axis": "1", "fc_ghosted": "Cint(size(Fc) == (nx + 2, ny + 2, nz + 2))"},
     "tools/Weno5_Routines.jl:172-212, tools/Weno5_Routines_v2.jl:264-304"),
    ("Boundaries_z_Weno5!", "ht3d_Boundaries_Weno5", ("Fc_exxx", "xxx"),
     {"axis": "2", "fc_ghosted": "Cint(size(Fc) == (nx + 2, ny + 2, nz + 2))"},
     "tools/Weno5_Routines.jl:214-255, tools/Weno5_Routines_v2.jl:306-347"),
    ("Advect!", "ht3d_Advect_v1", (GRID_N, "Fc"), {}, "tools/Weno5_Routines.jl:257-262"),
    # the reference numbers the v2 axes 1, 2, 3; the C entry point 0, 1, 2
    ("Advect!", "ht3d_Advect_v2", ("Fc_ex", "ex"), {"axis": "Cint(axis - 1)", "quirk": "Cint(quirk)"},
     "tools/Weno5_Routines_v2.jl:55-212"),
    # Dimensional/kernels_HT3D_postprocessing.jl
    ("Phase!", "ht3d_Phase", ("X", "c"), {}, "Dimensional/kernels_HT3D_postprocessing.jl:1-10"),
    ("Pressure!", "ht3d_Pressure", ("X", "c"), {}, "Dimensional/kernels_HT3D_postprocessing.jl:12-21"),
    ("Temperature!", "ht3d_Temperature", ("X", "c"), {}, "Dimensional/kernels_HT3D_postprocessing.jl:23-32"),
    ("Velocity!", "ht3d_Velocity", ("X", "c"), {}, "Dimensional/kernels_HT3D_postprocessing.jl:34-45"),
    ("EffectiveThermalConductivity!", "ht3d_EffectiveThermalConductivity", ("X", "c"), {},
     "Dimensional/kernels_HT3D_postprocessing.jl:47-57"),
    ("EffectiveHeatCapacity!", "ht3d_EffectiveHeatCapacity", ("Ceff", "c"), {},
     "Dimensional/kernels_HT3D_postprocessing.jl:60-70"),
    ("Permeability!", "ht3d_Permeability", ("X", "c"), {}, "Dimensional/kernels_HT3D_postprocessing.jl:72-85"),
    ("FluidDensity!", "ht3d_FluidDensity", ("X", "c"), {}, "Dimensional/kernels_HT3D_postprocessing.jl:87-98"),
    ("Viscosity!", "ht3d_Viscosity", ("X", "c"), {}, "Dimensional/kernels_HT3D_postprocessing.jl:100-109"),
    ("Peclet!", "ht3d_Peclet", ("X", "c"), {}, "Dimensional/kernels_HT3D_postprocessing.jl:111-129"),
]
# optional trailing arguments of the drop-ins (not in the reference's signature)
KEYWORDS = {"ht3d_ComputeHydroConductivity": ("kmul_v", "CU_NULL"), "ht3d_Advect_v2": ("quirk", "1")}
GRID_PARAMS = ("nx", "ny", "nz")


def grid_line(grid):
    arr, kind = grid
    if arr == GRID_N:
        return None
    off = {"c": "0", "ex": "2", "v": "1", "xxx": "6", "fy": "(0, 1, 0)"}[kind]
    return f"    nx, ny, nz = size({arr}) .- {off}"


def dropin(jname, cname, grid, fixed, cite, protos, shapes):
    ret, name, params = protos[cname]
    ref_args, call_args = [], []
    kw = KEYWORDS.get(cname)
    for ctype, p in params:
        if ctype.replace("const ", "") == "ht3d_ctx*":
            call_args.append("ctx.ptr")
        elif p in GRID_PARAMS:
            call_args.append(p)
        elif p == "n" and grid[0] == GRID_N:
            call_args.append(f"length({grid[1]})")
        elif p in fixed:
            call_args.append(fixed[p])
            if p == "axis" and "axis - 1" in fixed[p]:
                ref_args.append("axis")
        elif kw and p == kw[0]:
            call_args.append(p)
        else:
            ref_args.append(p)
            call_args.append(p)
    sig = ", ".join(ref_args)
    kws = ["ctx::Context = context()"]
    if kw:
        kws.insert(0, f"{kw[0]} = {kw[1]}")
    lines = [f'"""', f"    {jname}({sig})", "", f"`@parallel {jname}(...)` of {cite}, on the GPU through `{cname}`.",
             f'"""', f"function {jname}({sig}; {', '.join(kws)})"]
    g = grid_line(grid)
    if g:
        lines.append(g)
    sh = shapes.get(cname, {})
    if g:
        for ctype, p in params:
            if p in sh and p in ref_args and sh[p] in SHAPE:
                lines.append(f'    _shape({p}, {SHAPE[sh[p]]}, "{p}")')
    lines.append(f"    _check(ctx, C.{cname}({', '.join(call_args)}))")
    lines.append("    return nothing")
    lines.append("end")
    return "\n".join(lines)


# fused entry points: (julia name, C name, grid array, staggering, returns)
FUSED = [
    ("dyrel_solve_dimless!", "ht3d_dyrel_solve_dimless", "X_ex", "ex", ["stats"]),
    ("dyrel_iterate!", "ht3d_dyrel_iterate", "X_ex", "ex", []),
    ("dyrel_thermal_iterate!", "ht3d_dyrel_thermal_iterate", "T_ex", "ex", []),
    ("dyrel_darcy_iterate!", "ht3d_dyrel_darcy_iterate", "P_ex", "ex", []),
    ("dyrel_iterate_f32!", "ht3d_dyrel_iterate_f32", "X_ex", "ex", []),
    ("weno5_advect!", "ht3d_weno5_advect", "Tc_ex", "ex", []),
    ("weno5_advect_f32!", "ht3d_weno5_advect_f32", "Tc_ex", "ex", []),
    ("step_hrl!", "ht3d_step_hrl", "Tc_ex", "ex", ["st_thermal", "st_darcy"]),
    ("step_v18!", "ht3d_step_v18", "Tc_ex", "ex", ["st_thermal", "st_darcy"]),
    ("postprocess_fields!", "ht3d_postprocess_fields", "Tc_ex", "ex", []),
    ("SetInitialConditions_Khaled!", "ht3d_SetInitialConditions_Khaled", "Tc_ex", "ex", []),
    ("Nusselt", "ht3d_Nusselt", "qy", "fy", ["Nu"]),
    ("breakpoint_write", "ht3d_breakpoint_write", "Tc_ex", "ex", []),
    ("breakpoint_read!", "ht3d_breakpoint_read", "Tc_ex", "ex", ["time", "dt"]),
    ("breakpoint_write_h5", "ht3d_breakpoint_write_h5", "Tc_ex", "ex", []),
    ("breakpoint_read_h5!", "ht3d_breakpoint_read_h5", "Tc_ex", "ex", ["time", "dt"]),
]
OUT_TYPES = {"stats": "DyrelStats", "st_thermal": "DyrelStats", "st_darcy": "DyrelStats", "Nu": "Cdouble",
             "time": "Cdouble", "dt": "Cdouble"}


def fused(jname, cname, arr, kind, outs, protos):
    ret, name, params = protos[cname]
    sig, call_args, pre = [], [], []
    for ctype, p in params:
        t = julia_type(cname, ctype, p)
        if t == "Ptr{Cvoid}" and p == "ctx":
            call_args.append("ctx.ptr")
        elif p in GRID_PARAMS:
            call_args.append(p)
        elif p in outs:
            pre.append(f"    {p} = Ref{{{OUT_TYPES[p]}}}()")
            call_args.append(p)
        elif t == "Ptr{Cint}":  # six-face BC types
            sig.append(p)
            call_args.append(f"Cint[{p}...]")
        elif t == "Ptr{Cdouble}" and p.startswith("bc_val"):
            sig.append(p)
            call_args.append(f"Cdouble[{p}...]")
        else:
            sig.append(p)
            call_args.append(p)
    off = {"ex": "2", "fy": "(0, 1, 0)"}[kind]
    lines = ['"""', f"    {jname}({', '.join(sig)})", "",
             f"`{cname}` (include/ht3d.h){'; returns ' + ', '.join(outs) if outs else ''}.", '"""',
             f"function {jname}({', '.join(sig)}; ctx::Context = context())",
             f"    nx, ny, nz = size({arr}) .- {off}"]
    lines += pre
    lines.append(f"    _check(ctx, C.{cname}({', '.join(call_args)}))")
    if outs:
        lines.append(f"    return {', '.join(o + '[]' for o in outs)}")
    else:
        lines.append("    return nothing")
    lines.append("end")
    return "\n".join(lines)


def header_constants():
    out = []
    with open(HEADER) as f:
        for line in f:
            m = re.match(r"#define (HT3D_[A-Z0-9_]+) (-?\d+)", line)
            if m and m.group(1) != "HT3D_H":
                out.append(f"const {m.group(1)[5:]} = Cint({m.group(2)})")
    return "\n".join(out)


def generate():
    protos_list = parse_header()
    protos = {name: (ret, name, params) for ret, name, params in protos_list}
    shapes = api_shapes()
    low = []
    for ret, name, params in protos_list:
        args = ", ".join(p for _, p in params)
        types = ", ".join(julia_type(name, c, p) for c, p in params)
        tup = f"({types},)" if len(params) == 1 else f"({types})"
        low.append(f"{name}({args}) =\n    ccall((:{name}, libht3d), {julia_ret(ret)}, {tup}{', ' if args else ''}{args})")
    drop = [dropin(*k, protos, shapes) for k in K]
    fus = [fused(*f, protos) for f in FUSED]
    return TEMPLATE.format(constants=header_constants(), structs=struct_defs(), low="\n".join(low),
                           dropins="\n\n".join(drop), fused="\n\n".join(fus))


TEMPLATE = '''# Generated by julia/generate.py from include/ht3d.h: do not edit.
#
# Julia binding of libht3d.so, the GB300 implementation of HydroThermal3D's
# pseudo-transient kernels.  A driver replaces `@parallel Kernel!(args...)` by
# `HT3D.Kernel!(args...)` with the same arguments (CuArray{{Float64,3}} in the
# reference's staggering); grid sizes are inferred from the array shapes, a
# wrong shape throws ArgumentError, a non-zero status Ht3dError.  Every call
# runs on the stream of its Context (by default one created on CUDA.jl's task
# stream) and returns after the kernel finished, like @parallel.
module HT3D

using CUDA

const libht3d = get(ENV, "HT3D_LIB", joinpath(@__DIR__, "..", "hydrothermal3d_gb300", "libht3d.so"))
const CU_NULL = CuPtr{{Cdouble}}(0)

# ---------------------------------------------------------------- constants
{constants}

# ---------------------------------------------------------------- structs
{structs}
# ---------------------------------------------------------------- C entry points (one per prototype)
module C
using CUDA
import ..HT3D: libht3d, DyrelParams, DyrelStats, HrlParams, V18Params, KhaledGeom, PostParams, PostFields, Instance

{low}

end  # module C

# ---------------------------------------------------------------- context and errors
struct Ht3dError <: Exception
    status::Cint
    msg::String
end
Base.showerror(io::IO, e::Ht3dError) = print(io, "libht3d status ", e.status, " (", e.msg, ")")

mutable struct Context
    ptr::Ptr{{Cvoid}}
end

"""
    Context(; device = 0, stream = CUDA.stream())

One libht3d context: its CUDA stream and scratch memory.  Destroyed by the GC.
"""
function Context(; device::Integer = 0, stream = CUDA.stream())
    r = Ref{{Ptr{{Cvoid}}}}(C_NULL)
    st = C.ht3d_ctx_create(r, Cint(device), Ptr{{Cvoid}}(stream.handle))
    st == OK || throw(Ht3dError(st, unsafe_string(C.ht3d_status_string(st))))
    ctx = Context(r[])
    finalizer(ctx) do c
        c.ptr == C_NULL || C.ht3d_ctx_destroy(c.ptr)
        c.ptr = C_NULL
    end
    return ctx
end

const _default = Ref{{Union{{Nothing, Context}}}}(nothing)
"""The default context (created on first use on CUDA.jl's current stream)."""
context() = (_default[] === nothing && (_default[] = Context()); _default[])

function _check(ctx::Context, st::Cint)
    st == OK && return nothing
    msg = unsafe_string(C.ht3d_status_string(st))
    detail = unsafe_string(C.ht3d_ctx_last_error(ctx.ptr))
    throw(Ht3dError(st, isempty(detail) ? msg : msg * ": " * detail))
end

function _shape(a, dims, name)
    size(a) == dims || throw(ArgumentError("$name: shape $(size(a)) does not match the staggering $dims"))
    return nothing
end

function __init__()
    C.ht3d_abi_version() == ABI_VERSION || error("libht3d ABI version mismatch")
    for (T, n) in ((DyrelParams, C.ht3d_sizeof_dyrel_params()), (DyrelStats, C.ht3d_sizeof_dyrel_stats()),
                   (HrlParams, C.ht3d_sizeof_hrl_params()), (V18Params, C.ht3d_sizeof_v18_params()),
                   (Instance, C.ht3d_sizeof_instance()), (PostParams, C.ht3d_sizeof_post_params()),
                   (PostFields, C.ht3d_sizeof_post_fields()))
        sizeof(T) == n || error("libht3d struct size mismatch: $T")
    end
end

"""DYREL controls with the reference's values (Dimensional/HydroThermal3D_v18.jl:292-303, 433-439)."""
reference_dyrel(; tol = 1e-8, nitmax = 10000, nitout = 1000, norm_scale = 1.0) =
    DyrelParams(tol_abs = tol, tol_rel = tol, nitmax = Cint(nitmax), nitout = Cint(nitout), cfl = 0.99,
                cfact = 0.5, lmin_ratio = 500.0, norm_scale = norm_scale)

# ---------------------------------------------------------------- drop-in kernels
{dropins}

"""
    TimeAveraging!(Fc, Fold, order)

`@parallel TimeAveraging!(...)`: tools/Weno5_Routines.jl:264-269 (Fc and Fold of
one shape) or tools/Weno5_Routines_v2.jl:214-219 (Fc ghosted, Fold n^3).
"""
function TimeAveraging!(Fc, Fold, order; ctx::Context = context())
    if size(Fc) == size(Fold)
        _check(ctx, C.ht3d_TimeAveraging_v1(ctx.ptr, Fc, Fold, order, length(Fc)))
    else
        nx, ny, nz = size(Fold)
        _shape(Fc, (nx + 2, ny + 2, nz + 2), "Fc")
        _check(ctx, C.ht3d_TimeAveraging_v2(ctx.ptr, Fc, Fold, order, nx, ny, nz))
    end
    return nothing
end

"""
    maximum_g(A), minimum_g(A), sum_g(A), mean_g(A), mean_abs_g(A)

tools/Macros.jl:20-25 and mean_g(abs.(F)) (Dimensional/HydroThermal3D_v18.jl:460):
reductions in the library's canonical tree order, result on the host.
"""
function _reduce(A, op; ctx::Context = context())
    out = Ref{{Cdouble}}(0.0)
    _check(ctx, C.ht3d_reduce(ctx.ptr, A, length(A), Cint(op), out))
    return out[]
end
sum_g(A; kw...) = _reduce(A, 0; kw...)
maximum_g(A; kw...) = _reduce(A, 2; kw...)
minimum_g(A; kw...) = _reduce(A, 3; kw...)
mean_g(A; kw...) = sum_g(A; kw...) / length(A)
mean_abs_g(A; kw...) = _reduce(A, 1; kw...) / length(A)

# ---------------------------------------------------------------- fused entry points
{fused}

"""
    ensemble_step!(members::Vector{{Instance}}, precision)

One time step of every member (`ht3d_ensemble_step`); returns the members' statuses.
"""
function ensemble_step!(members::Vector{{Instance}}, precision; ctx::Context = context())
    st = GC.@preserve members C.ht3d_ensemble_step(ctx.ptr, pointer(members), Cint(length(members)), Cint(precision))
    st == OK || st == ERR_NAN || st == ERR_DIVERGED || _check(ctx, st)
    return [m.status for m in members]
end

end  # module HT3D
'''

if __name__ == "__main__":
    with open(OUT, "w") as f:
        f.write(generate())
    print(OUT)
