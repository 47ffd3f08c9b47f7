/*
 * ht3d.h -- C ABI of libht3d.so, a GB300 (sm_103a) CUDA implementation of the
 * pseudo-transient hot path of HydroThermal3D (tduretz/HydroThermal3D).
 *
 * Each `ht3d_<Kernel>` entry point replaces one ParallelStencil call
 * `@parallel Kernel!(args...)` of the reference, with the same argument order;
 * the reference file:line of every replaced kernel is cited beside it.
 *
 * Conventions
 *   - Arrays are caller-owned DEVICE pointers to FP64 data laid out exactly
 *     like the reference's Data.Array: 3-D, column-major (x fastest), with the
 *     reference's staggering. nx, ny, nz are numbers of cells:
 *       cell   : nx   x ny   x nz        ghosted "ex" : (nx+2)x(ny+2)x(nz+2)
 *       x-face : (nx+1) x ny x nz        y-face : nx x (ny+1) x nz
 *       z-face : nx x ny x (nz+1)        vertex : (nx+1)x(ny+1)x(nz+1)
 *       WENO "exxx" : (nx+6)x(ny+6)x(nz+6)   wN : (nx+2)x(nz+2)
 *     Phase fields are FP64 codes {-1,0,1,2,3} as in the reference.
 *   - Scalars are passed by value, in the reference's order.
 *   - Every call returns an int status (HT3D_OK = 0). Nothing aborts or traps.
 *   - One ctx = one CUDA stream = one host thread. By default every call is
 *     synchronous (like @parallel); ht3d_ctx_set_sync(ctx, 0) makes the
 *     per-kernel calls asynchronous on the ctx stream.
 *   - The ctx owns only scratch memory (reduction partials, ping-pong and
 *     FP32 shadow buffers); it never frees or reallocates caller buffers.
 */
#ifndef HT3D_H
#define HT3D_H

#ifdef __cplusplus
extern "C" {
#endif

#define HT3D_ABI_VERSION 1

/* status codes */
#define HT3D_OK 0
#define HT3D_ERR_ARG 1         /* bad dimensions / null pointer / bad option */
#define HT3D_ERR_CUDA 2        /* CUDA runtime error (see ht3d_ctx_last_error) */
#define HT3D_ERR_NAN 3         /* residual became NaN (reference: error("Nan T...")) */
#define HT3D_ERR_DIVERGED 4    /* nF_rel > 100 (reference: error("Diverged T...")) */
#define HT3D_ERR_MAXITER 5     /* reserved: the reference does not error at nitmax */
#define HT3D_ERR_TIMEOUT 6     /* a bounded device wait gave up */
#define HT3D_ERR_NOMEM 7
#define HT3D_ERR_SCRATCH 8     /* grid larger than the static scratch of ht3d_dyrel_iterate_noalloc */
#define HT3D_ERR_IO 9          /* a file could not be opened, written or read */

/* precision forms */
#define HT3D_FP64 0            /* plain FP64, reproduces the reference */
#define HT3D_MIXED 1           /* FP32 storage/stencils + FP64 norms, defect correction, T accumulation */

/* face boundary-condition types (tools/Weno5_Routines.jl:134-168) */
#define HT3D_BC_NEUMANN 0
#define HT3D_BC_DIRICHLET 1
#define HT3D_BC_PERIODIC 2

/* WENO5 variants */
#define HT3D_WENO_V1 0         /* tools/Weno5_Routines.jl (unfused reference, textbook stencil) */
#define HT3D_WENO_V2_REF 1     /* tools/Weno5_Routines_v2.jl incl. its minus-branch v5 stencil */
#define HT3D_WENO_V2_FIXED 2   /* v2 loop structure with the textbook v5 stencil */

/* tuning keys for ht3d_ctx_set_tuning */
#define HT3D_TUNE_DYREL_VARIANT 1   /* thread layout of the fused DYREL iteration:   */
#define HT3D_DYREL_AUTO 0           /*   per precision: z-march FP64, per-cell FP32  */
#define HT3D_DYREL_ZMARCH 1         /*   32x8 column tiles marching in z              */
#define HT3D_DYREL_CELL 2           /*   one thread per cell                          */
#define HT3D_TUNE_MIXED_REFRESH 2   /* mixed form: FP64 defect-correction refresh every N
                                       inner iterations between checks (default 512; 0 = only
                                       at the reference's check iterations)             */
#define HT3D_TUNE_TIME_INNER 3      /* 1: the mixed solver brackets every run of consecutive
                                       FP32 inner-iteration launches with CUDA events on the
                                       ctx stream (read back by ht3d_ctx_inner_timing)    */
#define HT3D_TUNE_ENS_BLOCK 4       /* threads per block of the batched ensemble iteration
                                       with one plane per thread: 64/128/256 fixes it, 0
                                       leaves the tile shape to HT3D_TUNE_ENS_TILE        */
#define HT3D_TUNE_ENS_GRAPH 5       /* 1 (default): replay windows of 16 batched inner
                                       iterations as CUDA graphs; 0: launch one by one    */
#define HT3D_TUNE_TEMPORAL 6        /* mixed form: 0 = one FP32 inner iteration per launch;
                                       1 (default) = two per pass through memory (temporal
                                       blocking, TMA-staged planes, z-chunk chosen per grid)
                                       on grids of >= 2^21 cells whose x extent fills 128-cell
                                       tiles to >= 3/4, one per launch otherwise; >= 2 = two
                                       per pass on every grid, that many planes per chunk;
                                       bit-identical results (255^3: 59.6 against 75.8 us
                                       per iteration)                                    */
#define HT3D_TUNE_ENS_TILE 8        /* tile shape of the batched ensemble iteration: 0 =
                                       autotune on first use of an ensemble shape over
                                       six shapes, or 1..6 fixed: threads per block x planes
                                       per thread = 64x1, 128x1, 256x1, 64x8 (z-march),
                                       128x8, 128x16; overrides HT3D_TUNE_ENS_BLOCK;
                                       bit-identical results                             */
#define HT3D_TUNE_WAIT_TEST 7       /* test hook of the bounded waits: v > 0 makes the next
                                       two-iteration pass (HT3D_TUNE_TEMPORAL) skip the
                                       copies of plane v - 1 and give up after 4096 polls;
                                       the solve returns HT3D_ERR_TIMEOUT and the context
                                       stays usable.  Reset after that pass.             */

typedef struct ht3d_ctx ht3d_ctx;

/* DYREL controls (Dimensional/HydroThermal3D_v18.jl:433-439, 292-303) */
typedef struct ht3d_dyrel_params {
    double tol_abs;     /* stop when nF_abs < tol_abs ...            (tolT / tolP)  */
    double tol_rel;     /* ... or nF_rel < tol_rel                                  */
    int nitmax;         /* maximum pseudo-iterations                 (nitmax = 1e4) */
    int nitout;         /* check cadence: iter % nitout == 0 || iter <= 2 (1000)   */
    double cfl;         /* CFL_T / CFL_P                              (0.99)        */
    double cfact;       /* damping factor                             (0.5)         */
    double lmin_ratio;  /* initial lambda_min = lambda_max / lmin_ratio (500)       */
    double norm_scale;  /* nF_abs multiplier (sc.rho*sc.C*sc.T/sc.t, 1 if dimensionless) */
} ht3d_dyrel_params;

typedef struct ht3d_dyrel_stats {
    int iters;          /* pseudo-iterations performed */
    int converged;      /* 1 if the stop test fired */
    int status;         /* HT3D_OK / HT3D_ERR_NAN / HT3D_ERR_DIVERGED */
    int checks;         /* number of check iterations */
    double nF_abs, nF_rel, nF_ini;
    double lambda_min, lambda_max, h1, h2, dtau;
} ht3d_dyrel_stats;

/* Dimensionless Horton-Rogers-Lapwood time step (see ht3d_step_hrl). */
typedef struct ht3d_hrl_params {
    double Ra, dx, dy, dz;
    double dt;                 /* in: this step's dt; out: next dt when dt_adapt */
    double Tbot, Ttop;
    int thermal_bc[6]; double thermal_val[6];   /* faces W,E,S,N,B,F */
    int darcy_bc[6];   double darcy_val[6];
    int weno_bc[6];    double weno_val[6];
    int weno_variant;          /* HT3D_WENO_* */
    int kill_ns;               /* KillNorthSouthFluxes! (Alban_v6.jl:153-159) */
    int dt_adapt;              /* dt = dt_fact/6.1*min(dx,dy,dz)/max|V| (v7.jl:220) */
    int advection;
    double dt_fact;
    ht3d_dyrel_params thermal, darcy;
    double dt_max;             /* > 0: upper bound of the adapted dt; 0 = the reference's
                                  rule, which has none */
} ht3d_hrl_params;

/* Dimensional time step (see ht3d_step_v18); values in the reference's scaled
   units (Dimensional/HydroThermal3D_v18.jl:135-312). */
typedef struct ht3d_v18_params {
    double dx, dy, dz, ymin;
    double dt;                 /* in: dt; out: dt_adv when dt_constant == 0 */
    double time;               /* in/out: model time, advanced by dt when it > 0 */
    double phi_i, k_fact, delta, g, Qt, qyS;
    double Ttop, Tbot, Ptop, Pbot, T_pluton;
    double C_adv;              /* advection multiplier (v18 "C"): dt_adv = C/6.1*min(dx,dy,dz)/max|V| */
    double sc_T, sc_L, sc_t, sc_eta, sc_sigma, sc_rho, sc_C, sc_kt;   /* scaling (scale_me!) */
    int it;                    /* time-step index: 0 = steady initialisation (transient = 0); 1 inserts the pluton */
    int thermal, hydro, advection, dt_constant;
    int weno_variant;          /* HT3D_WENO_V2_REF reproduces AdvectWithWeno5_v2 */
    ht3d_dyrel_params thermal_dyrel, darcy_dyrel;   /* norm_scale: sc.rho*sc.C*sc.T/sc.t and sc.rho/sc.t */
    int n_adv;                 /* out: advection sub-steps taken */
    int pad_;
} ht3d_v18_params;

/* ------------------------------------------------------------------ */
/* library / context                                                   */
/* ------------------------------------------------------------------ */
int ht3d_abi_version(void);
const char* ht3d_status_string(int status);
/* stream: a cudaStream_t (NULL creates a private non-blocking stream) */
int ht3d_ctx_create(ht3d_ctx** out, int device, void* stream);
int ht3d_ctx_destroy(ht3d_ctx* ctx);
int ht3d_ctx_set_stream(ht3d_ctx* ctx, void* stream);
int ht3d_ctx_set_sync(ht3d_ctx* ctx, int sync_each_call);
int ht3d_ctx_synchronize(ht3d_ctx* ctx);
/* set a tuning knob (HT3D_TUNE_*); results never depend on it */
int ht3d_ctx_set_tuning(ht3d_ctx* ctx, int key, int value);
/* number of CUDA kernels this ctx has launched (monotonic) */
unsigned long long ht3d_ctx_launch_count(const ht3d_ctx* ctx);
/* device time (ms) and inner-iteration count of the mixed solver's timed
   inner-iteration runs since the last reset (HT3D_TUNE_TIME_INNER); reset != 0
   clears them */
int ht3d_ctx_inner_timing(ht3d_ctx* ctx, double* ms, unsigned long long* launches, int reset);
const char* ht3d_ctx_last_error(const ht3d_ctx* ctx);
/* sizes of the parameter structs, for binding checks */
int ht3d_sizeof_dyrel_params(void);
int ht3d_sizeof_dyrel_stats(void);
int ht3d_sizeof_hrl_params(void);
int ht3d_sizeof_instance(void);
int ht3d_sizeof_v18_params(void);

/* ------------------------------------------------------------------ */
/* Reductions (tools/Macros.jl:20-25: maximum_g, minimum_g, mean_g,    */
/* sum_g; and mean_g(abs.(F)) at Dimensional/HydroThermal3D_v18.jl:460)*/
/* op: 0 sum, 1 sum|.|, 2 max, 3 min, 4 max|.| ; result to *out (host) */
/* ------------------------------------------------------------------ */
int ht3d_reduce(ht3d_ctx* ctx, const double* a, long long n, int op, double* out);

/* ------------------------------------------------------------------ */
/* Dimensionless kernels (Dimensionless/kernels_HT3D.jl,               */
/* Dimensionless/HydroThermal3D_Alban_v6.jl, tools/Macros.jl)          */
/* ------------------------------------------------------------------ */
/* Init_vel!            Dimensionless/kernels_HT3D.jl:73-80 */
int ht3d_Init_vel(ht3d_ctx* ctx, double* Vx, double* Vy, double* Vz, const double* kx, const double* ky,
                  const double* kz, const double* Pc_ex, const double* Ty, double Ra, double _dx, double _dy,
                  double _dz, int nx, int ny, int nz);
/* InitDarcy!           Dimensionless/kernels_HT3D.jl:82-90 */
int ht3d_InitDarcy(ht3d_ctx* ctx, double* Ty, double* kx, double* ky, double* kz, const double* Tc_ex,
                   const double* kfv, double _dt, int nx, int ny, int nz);
/* Compute_Rp!          Dimensionless/kernels_HT3D.jl:92-97 */
int ht3d_Compute_Rp(ht3d_ctx* ctx, double* Rp, const double* ky, const double* Ty, double Ra, double _dy,
                    int nx, int ny, int nz);
/* InitThermal!         Dimensionless/kernels_HT3D.jl:99-107 */
int ht3d_InitThermal(ht3d_ctx* ctx, double* Rt, double* kx, double* ky, double* kz, const double* Tc_ex,
                     const double* ktv, double _dt, int nx, int ny, int nz);
/* ComputeFlux!         Dimensionless/kernels_HT3D.jl:109-117, Dimensional/kernels_HT3D_dimensional.jl:140-146 */
int ht3d_ComputeFlux(ht3d_ctx* ctx, double* qx, double* qy, double* qz, const double* kx, const double* ky,
                     const double* kz, const double* A, double _dx, double _dy, double _dz, int nx, int ny, int nz);
/* UpdateT!             Dimensionless/kernels_HT3D.jl:119-126 */
int ht3d_UpdateT(ht3d_ctx* ctx, double* F, double* T, const double* R, const double* qx, const double* qy,
                 const double* qz, double _dt, double dtau, double _dx, double _dy, double _dz, int nx, int ny, int nz);
/* ResidualDiffusion!   Dimensionless/kernels_HT3D.jl:128-134 */
int ht3d_ResidualDiffusion(ht3d_ctx* ctx, double* F, const double* R, const double* qx, const double* qy,
                           const double* qz, double _dx, double _dy, double _dz, int nx, int ny, int nz);
/* ResidualDiffusionTransient!  Dimensionless/HydroThermal3D_Alban_v6.jl:84-90 */
int ht3d_ResidualDiffusionTransient(ht3d_ctx* ctx, double* F, const double* T, const double* R, const double* qx,
                                    const double* qy, const double* qz, double _dt, double _dx, double _dy,
                                    double _dz, int nx, int ny, int nz);
/* UpdateP!             Dimensionless/kernels_HT3D.jl:136-142
   (== DampedUpdate!    Dimensional/kernels_HT3D_dimensional.jl:316-320) */
int ht3d_UpdateP(ht3d_ctx* ctx, double* F0, double* P, const double* F, double dampx, double dtau,
                 int nx, int ny, int nz);
/* DYRELUpdate!         Dimensional/kernels_HT3D_dimensional.jl:322-326 */
int ht3d_DYRELUpdate(ht3d_ctx* ctx, double* F0, double* X, const double* F, double h1, double h2, double dtau,
                     int nx, int ny, int nz);
/* SetPressureBCs!      Dimensionless/kernels_HT3D.jl:144-154 (x,z Neumann; y Dirichlet Pbot/Ptop) */
int ht3d_SetPressureBCs(ht3d_ctx* ctx, double* Pc_ex, double Pbot, double Ptop, int nx, int ny, int nz);
/* Generic six-face ghost BCs covering SetPressureBCs!/SetTemperatureBCs! of
   Dimensionless/HydroThermal3D_Alban_v6.jl:108-130. type/val: W,E,S,N,B,F.
   Face ghosts are exact; edge and corner ghosts are not written. */
int ht3d_SetFaceBCs(ht3d_ctx* ctx, double* X_ex, const int* bc_type6, const double* bc_val6, int nx, int ny, int nz);
/* KillNorthSouthFluxes!  Dimensionless/HydroThermal3D_Alban_v6.jl:153-159 */
int ht3d_KillNorthSouthFluxes(ht3d_ctx* ctx, double* Ty, int nx, int ny, int nz);
/* ResetA!              tools/Macros.jl:171-177 (two arrays of n elements) */
int ht3d_ResetA(ht3d_ctx* ctx, double* A, double* B, long long n);
/* Cpy_inn_to_all!      tools/Macros.jl:187-192  A(n^3) = inn(B) */
int ht3d_Cpy_inn_to_all(ht3d_ctx* ctx, double* A, const double* B_ex, int nx, int ny, int nz);
/* Cpy_all_to_inn!      tools/Macros.jl:194-199  inn(A) = B(n^3) */
int ht3d_Cpy_all_to_inn(ht3d_ctx* ctx, double* A_ex, const double* B, int nx, int ny, int nz);
/* ArrayEqualArray!     tools/Weno5_Routines.jl:271-276 */
int ht3d_ArrayEqualArray(ht3d_ctx* ctx, double* A, const double* B, long long n);
/* Multiply             Dimensional/kernels_HT3D_dimensional.jl:106-109 */
int ht3d_Multiply(ht3d_ctx* ctx, double* a, const double* b, const double* c, long long n);

/* ------------------------------------------------------------------ */
/* DYREL support kernels (Dimensional/kernels_HT3D_dimensional.jl)     */
/* ------------------------------------------------------------------ */
/* GershgorinPoisson!   :207-221 (G <- Gershgorin bound / diagonal, D <- diagonal) */
int ht3d_GershgorinPoisson(ht3d_ctx* ctx, double* G, double* D, const double* rhoC_eff, const double* kx,
                           const double* ky, const double* kz, double transient, double dt, double dx, double dy,
                           double dz, int nx, int ny, int nz);
/* GershgorinHydro!     :335-347 */
int ht3d_GershgorinHydro(ht3d_ctx* ctx, double* G, const double* phidrhodP, const double* kx, const double* ky,
                         const double* kz, double transient, double dt, double dx, double dy, double dz,
                         int nx, int ny, int nz);
/* SwapDYREL!           :122-126 */
int ht3d_SwapDYREL(ht3d_ctx* ctx, double* Xc, double* Yc, const double* X0c_ex, const double* Y0c,
                   int nx, int ny, int nz);
/* RayleighQuotientNumerator!   :349-355 */
int ht3d_RayleighQuotientNumerator(ht3d_ctx* ctx, double* G, const double* Fc0, const double* Fcit,
                                   const double* Fc, double dtau, long long n);
/* RayleighQuotientDenominator! :357-363 */
int ht3d_RayleighQuotientDenominator(ht3d_ctx* ctx, double* G, const double* Fc0, double dtau, long long n);

/* ------------------------------------------------------------------ */
/* Dimensional kernels (Dimensional/kernels_HT3D_dimensional.jl) and   */
/* material laws (Dimensional/HydroThermal3D_v18.jl:29-39).            */
/* Boundary kernels use snapshot semantics: every rule reads the other */
/* cells as they were before the call (the reference races there).     */
/* ------------------------------------------------------------------ */
/* ComputeThermalConductivity   :40-50 (ktv at vertices) */
int ht3d_ComputeThermalConductivity(ht3d_ctx* ctx, double* ktv, const double* Tce, const double* phv, double phi0,
                                    double scale_kt, double scale_T, int nx, int ny, int nz);
/* ComputeHydroConductivity     :52-86 (mode 1 rho*k/mu, 2 k/mu, 3 k).  kmul_v (vertex
   field, may be NULL) multiplies the permeability law kF(y) for heterogeneous
   permeability; NULL is the reference kernel. */
int ht3d_ComputeHydroConductivity(ht3d_ctx* ctx, double* kfv, const double* Tce, const double* Pce, const double* phv,
                                  double ymin, double dy, double k_fact, double delta, double scale_sigma,
                                  double scale_T, double scale_L, double scale_t, double scale_eta, int mode,
                                  const double* kmul_v, int nx, int ny, int nz);
/* ComputeFluidDensity          :88-104 */
int ht3d_ComputeFluidDensity(ht3d_ctx* ctx, double* rhofv, const double* Tce, const double* Pce, const double* phv,
                             double scale_sigma, double scale_T, double scale_rho, int nx, int ny, int nz);
/* SmoothConductivityV2C        :111-114 */
int ht3d_SmoothConductivityV2C(ht3d_ctx* ctx, double* ktc, const double* ktv, int nx, int ny, int nz);
/* SmoothConductivityC2V        :116-119 */
int ht3d_SmoothConductivityC2V(ht3d_ctx* ctx, double* ktv, const double* ktc, int nx, int ny, int nz);
/* InitConductivity!            :133-138 */
int ht3d_InitConductivity(ht3d_ctx* ctx, double* kx, double* ky, double* kz, const double* ktv, int nx, int ny, int nz);
/* ComputeρCeffective!          :148-160 */
int ht3d_ComputeRhoCeffective(ht3d_ctx* ctx, double* rhoC_eff, const double* Tc_ex, const double* Pc_ex,
                              const double* phc_ex, double phi_i, double sca_T, double sca_sigma, double sca_C,
                              double sca_rho, int nx, int ny, int nz);
/* ResidualTemperatureLinearised!  :162-181 */
int ht3d_ResidualTemperatureLinearised(ht3d_ctx* ctx, double* F, const double* Tc_ex, const double* Tc_old,
                                       const double* rhoC_eff, const double* phc_ex, const double* PC,
                                       const double* qx, const double* qy, const double* qz, double Qt,
                                       double transient, double _dt, double _dx, double _dy, double _dz, int nx,
                                       int ny, int nz);
/* SetTemperatureBCs! (dimensional)  :183-205; the reference's unused arguments are kept */
int ht3d_SetTemperatureBCs(ht3d_ctx* ctx, double* Tc_ex, const double* ky, const double* wN, const double* phc_ex,
                           double qyS, double _dy, double kS, double TS, double TN, double y_plateau, double a2,
                           double b2, double dTdy, double dx, double dy, int sticky_air, double sca_T, double sca_kT,
                           double phi_i, int nx, int ny, int nz);
/* SetPressureBCs! (dimensional)     :291-314 */
int ht3d_SetPressureBCs_dim(ht3d_ctx* ctx, double* Pc_ex, const double* wN, const double* phc_ex, double PS,
                            double PN, double y_plateau, double a2, double b2, double rhof, double g, double dx,
                            double dy, int sticky_air, int nx, int ny, int nz);
/* ϕρf                          :225-235 */
int ht3d_PhiRhof(ht3d_ctx* ctx, double* phirhofc, const double* Tc_ex, const double* Pc_ex, const double* phc_ex,
                 double phi_i, double scale_rho, double scale_T, double scale_sigma, int nx, int ny, int nz);
/* ϕρf_old                      :237-247 */
int ht3d_PhiRhofOld(ht3d_ctx* ctx, double* phirhofc, const double* Tc0, const double* Pc0, const double* phc_ex,
                    double phi_i, double scale_rho, double scale_T, double scale_sigma, int nx, int ny, int nz);
/* ϕdρdP!                       :249-259 */
int ht3d_PhiDrhodP(ht3d_ctx* ctx, double* phidrhodP, const double* Tc_ex, const double* Pc_ex, const double* phc_ex,
                   double phi_i, double scale_rho, double scale_T, double scale_sigma, int nx, int ny, int nz);
/* ComputeDarcyFlux!            :266-272 */
int ht3d_ComputeDarcyFlux(ht3d_ctx* ctx, double* qx, double* qy, double* qz, const double* rhofv, const double* kx,
                          const double* ky, const double* kz, const double* Pf, double g, double _dx, double _dy,
                          double _dz, int nx, int ny, int nz);
/* ResidualFluidPressure!       :274-289 */
int ht3d_ResidualFluidPressure(ht3d_ctx* ctx, double* F, const double* phc_ex, const double* phirhofc,
                               const double* phirhofc0, const double* PC, const double* qx, const double* qy,
                               const double* qz, double transient, double _dt, double _dx, double _dy, double _dz,
                               int nx, int ny, int nz);
/* Init_vel! (dimensional)      :328-333 */
int ht3d_Init_vel_dim(ht3d_ctx* ctx, double* Vx, double* Vy, double* Vz, const double* qx, const double* qy,
                      const double* qz, const double* rhofv, int nx, int ny, int nz);
/* material laws (Dimensional/HydroThermal3D_v18.jl:29-39) evaluated elementwise:
   which 0 kTs(T), 1 kTf(T), 2 Cf(T), 3 Cs(T), 4 ρs(T), 5 ρf_C(T_C,p), 6 dρdP_C(T_C,p),
   7 μf(T), 8 kF(y,δ), 9 ϕ(phase,ϕ0), 10 e^a and 11 10^a (the exponentials μf and kF use:
   one implementation, below 1 ulp, whose bits are the same on every machine);
   b may be NULL for one-argument laws */
int ht3d_material_law(ht3d_ctx* ctx, int which, const double* a, const double* b, double* out, long long n);

/* ------------------------------------------------------------------ */
/* WENO5 advection                                                     */
/* ------------------------------------------------------------------ */
/* V{x,y,z}PlusMinus!   tools/Weno5_Routines.jl:5-42 (axis 0,1,2) */
int ht3d_VPlusMinus(ht3d_ctx* ctx, double* Vm, double* Vp, const double* V, int axis, int nx, int ny, int nz);
/* dFdx_Weno5!          tools/Weno5_Routines.jl:44-68 */
int ht3d_dFdx_Weno5(ht3d_ctx* ctx, double* dFdxi, const double* V1, const double* V2, const double* V3,
                    const double* V4, const double* V5, long long n);
/* Gradients_{minus,plus}_{x,y,z}_Weno5!  tools/Weno5_Routines.jl:70-128 (sign -1 minus, +1 plus) */
int ht3d_Gradients_Weno5(ht3d_ctx* ctx, double* v1, double* v2, double* v3, double* v4, double* v5,
                         const double* Fc_exxx, int axis, int sign, double _dx, double _dy, double _dz,
                         int nx, int ny, int nz);
/* Boundaries_{x,y,z}_Weno5!  v1 tools/Weno5_Routines.jl:130-255 (Fc is n^3, fc_ghosted = 0),
                              v2 tools/Weno5_Routines_v2.jl:221-347 (Fc is ex, fc_ghosted = 1) */
int ht3d_Boundaries_Weno5(ht3d_ctx* ctx, double* Fc_exxx, const double* Fc, int axis, int type_L, double val_L,
                          int type_R, double val_R, int fc_ghosted, int nx, int ny, int nz);
/* Advect! v1           tools/Weno5_Routines.jl:257-262 */
int ht3d_Advect_v1(ht3d_ctx* ctx, double* Fc, const double* Vxp, const double* dTdxm, const double* Vxm,
                   const double* dTdxp, double dt, long long n);
/* TimeAveraging! v1    tools/Weno5_Routines.jl:264-269 */
int ht3d_TimeAveraging_v1(ht3d_ctx* ctx, double* Fc, const double* Fold, double order, long long n);
/* Advect! v2           tools/Weno5_Routines_v2.jl:55-212 (quirk 1 = reference v5 stencil) */
int ht3d_Advect_v2(ht3d_ctx* ctx, double* Fc_ex, const double* X_exxx, const double* V, int axis, double dt,
                   double _dx, double _dy, double _dz, int quirk, int nx, int ny, int nz);
/* TimeAveraging! v2    tools/Weno5_Routines_v2.jl:214-219 */
int ht3d_TimeAveraging_v2(ht3d_ctx* ctx, double* Fc_ex, const double* Fold, double order, int nx, int ny, int nz);

/* Fused advection: one SSP-RK2 (Heun) sweep per axis x, y, z, ghost cells
   computed on the fly (no exxx buffer).  Replaces AdvectWithWeno5
   (Dimensionless/kernels_HT3D.jl:156-233, minus its Init_vel! call) for
   HT3D_WENO_V1 and AdvectWithWeno5_v2 (tools/Weno5_Routines_v2.jl:1-50) for
   HT3D_WENO_V2_*.  bc_type6/bc_val6: W,E,S,N,B,F.  Needs n >= 3 per axis. */
int ht3d_weno5_advect(ht3d_ctx* ctx, double* Tc_ex, const double* Vx, const double* Vy, const double* Vz, double dt,
                      double _dx, double _dy, double _dz, const int* bc_type6, const double* bc_val6, int variant,
                      int precision, int nx, int ny, int nz);

/* FP32 storage and arithmetic variant of ht3d_weno5_advect (float fields of the
   same shapes); the weights' epsilon floor is 1e-18 instead of the reference's
   1e-99, which underflows in FP32.  For the standalone large-grid sweep. */
int ht3d_weno5_advect_f32(ht3d_ctx* ctx, float* Tc_ex, const float* Vx, const float* Vy, const float* Vz, double dt,
                          double _dx, double _dy, double _dz, const int* bc_type6, const double* bc_val6, int variant,
                          int nx, int ny, int nz);

/* ------------------------------------------------------------------ */
/* Fused DYREL solver (replaces the loop Dimensional/HydroThermal3D_v18.jl:448-477
   composed with the dimensionless residuals):
     F = (R + cX*inn(X) + div q(X)) / PC,  q = -k grad X,
   cX = _dt gives ResidualDiffusionTransient! (Alban_v6.jl:84-90), cX = 0
   gives ResidualDiffusion! (kernels_HT3D.jl:128-134); PC is the diagonal of
   GershgorinPoisson! with rhoC = 1.  Face BCs as ht3d_SetFaceBCs.
   On return X holds the solution (inner cells + face ghosts as the reference
   leaves them), F the last residual and F0 the DYREL momentum (both n^3).
   n_iter_fixed > 0 runs exactly that many iterations with no stop test. */
int ht3d_dyrel_solve_dimless(ht3d_ctx* ctx, double* X_ex, const double* R, const double* kx, const double* ky,
                             const double* kz, double cX, double dx, double dy, double dz, const int* bc_type6,
                             const double* bc_val6, const ht3d_dyrel_params* prm, int n_iter_fixed, double* F,
                             double* F0, int precision, ht3d_dyrel_stats* stats, int nx, int ny, int nz);

/* n_iter plain pseudo-iterations of the fused DYREL kernel with fixed
   (h1, h2, dtau) and no checks -- the inner loop of ht3d_dyrel_solve_dimless
   (Dimensional/HydroThermal3D_v18.jl:451-455 without the check block), for
   callers that run their own schedule.  The FP64 form takes PC (n^3) and
   divides by it like the reference (F /= PC); the _f32 variant takes FP32
   fields and invPC = 1/PC, which it multiplies. */
int ht3d_dyrel_iterate(ht3d_ctx* ctx, double* X_ex, const double* R, const double* kx, const double* ky,
                       const double* kz, const double* PC, double* F0, double cX, double dx, double dy, double dz,
                       const int* bc_type6, const double* bc_val6, double h1, double h2, double dtau, int n_iter,
                       int nx, int ny, int nz);
/* The same iteration for the two dimensionless problems by name: the thermal
   one (ResidualDiffusionTransient!, cX = _dt, Dimensionless/HydroThermal3D_Alban_v6.jl:84-90)
   and the Darcy one (ResidualDiffusion!, cX = 0, Dimensionless/kernels_HT3D.jl:128-134). */
int ht3d_dyrel_thermal_iterate(ht3d_ctx* ctx, int n_iter, double* T_ex, const double* Rt, const double* kx,
                               const double* ky, const double* kz, const double* PC, double* F0, double _dt,
                               double dx, double dy, double dz, const int* bc_type6, const double* bc_val6, double h1,
                               double h2, double dtau, int nx, int ny, int nz);
int ht3d_dyrel_darcy_iterate(ht3d_ctx* ctx, int n_iter, double* P_ex, const double* Rp, const double* kx,
                             const double* ky, const double* kz, const double* PC, double* F0, double dx, double dy,
                             double dz, const int* bc_type6, const double* bc_val6, double h1, double h2, double dtau,
                             int nx, int ny, int nz);
int ht3d_dyrel_iterate_f32(ht3d_ctx* ctx, float* X_ex, const float* R, const float* kx, const float* ky,
                           const float* kz, const float* invPC, float* F0, double cX, double dx, double dy, double dz,
                           const int* bc_type6, const double* bc_val6, double h1, double h2, double dtau, int n_iter,
                           int nx, int ny, int nz);

/* Allocation-free variant of ht3d_dyrel_iterate, for callers that cannot let
   a library allocate device memory (their allocator owns the device heap, or
   memory management is frozen while they run).  No reference counterpart: the
   reference allocates its arrays with @zeros and never needs this.
   Same arguments as ht3d_dyrel_iterate (PC is the Jacobi diagonal, not its
   inverse) without a ctx, plus the cudaStream_t to launch on; results are
   identical to ht3d_dyrel_iterate's.
   - Scratch: one static device array of 2^20 doubles (8 MiB) in the library,
     present on every device that loads it until the process exits.  Grids with
     (nx+2)(ny+2)(nz+2) > 1048576 are rejected with HT3D_ERR_SCRATCH.
   - Never calls cudaMalloc, cudaFree or any allocating routine.
   - The first call on a device looks up the array's device address with that
     device current; make that first call before any stream capture.  The
     address is kept for the life of the process: after cudaDeviceReset on a
     device, do not call this entry point on that device again.
   - n_iter == 0 checks the arguments and returns HT3D_OK without touching
     the device.
   - A launch that fails returns HT3D_ERR_CUDA; errors left on the thread by
     other launches are neither reported nor cleared.
   - Asynchronous: returns after queueing its kernels on `stream`.
   - All calls share the one array, whose contents persist between calls
     (nothing is read before it is written); calls that overlap on the GPU,
     on any stream, race on it. */
int ht3d_dyrel_iterate_noalloc(double* X_ex, const double* R, const double* kx, const double* ky, const double* kz,
                               const double* PC, double* F0, double cX, double dx, double dy, double dz,
                               const int* bc_type6, const double* bc_val6, double h1, double h2, double dtau,
                               int n_iter, int nx, int ny, int nz, void* stream);

/* One time step of the dimensionless Horton-Rogers-Lapwood model:
   thermal DYREL solve, Darcy DYREL solve, Init_vel!, WENO5 advection and the
   adaptive dt (Dimensionless/HydroThermal3D_Alban_v6.jl:322-464,
   Dimensionless/HydroThermal3D_v7.jl:167-222).  Tc_ex, Pc_ex are updated in
   place; Vx,Vy,Vz receive the Darcy velocity; p->dt is updated when dt_adapt. */
int ht3d_step_hrl(ht3d_ctx* ctx, double* Tc_ex, double* Pc_ex, const double* ktv, const double* kfv, double* Vx,
                  double* Vy, double* Vz, ht3d_hrl_params* p, ht3d_dyrel_stats* st_thermal,
                  ht3d_dyrel_stats* st_darcy, int precision, int nx, int ny, int nz);

/* One member of an ensemble of independent HRL runs (the arguments of one
   ht3d_step_hrl call).  No reference counterpart: the reference runs one
   model per process. */
typedef struct ht3d_instance {
    double* Tc_ex;             /* (nx+2)(ny+2)(nz+2) */
    double* Pc_ex;             /* (nx+2)(ny+2)(nz+2) */
    const double* ktv;         /* vertices (nx+1)(ny+1)(nz+1) */
    const double* kfv;         /* vertices */
    double* Vx;                /* x-faces (nx+1) ny nz */
    double* Vy;                /* y-faces nx (ny+1) nz */
    double* Vz;                /* z-faces nx ny (nz+1) */
    ht3d_hrl_params* params;   /* host; dt updated in place when dt_adapt */
    ht3d_dyrel_stats* st_thermal;  /* host, may be NULL */
    ht3d_dyrel_stats* st_darcy;    /* host, may be NULL */
    int nx, ny, nz;
    int status;                /* out: HT3D_* of this member's step */
} ht3d_instance;

/* One time step of every member: the same result, bit for bit, as calling
   ht3d_step_hrl on each member in turn.  HT3D_MIXED batches the members: the
   thermal solves of all members iterate in lockstep with one launch per
   pseudo-iteration over every member still iterating (windows of them
   replayed as CUDA graphs), then the Darcy solves; each member keeps its own
   DYREL parameters, checks and stop test (members must share nitout and
   nitmax).  HT3D_FP64 steps the members one after another.  A member that
   fails (NaN, divergence) stops with its status; the others go on.  Returns
   the first failing member's status, or HT3D_OK. */
int ht3d_ensemble_step(ht3d_ctx* ctx, ht3d_instance* members, int n_members, int precision);

/* Geometry of the detachment-fault model: the driver's `geometry` NamedTuple
   (Dimensional/HydroThermal3D_v18.jl:236-287), lines y = a x + b. */
typedef struct ht3d_khaled_geom {
    double y_plateau;
    double surf_a1, surf_b1;   /* topography slope */
    double fault[4][6];        /* detachment, fault1, fault2, fault3: a1, b1, a2, b2, a3, b3 */
} ht3d_khaled_geom;

/* SetInitialConditions_Khaled (Dimensional/HydroThermal3D_v18.jl:59-129) on the
   device: phases of the ghosted cells (phc_ex) and vertices (phv) -- crust 0,
   fault wedges 2, rotated pluton 3, air 1 above the topography -- and the
   initial T and P (linear from the topography down to y = -30 km in scaled
   units L, ghost rules and the air override of the reference).  The grid is
   the driver's: cell centres LinRange(xmin - dx/2, xmax + dx/2, nx + 2), vertices
   LinRange(xmin, xmax, nx + 1).  wN is left unchanged, as in the reference (its
   loop looks for phase -1, which the function never assigns).  geom is a host
   pointer. */
int ht3d_SetInitialConditions_Khaled(ht3d_ctx* ctx, double* phc_ex, double* phv, double* wN,
                                     const ht3d_khaled_geom* geom, double* Tc_ex, double* Pc_ex, double Tbot,
                                     double Ttop, double Pbot, double Ptop, double xmin, double ymin, double zmin,
                                     double xmax, double ymax, double zmax, double L, int nx, int ny, int nz);

/* One time step of the dimensional model, Dimensional/HydroThermal3D_v18.jl:404-572:
   pluton insertion at it == 1, thermal DYREL solve (conductivity, smoothing,
   ρC_eff, Gershgorin), Darcy DYREL solve (ρk/μ, ϕ∂ρ/∂P, ϕρf_old, ρf), Darcy
   velocity and WENO5-v2 advection with sub-stepping.  phc_ex (ex) and phv
   (vertices) are phase codes, wN the immersed-surface weights (nx+2, nz+2),
   kmul_v an optional vertex multiplier of kF(y) (NULL = reference law).
   Fused FP64 kernels with the reference's rounding. */
int ht3d_step_v18(ht3d_ctx* ctx, double* Tc_ex, double* Pc_ex, const double* phc_ex, const double* phv,
                  const double* wN, const double* kmul_v, double* Vx, double* Vy, double* Vz, ht3d_v18_params* p,
                  ht3d_dyrel_stats* st_thermal, ht3d_dyrel_stats* st_darcy, int nx, int ny, int nz);

/* ------------------------------------------------------------------ */
/* Output diagnostics (Dimensional/kernels_HT3D_postprocessing.jl) and */
/* the Nusselt number (Dimensionless/HydroThermal3D_Alban_v6.jl:345-348)*/
/* ------------------------------------------------------------------ */
/* Every output is a cell array (nx, ny, nz).  Cells whose phase phc_ex is 1
   (air) get NaN, except the Y/Z outputs of ht3d_Velocity and
   ht3d_EffectiveHeatCapacity, which leave air cells untouched as the
   reference does.  Vx (nx+1,ny,nz), Vy (nx,ny+1,nz), Vz (nx,ny,nz+1). */
/* Phase!                         kernels_HT3D_postprocessing.jl:1-10 */
int ht3d_Phase(ht3d_ctx* ctx, double* X, const double* phc_ex, int nx, int ny, int nz);
/* Pressure!                      :12-21 */
int ht3d_Pressure(ht3d_ctx* ctx, double* X, const double* Pc_ex, const double* phc_ex, double scale_sigma, int nx,
                  int ny, int nz);
/* Temperature!                   :23-32 */
int ht3d_Temperature(ht3d_ctx* ctx, double* X, const double* Tc_ex, const double* phc_ex, double scale_T, int nx,
                     int ny, int nz);
/* Velocity!                      :34-45 */
int ht3d_Velocity(ht3d_ctx* ctx, double* X, double* Y, double* Z, const double* Vx, const double* Vy, const double* Vz,
                  const double* phc_ex, double scale_V, int nx, int ny, int nz);
/* EffectiveThermalConductivity!  :47-57 */
int ht3d_EffectiveThermalConductivity(ht3d_ctx* ctx, double* X, const double* Tc_ex, double phi0,
                                      const double* phc_ex, double scale_T, int nx, int ny, int nz);
/* EffectiveHeatCapacity!         :60-70 (solid Cs(T) only; Pc_ex, phi_i and the
   sigma/C/rho scales are accepted and unused, as in the reference) */
int ht3d_EffectiveHeatCapacity(ht3d_ctx* ctx, double* Ceff, const double* Tc_ex, const double* Pc_ex,
                               const double* phc_ex, double phi_i, double sca_T, double sca_sigma, double sca_C,
                               double sca_rho, int nx, int ny, int nz);
/* Permeability!                  :72-85 */
int ht3d_Permeability(ht3d_ctx* ctx, double* X, double k_fact, double ymin, double dy, const double* phc_ex,
                      double delta, double scale_L, int nx, int ny, int nz);
/* FluidDensity!                  :87-98 */
int ht3d_FluidDensity(ht3d_ctx* ctx, double* X, const double* Tc_ex, const double* Pc_ex, const double* phc_ex,
                      double scale_T, double scale_sigma, int nx, int ny, int nz);
/* Viscosity!                     :100-109 */
int ht3d_Viscosity(ht3d_ctx* ctx, double* X, const double* Tc_ex, const double* phc_ex, double scale_T, int nx,
                   int ny, int nz);
/* Peclet!                        :111-129 */
int ht3d_Peclet(ht3d_ctx* ctx, double* X, const double* Tc_ex, const double* Pc_ex, const double* Vx, const double* Vy,
                const double* Vz, const double* phc_ex, double phi0, double scale_T, double scale_sigma, double scale_V,
                double scale_L, int nx, int ny, int nz);

/* Scales and constants of the diagnostics (the driver's sc.T, sc.σ, sc.V,
   sc.L, ϕi, k_fact, ymin, Δy, δ). */
typedef struct ht3d_post_params {
    double phi0, scale_T, scale_sigma, scale_V, scale_L, k_fact, ymin, dy, delta;
} ht3d_post_params;
/* Output arrays of ht3d_postprocess_fields, named as the driver's VTK fields
   (Dimensional/HydroThermal3D_v18.jl:664-685); NULL skips a field.  vx, vy
   and vz go together. */
typedef struct ht3d_post_fields {
    double *phase, *pressure, *temperature, *vx, *vy, *vz, *k_thermal, *heat_capacity, *permeability, *density,
        *viscosity, *peclet;
} ht3d_post_fields;
/* All requested diagnostics in one pass over the grid (the ten kernels above
   fused: phc_ex, T, P and V are read once).  Each field is bit-identical to
   the single-field entry point's.  out and prm are host pointers. */
int ht3d_postprocess_fields(ht3d_ctx* ctx, const ht3d_post_fields* out, const double* Tc_ex, const double* Pc_ex,
                            const double* Vx, const double* Vy, const double* Vz, const double* phc_ex,
                            const ht3d_post_params* prm, int nx, int ny, int nz);
int ht3d_sizeof_post_params(void);
int ht3d_sizeof_post_fields(void);

/* Nusselt number Nu = sum(qy[:,end,:]) / (Lx*Lz) / (nx*nz)
   (Dimensionless/HydroThermal3D_Alban_v6.jl:345-348); qy is the (nx, ny+1, nz)
   y-flux of ComputeFlux!.  The top-face sum uses the library's canonical tree
   order (deterministic).  Result to *Nu (host). */
int ht3d_Nusselt(ht3d_ctx* ctx, const double* qy, double Lx, double Lz, int nx, int ny, int nz, double* Nu);

/* ------------------------------------------------------------------ */
/* Output and restart files (Dimensional/HydroThermal3D_v18.jl)        */
/* ------------------------------------------------------------------ */
/* VTK rectilinear-grid file of vtk_grid(path, xc, yc, zc) with fields
   vtkfile[name] = array (v18.jl:664-686): x (nx), y (ny), z (nz) are the
   cell-centre coordinates, each field has one value per cell (column-major)
   and 1 or 3 components; data holds ncomp[f] HOST pointers per field, in
   field order (a 3-component field gives its X, Y, Z arrays, interleaved in
   the file like WriteVTK's tuple).  VTK XML, Float64, one appended raw block
   (UInt64 headers, little-endian).  ".vtr" is appended to path unless present.
   Field names: 1-200 bytes, none of " < > & or control characters
   (HT3D_ERR_ARG otherwise).  Host-only: needs no context or GPU.  HT3D_ERR_IO
   if the file cannot be written. */
int ht3d_write_vtr(const char* path, const double* x, const double* y, const double* z, int nx, int ny, int nz,
                   int nfields, const char* const* names, const int* ncomp, const double* const* data);

/* Restart state of v18.jl:579-588 (write) and :384-395 (read): the device
   arrays Tc_ex and Pc_ex ((nx+2)(ny+2)(nz+2) each) and time, dt.  The
   reference writes HDF5 (Breakpoint%05d.h5); this library writes a raw
   binary file: the 8 bytes "HT3DBRK1", int64 nx, ny, nz, float64 time, dt,
   then Tc_ex and Pc_ex as column-major float64, little-endian.  Reading
   checks the magic and the grid (HT3D_ERR_ARG on a different grid,
   HT3D_ERR_IO on a missing, foreign or truncated file). */
int ht3d_breakpoint_write(ht3d_ctx* ctx, const char* path, const double* Tc_ex, const double* Pc_ex, double time,
                          double dt, int nx, int ny, int nz);
int ht3d_breakpoint_read(ht3d_ctx* ctx, const char* path, double* Tc_ex, double* Pc_ex, double* time, double* dt,
                         int nx, int ny, int nz);

/* The same restart state in the reference's own file format: the HDF5 file
   Breakpoint%05d.h5 that v18.jl:579-588 writes with HDF5.jl (datasets Tc_ex and
   Pc_ex, float64, dataspace dimensions (nz+2, ny+2, nx+2) -- the Julia array
   (nx+2, ny+2, nz+2) as HDF5.jl stores it -- and the float64 scalars time and
   dt), so each side can restart from the other's files.  Written and read
   without an HDF5 library, from the public file-format specification:
   superblock version 0, a symbol-table root group, version-1 object headers,
   contiguous storage.  Reading accepts superblock versions 0-1, version-1
   object headers and contiguous or compact datasets; other HDF5 layouts give
   HT3D_ERR_IO, a grid other than nx, ny, nz HT3D_ERR_ARG. */
int ht3d_breakpoint_write_h5(ht3d_ctx* ctx, const char* path, const double* Tc_ex, const double* Pc_ex, double time,
                             double dt, int nx, int ny, int nz);
int ht3d_breakpoint_read_h5(ht3d_ctx* ctx, const char* path, double* Tc_ex, double* Pc_ex, double* time, double* dt,
                            int nx, int ny, int nz);
/* Host-only forms of the two above (HOST arrays, no context or GPU). */
int ht3d_h5_breakpoint_image(const char* path, const double* Tc_ex, const double* Pc_ex, double time, double dt,
                             int nx, int ny, int nz);
int ht3d_h5_breakpoint_parse(const char* path, double* Tc_ex, double* Pc_ex, double* time, double* dt, int nx, int ny,
                             int nz);

#ifdef __cplusplus
}
#endif
#endif /* HT3D_H */
