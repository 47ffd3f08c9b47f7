// Output diagnostics (Dimensional/kernels_HT3D_postprocessing.jl) and the
// Nusselt number (Dimensionless/HydroThermal3D_Alban_v6.jl:345-348).
//
// The reference runs one kernel per output field, each re-reading phc_ex and
// T/P/V.  Here one kernel, k_post, computes any subset of the fields in one
// pass: every output whose pointer is non-null is written.  The ten drop-in
// entry points below launch it with a single output, ht3d_postprocess_fields
// with all the outputs a caller asks for.  Compiled with -fmad=false; each
// expression keeps the reference's evaluation order, so a field is the same
// bits whichever entry point produced it.
#include "dyrel_common.cuh"
#include "laws.cuh"

namespace {

struct PostOut {
    double *phase, *P, *T, *Vx, *Vy, *Vz, *keff, *Ceff, *perm, *rhof, *mu, *Pe;
};
struct PostIn {
    const double *phc, *Tc, *Pc, *Vx, *Vy, *Vz;
};

// Air cells (phase 1) get NaN, except Velocity!'s Y/Z components and
// EffectiveHeatCapacity!, which the reference leaves untouched there.
// Permeability! depends on the row j only: kF of the ny cell-centre depths,
// evaluated once per row (an FP64 exponential costs the same warp issue
// slots whatever the number of active lanes)
__global__ void k_perm_rows(double* __restrict__ kf, ht3d_post_params p, int ny) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= ny) return;
    const double y = p.ymin + (double)j * p.dy + p.dy / 2;
    kf[j] = law_kF(y * p.scale_L, p.delta * p.scale_L);
}

// kf_rows: the table of k_perm_rows when o.perm is set
__global__ void k_post(PostOut o, PostIn a, ht3d_post_params p, const double* __restrict__ kf_rows, int nx, int ny,
                       int nz) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= nx || j >= ny) return;
    const long long c = (long long)i + (long long)nx * ((long long)j + (long long)ny * k);
    const long long e = (long long)(i + 1) + (long long)(nx + 2) * ((long long)(j + 1) + (long long)(ny + 2) * (k + 1));
    const double ph = a.phc[e];
    const bool air = ph_eq(ph, 1.0);
    const double nan = __longlong_as_double(0x7ff8000000000000LL);
    if (o.phase) o.phase[c] = air ? nan : ph;
    if (o.P) o.P[c] = air ? nan : a.Pc[e] * p.scale_sigma;
    if (o.T) o.T[c] = air ? nan : a.Tc[e] * p.scale_T;
    // face velocities averaged to the cell centre (Velocity!, Peclet!)
    double vx = 0.0, vy = 0.0, vz = 0.0;
    if (!air && (o.Vx || o.Pe)) {
        const long long fx = (long long)i + (long long)(nx + 1) * ((long long)j + (long long)ny * k);
        const long long fy = (long long)i + (long long)nx * ((long long)j + (long long)(ny + 1) * k);
        const long long fz = c;
        vx = 0.5 * (a.Vx[fx] + a.Vx[fx + 1]) * p.scale_V;
        vy = 0.5 * (a.Vy[fy] + a.Vy[fy + nx]) * p.scale_V;
        vz = 0.5 * (a.Vz[fz] + a.Vz[fz + (long long)nx * ny]) * p.scale_V;
    }
    if (o.Vx) {
        if (air) {
            o.Vx[c] = nan;
        } else {
            o.Vx[c] = vx;
            o.Vy[c] = vy;
            o.Vz[c] = vz;
        }
    }
    if (air) {
        if (o.keff) o.keff[c] = nan;
        if (o.perm) o.perm[c] = nan;
        if (o.rhof) o.rhof[c] = nan;
        if (o.mu) o.mu[c] = nan;
        if (o.Pe) o.Pe[c] = nan;
        return;
    }
    if (o.perm) {
        double v = kf_rows[j];
        if (ph_eq(ph, 2.0)) v *= p.k_fact;
        o.perm[c] = v;
    }
    // every read below is of an input that post_launch checked for the
    // outputs requested: Tc for any T-dependent field, Pc for density/Peclet
    if (!(o.keff || o.Pe || o.Ceff || o.rhof || o.mu)) return;
    const double T = a.Tc[e] * p.scale_T;
    // FluidDensity! and Peclet! evaluate rho_f at the same (T - 273.15, P):
    // once here serves both (the ALU, not HBM, bounds this kernel in FP64)
    const double rho = (o.rhof || o.Pe) ? law_rhof_C(T - 273.15, a.Pc[e] * p.scale_sigma) : 0.0;
    if (o.rhof) o.rhof[c] = rho;
    if (o.keff || o.Pe) {
        const double keff = ((1.0 - law_phi(ph, p.phi0)) * law_kTs(T) + law_phi(ph, p.phi0) * law_kTf(T));
        if (o.keff) o.keff[c] = keff;
        if (o.Pe) {
            const double V = sqrt(vx * vx + vy * vy + vz * vz);
            const double C = law_Cf(T);
            o.Pe[c] = p.scale_L * rho * C * V / keff;
        }
    }
    if (o.Ceff) o.Ceff[c] = law_Cs(T);
    if (o.mu) o.mu[c] = law_muf(T);
}

// top face of qy (nx, ny+1, nz) gathered into a contiguous (nx, nz) array
__global__ void k_top_face(double* __restrict__ face, const double* __restrict__ qy, int nx, int ny, int nz) {
    const long long n = (long long)nx * nz;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const long long i = t % nx, k = t / nx;
        face[t] = qy[i + (long long)nx * ((long long)ny + (long long)(ny + 1) * k)];
    }
}

int post_launch(ht3d_ctx* ctx, const PostOut& o, const PostIn& a, const ht3d_post_params& p, int nx, int ny, int nz) {
    ht3d_check_dims(nx, ny, nz, 1);
    HT3D_REQUIRE(a.phc, "null argument");
    const bool needT = o.T || o.keff || o.Ceff || o.rhof || o.mu || o.Pe;
    const bool needP = o.P || o.rhof || o.Pe;
    const bool needV = o.Vx || o.Vy || o.Vz || o.Pe;
    HT3D_REQUIRE(!needT || a.Tc, "null argument");
    HT3D_REQUIRE(!needP || a.Pc, "null argument");
    HT3D_REQUIRE(!needV || all_nonnull(a.Vx, a.Vy, a.Vz), "null argument");
    HT3D_REQUIRE(!(o.Vx || o.Vy || o.Vz) || all_nonnull(o.Vx, o.Vy, o.Vz), "velocity needs all three outputs");
    double* kf_rows = nullptr;
    if (o.perm) {
        kf_rows = (double*)ht3d_scratch(ctx, SLOT_AUX1, sizeof(double) * ny);
        HT3D_LAUNCH(ctx, k_perm_rows, (ny + 127) / 128, 128, 0, kf_rows, p, ny);
    }
    dim3 b(32, 8, 1), g((nx + 31) / 32, (ny + 7) / 8, nz);
    HT3D_LAUNCH(ctx, k_post, g, b, 0, o, a, p, kf_rows, nx, ny, nz);
    return HT3D_OK;
}

ht3d_post_params post_params() { return ht3d_post_params{}; }

}  // namespace

extern "C" {

int ht3d_sizeof_post_params(void) { return (int)sizeof(ht3d_post_params); }
int ht3d_sizeof_post_fields(void) { return (int)sizeof(ht3d_post_fields); }

int ht3d_Phase(ht3d_ctx* ctx, double* X, const double* phc_ex, int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(X, phc_ex), "null argument");
        PostOut o{};
        o.phase = X;
        return post_launch(ctx, o, PostIn{phc_ex, nullptr, nullptr, nullptr, nullptr, nullptr}, post_params(), nx, ny,
                           nz);
    });
}

int ht3d_Pressure(ht3d_ctx* ctx, double* X, const double* Pc_ex, const double* phc_ex, double scale_sigma, int nx,
                  int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(X, Pc_ex, phc_ex), "null argument");
        PostOut o{};
        o.P = X;
        ht3d_post_params p = post_params();
        p.scale_sigma = scale_sigma;
        return post_launch(ctx, o, PostIn{phc_ex, nullptr, Pc_ex, nullptr, nullptr, nullptr}, p, nx, ny, nz);
    });
}

int ht3d_Temperature(ht3d_ctx* ctx, double* X, const double* Tc_ex, const double* phc_ex, double scale_T, int nx,
                     int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(X, Tc_ex, phc_ex), "null argument");
        PostOut o{};
        o.T = X;
        ht3d_post_params p = post_params();
        p.scale_T = scale_T;
        return post_launch(ctx, o, PostIn{phc_ex, Tc_ex, nullptr, nullptr, nullptr, nullptr}, p, nx, ny, nz);
    });
}

int ht3d_Velocity(ht3d_ctx* ctx, double* X, double* Y, double* Z, const double* Vx, const double* Vy, const double* Vz,
                  const double* phc_ex, double scale_V, int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(X, Y, Z, Vx, Vy, Vz, phc_ex), "null argument");
        PostOut o{};
        o.Vx = X;
        o.Vy = Y;
        o.Vz = Z;
        ht3d_post_params p = post_params();
        p.scale_V = scale_V;
        return post_launch(ctx, o, PostIn{phc_ex, nullptr, nullptr, Vx, Vy, Vz}, p, nx, ny, nz);
    });
}

int ht3d_EffectiveThermalConductivity(ht3d_ctx* ctx, double* X, const double* Tc_ex, double phi0,
                                      const double* phc_ex, double scale_T, int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(X, Tc_ex, phc_ex), "null argument");
        PostOut o{};
        o.keff = X;
        ht3d_post_params p = post_params();
        p.phi0 = phi0;
        p.scale_T = scale_T;
        return post_launch(ctx, o, PostIn{phc_ex, Tc_ex, nullptr, nullptr, nullptr, nullptr}, p, nx, ny, nz);
    });
}

int ht3d_EffectiveHeatCapacity(ht3d_ctx* ctx, double* Ceff, const double* Tc_ex, const double* Pc_ex,
                               const double* phc_ex, double phi_i, double sca_T, double sca_sigma, double sca_C,
                               double sca_rho, int nx, int ny, int nz) {
    (void)Pc_ex, (void)phi_i, (void)sca_sigma, (void)sca_C, (void)sca_rho;
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(Ceff, Tc_ex, phc_ex), "null argument");
        PostOut o{};
        o.Ceff = Ceff;
        ht3d_post_params p = post_params();
        p.scale_T = sca_T;
        return post_launch(ctx, o, PostIn{phc_ex, Tc_ex, nullptr, nullptr, nullptr, nullptr}, p, nx, ny, nz);
    });
}

int ht3d_Permeability(ht3d_ctx* ctx, double* X, double k_fact, double ymin, double dy, const double* phc_ex,
                      double delta, double scale_L, int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(X, phc_ex), "null argument");
        PostOut o{};
        o.perm = X;
        ht3d_post_params p = post_params();
        p.k_fact = k_fact;
        p.ymin = ymin;
        p.dy = dy;
        p.delta = delta;
        p.scale_L = scale_L;
        return post_launch(ctx, o, PostIn{phc_ex, nullptr, nullptr, nullptr, nullptr, nullptr}, p, nx, ny, nz);
    });
}

int ht3d_FluidDensity(ht3d_ctx* ctx, double* X, const double* Tc_ex, const double* Pc_ex, const double* phc_ex,
                      double scale_T, double scale_sigma, int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(X, Tc_ex, Pc_ex, phc_ex), "null argument");
        PostOut o{};
        o.rhof = X;
        ht3d_post_params p = post_params();
        p.scale_T = scale_T;
        p.scale_sigma = scale_sigma;
        return post_launch(ctx, o, PostIn{phc_ex, Tc_ex, Pc_ex, nullptr, nullptr, nullptr}, p, nx, ny, nz);
    });
}

int ht3d_Viscosity(ht3d_ctx* ctx, double* X, const double* Tc_ex, const double* phc_ex, double scale_T, int nx,
                   int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(X, Tc_ex, phc_ex), "null argument");
        PostOut o{};
        o.mu = X;
        ht3d_post_params p = post_params();
        p.scale_T = scale_T;
        return post_launch(ctx, o, PostIn{phc_ex, Tc_ex, nullptr, nullptr, nullptr, nullptr}, p, nx, ny, nz);
    });
}

int ht3d_Peclet(ht3d_ctx* ctx, double* X, const double* Tc_ex, const double* Pc_ex, const double* Vx, const double* Vy,
                const double* Vz, const double* phc_ex, double phi0, double scale_T, double scale_sigma, double scale_V,
                double scale_L, int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(X, Tc_ex, Pc_ex, Vx, Vy, Vz, phc_ex), "null argument");
        PostOut o{};
        o.Pe = X;
        ht3d_post_params p = post_params();
        p.phi0 = phi0;
        p.scale_T = scale_T;
        p.scale_sigma = scale_sigma;
        p.scale_V = scale_V;
        p.scale_L = scale_L;
        return post_launch(ctx, o, PostIn{phc_ex, Tc_ex, Pc_ex, Vx, Vy, Vz}, p, nx, ny, nz);
    });
}

int ht3d_postprocess_fields(ht3d_ctx* ctx, const ht3d_post_fields* out, const double* Tc_ex, const double* Pc_ex,
                            const double* Vx, const double* Vy, const double* Vz, const double* phc_ex,
                            const ht3d_post_params* prm, int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(out, phc_ex, prm), "null argument");
        PostOut o{out->phase, out->pressure, out->temperature, out->vx, out->vy, out->vz, out->k_thermal,
                  out->heat_capacity, out->permeability, out->density, out->viscosity, out->peclet};
        return post_launch(ctx, o, PostIn{phc_ex, Tc_ex, Pc_ex, Vx, Vy, Vz}, *prm, nx, ny, nz);
    });
}

int ht3d_Nusselt(ht3d_ctx* ctx, const double* qy, double Lx, double Lz, int nx, int ny, int nz, double* Nu) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(qy, Nu), "null argument");
        ht3d_check_dims(nx, ny, nz, 1);
        const long long n = (long long)nx * nz;
        long long m = (n + 1023) / 1024;
        double* face = (double*)ht3d_scratch(ctx, SLOT_AUX0, sizeof(double) * (n + 2 * m + 2));
        double* a = face + n;
        double* b = a + m + 1;
        const int blocks = (int)std::min<long long>((n + 255) / 256, (long long)ctx->num_sms * 8);
        HT3D_LAUNCH(ctx, k_top_face, blocks, 256, 0, face, qy, nx, ny, nz);
        HT3D_LAUNCH(ctx, (k_tree_pass<1, false>), (unsigned)m, 1024, 0, face, n, 0LL, a);
        while (m > 1) {
            const long long m2 = (m + 1023) / 1024;
            HT3D_LAUNCH(ctx, (k_tree_pass<1, false>), (unsigned)m2, 1024, 0, a, m, 0LL, b);
            std::swap(a, b);
            m = m2;
        }
        ht3d_fetch_results(ctx, a, 1);
        *Nu = ctx->h_result[0] / (Lx * Lz) / (double)n;
        return HT3D_OK;
    });
}

}  // extern "C"
