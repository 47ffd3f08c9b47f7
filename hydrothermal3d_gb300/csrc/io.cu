// Output and restart files of the dimensional driver:
//  * ht3d_write_vtr: the VTK rectilinear-grid file that WriteVTK's
//    vtk_grid(path, xc, yc, zc) + vtkfile[name] = array writes at
//    Dimensional/HydroThermal3D_v18.jl:664-686 (cell-centre coordinates, one
//    point per cell, scalar or 3-component fields), as VTK XML with the arrays
//    in one appended raw block (UInt64 size headers).
//  * ht3d_breakpoint_write / _read: the restart state of
//    Dimensional/HydroThermal3D_v18.jl:384-395 and :579-588 (Tc_ex, Pc_ex,
//    time, dt).  The reference stores it in HDF5; with no HDF5 library to
//    link, the library writes the same four items to a raw binary file
//    (layout in include/ht3d.h) straight from device memory.
// Host code only; it writes little-endian data (x86-64 and AArch64 hosts),
// which the VTK header states.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "ht3d_internal.cuh"

namespace {

struct File {
    FILE* f = nullptr;
    explicit File(const std::string& p, const char* mode) : f(std::fopen(p.c_str(), mode)) {}
    ~File() {
        if (f) std::fclose(f);
    }
};

bool write_all(FILE* f, const void* p, size_t n) { return n == 0 || std::fwrite(p, 1, n, f) == n; }
bool read_all(FILE* f, void* p, size_t n) { return n == 0 || std::fread(p, 1, n, f) == n; }

// a field name is written into an XML attribute: non-empty, at most 200
// bytes, none of the characters that would need escaping
bool valid_name(const char* s) {
    if (!s || !*s || std::strlen(s) > 200) return false;
    for (; *s; ++s)
        if (*s == '"' || *s == '<' || *s == '>' || *s == '&' || (unsigned char)*s < 0x20) return false;
    return true;
}

// breakpoint file: magic, then int64 nx, ny, nz, then double time, dt, then
// Tc_ex and Pc_ex ((nx+2)(ny+2)(nz+2) doubles each, column-major)
const char kBreakMagic[8] = {'H', 'T', '3', 'D', 'B', 'R', 'K', '1'};

}  // namespace

extern "C" {

int ht3d_write_vtr(const char* path, const double* x, const double* y, const double* z, int nx, int ny, int nz,
                   int nfields, const char* const* names, const int* ncomp, const double* const* data) {
    if (!path || !x || !y || !z || nx < 1 || ny < 1 || nz < 1 || nfields < 0) return HT3D_ERR_ARG;
    if (nfields > 0 && (!names || !ncomp || !data)) return HT3D_ERR_ARG;
    int nptr = 0;
    for (int f = 0; f < nfields; ++f) {
        if (!valid_name(names[f]) || (ncomp[f] != 1 && ncomp[f] != 3)) return HT3D_ERR_ARG;
        for (int c = 0; c < ncomp[f]; ++c)
            if (!data[nptr + c]) return HT3D_ERR_ARG;
        nptr += ncomp[f];
    }
    std::string p(path);
    if (p.size() < 4 || p.compare(p.size() - 4, 4, ".vtr") != 0) p += ".vtr";  // vtk_grid appends the extension
    const unsigned long long npts = (unsigned long long)nx * ny * nz;

    // XML header with the offsets of each array in the appended block
    std::string xml;
    char buf[512];
    std::snprintf(buf, sizeof buf,
                  "<?xml version=\"1.0\"?>\n"
                  "<VTKFile type=\"RectilinearGrid\" version=\"1.0\" byte_order=\"LittleEndian\" "
                  "header_type=\"UInt64\">\n"
                  "  <RectilinearGrid WholeExtent=\"0 %d 0 %d 0 %d\">\n"
                  "    <Piece Extent=\"0 %d 0 %d 0 %d\">\n"
                  "      <PointData>\n",
                  nx - 1, ny - 1, nz - 1, nx - 1, ny - 1, nz - 1);
    xml += buf;
    unsigned long long off = 0;
    for (int f = 0; f < nfields; ++f) {
        std::snprintf(buf, sizeof buf,
                      "        <DataArray type=\"Float64\" Name=\"%s\" NumberOfComponents=\"%d\" "
                      "format=\"appended\" offset=\"%llu\"/>\n",
                      names[f], ncomp[f], off);
        xml += buf;
        off += 8 + 8ULL * npts * ncomp[f];
    }
    xml += "      </PointData>\n      <Coordinates>\n";
    const char* cname[3] = {"x", "y", "z"};
    const int cn[3] = {nx, ny, nz};
    for (int a = 0; a < 3; ++a) {
        std::snprintf(buf, sizeof buf,
                      "        <DataArray type=\"Float64\" Name=\"%s\" NumberOfComponents=\"1\" format=\"appended\" "
                      "offset=\"%llu\"/>\n",
                      cname[a], off);
        xml += buf;
        off += 8 + 8ULL * cn[a];
    }
    xml += "      </Coordinates>\n    </Piece>\n  </RectilinearGrid>\n  <AppendedData encoding=\"raw\">\n_";

    File out(p, "wb");
    if (!out.f) return HT3D_ERR_IO;
    if (!write_all(out.f, xml.data(), xml.size())) return HT3D_ERR_IO;
    std::vector<double> inter;
    nptr = 0;
    for (int f = 0; f < nfields; ++f) {
        const unsigned long long bytes = 8ULL * npts * ncomp[f];
        if (!write_all(out.f, &bytes, 8)) return HT3D_ERR_IO;
        if (ncomp[f] == 1) {
            if (!write_all(out.f, data[nptr], (size_t)bytes)) return HT3D_ERR_IO;
        } else {  // components interleaved per point, in chunks
            const unsigned long long chunk = 1ULL << 16;
            inter.resize((size_t)(3 * chunk));
            for (unsigned long long s = 0; s < npts; s += chunk) {
                const unsigned long long m = std::min(chunk, npts - s);
                for (unsigned long long t = 0; t < m; ++t)
                    for (int c = 0; c < 3; ++c) inter[(size_t)(3 * t + c)] = data[nptr + c][s + t];
                if (!write_all(out.f, inter.data(), (size_t)(24 * m))) return HT3D_ERR_IO;
            }
        }
        nptr += ncomp[f];
    }
    const double* cd[3] = {x, y, z};
    for (int a = 0; a < 3; ++a) {
        const unsigned long long bytes = 8ULL * cn[a];
        if (!write_all(out.f, &bytes, 8) || !write_all(out.f, cd[a], (size_t)bytes)) return HT3D_ERR_IO;
    }
    const char* tail = "\n  </AppendedData>\n</VTKFile>\n";
    if (!write_all(out.f, tail, std::strlen(tail))) return HT3D_ERR_IO;
    return std::fflush(out.f) == 0 ? HT3D_OK : HT3D_ERR_IO;
}

int ht3d_breakpoint_write(ht3d_ctx* ctx, const char* path, const double* Tc_ex, const double* Pc_ex, double time,
                          double dt, int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(path, Tc_ex, Pc_ex), "null argument");
        ht3d_check_dims(nx, ny, nz, 1);
        const size_t nex = (size_t)(nx + 2) * (ny + 2) * (nz + 2);
        std::vector<double> h(2 * nex);
        HT3D_CUDA(cudaMemcpyAsync(h.data(), Tc_ex, 8 * nex, cudaMemcpyDeviceToHost, ctx->stream));
        HT3D_CUDA(cudaMemcpyAsync(h.data() + nex, Pc_ex, 8 * nex, cudaMemcpyDeviceToHost, ctx->stream));
        HT3D_CUDA(cudaStreamSynchronize(ctx->stream));
        const long long dims[3] = {nx, ny, nz};
        const double td[2] = {time, dt};
        File out(path, "wb");
        if (!out.f) throw ht3d_error(HT3D_ERR_IO, std::string("cannot open ") + path);
        if (!write_all(out.f, kBreakMagic, 8) || !write_all(out.f, dims, sizeof dims) ||
            !write_all(out.f, td, sizeof td) || !write_all(out.f, h.data(), 16 * nex) || std::fflush(out.f) != 0)
            throw ht3d_error(HT3D_ERR_IO, std::string("write failed: ") + path);
        return HT3D_OK;
    });
}

int ht3d_breakpoint_read(ht3d_ctx* ctx, const char* path, double* Tc_ex, double* Pc_ex, double* time, double* dt,
                         int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(path, Tc_ex, Pc_ex, time, dt), "null argument");
        ht3d_check_dims(nx, ny, nz, 1);
        const size_t nex = (size_t)(nx + 2) * (ny + 2) * (nz + 2);
        File in(path, "rb");
        if (!in.f) throw ht3d_error(HT3D_ERR_IO, std::string("cannot open ") + path);
        char magic[8];
        long long dims[3];
        double td[2];
        if (!read_all(in.f, magic, 8) || std::memcmp(magic, kBreakMagic, 8) != 0)
            throw ht3d_error(HT3D_ERR_IO, std::string("not a breakpoint file: ") + path);
        if (!read_all(in.f, dims, sizeof dims) || !read_all(in.f, td, sizeof td))
            throw ht3d_error(HT3D_ERR_IO, std::string("truncated breakpoint file: ") + path);
        HT3D_REQUIRE(dims[0] == nx && dims[1] == ny && dims[2] == nz, "breakpoint grid differs from nx, ny, nz");
        std::vector<double> h(2 * nex);
        if (!read_all(in.f, h.data(), 16 * nex))
            throw ht3d_error(HT3D_ERR_IO, std::string("truncated breakpoint file: ") + path);
        HT3D_CUDA(cudaMemcpyAsync(Tc_ex, h.data(), 8 * nex, cudaMemcpyHostToDevice, ctx->stream));
        HT3D_CUDA(cudaMemcpyAsync(Pc_ex, h.data() + nex, 8 * nex, cudaMemcpyHostToDevice, ctx->stream));
        HT3D_CUDA(cudaStreamSynchronize(ctx->stream));  // h is released on return
        *time = td[0];
        *dt = td[1];
        return HT3D_OK;
    });
}

}  // extern "C"
