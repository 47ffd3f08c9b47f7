// Restart files in the reference's own format: Breakpoint%05d.h5 of
// Dimensional/HydroThermal3D_v18.jl:579-588 (write) and :384-395 (read), an
// HDF5 file holding the datasets Tc_ex and Pc_ex (the ghosted fields, FP64)
// and the scalars time and dt.
//
// No HDF5 library is linked: the file is written and read here from the
// public HDF5 file-format specification, in the layout the HDF5 library
// itself writes with its default ("earliest") format settings, which HDF5.jl
// uses:
//   superblock version 0 (8-byte offsets and lengths), the root group as a
//   symbol table (a version-1 B-tree node of group type, one symbol table
//   node, a local heap with the link names), version-1 object headers, and
//   per dataset a dataspace message (version 1), an IEEE little-endian
//   64-bit float datatype message (version 1) and a contiguous data layout
//   message (version 3) pointing at the raw data.
// A Julia array of size (n1, n2, n3) is stored by HDF5.jl with the dataspace
// dimensions reversed, (n3, n2, n1), and its column-major bytes unchanged;
// this file does the same, so read(file, "Tc_ex") in the reference returns the
// (nx+2, ny+2, nz+2) array.  Scalars are scalar dataspaces.
//
// The reader follows the same structures in general: superblock version 0
// or 1, any depth of group B-tree, symbol table nodes, version-1 object headers
// with continuation blocks, dataspace versions 1 and 2, layout versions 1-3
// (contiguous or compact storage); anything else is refused with HT3D_ERR_IO.
// Host code only, little-endian hosts (x86-64, AArch64).
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "ht3d_internal.cuh"

namespace {

constexpr uint64_t kUndef = ~0ULL;
const unsigned char kSig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};

// ------------------------------------------------------------------ writer
struct Out {
    std::vector<unsigned char> b;
    void u8(unsigned v) { b.push_back((unsigned char)v); }
    void u16(unsigned v) { u8(v & 0xff), u8((v >> 8) & 0xff); }
    void u32(uint32_t v) {
        for (int i = 0; i < 4; ++i) u8((v >> (8 * i)) & 0xff);
    }
    void u64(uint64_t v) {
        for (int i = 0; i < 8; ++i) u8((unsigned)((v >> (8 * i)) & 0xff));
    }
    void raw(const void* p, size_t n) { b.insert(b.end(), (const unsigned char*)p, (const unsigned char*)p + n); }
    void zeros(size_t n) { b.insert(b.end(), n, 0); }
    void pad_to(size_t pos) { zeros(pos - b.size()); }
};

// version-1 object header message: type, data size (a multiple of 8), flags
void msg_header(Out& o, unsigned type, unsigned size) {
    o.u16(type);
    o.u16(size);
    o.u8(0);
    o.zeros(3);
}

// symbol table entry (40 bytes)
void sym_entry(Out& o, uint64_t name_off, uint64_t oh, uint32_t cache, uint64_t s0 = 0, uint64_t s1 = 0) {
    o.u64(name_off);
    o.u64(oh);
    o.u32(cache);
    o.u32(0);
    o.u64(s0);
    o.u64(s1);
}

struct Dataset {
    const char* name;
    int rank;          // 0: scalar
    uint64_t dims[3];  // HDF5 order (slowest first)
    const double* data;
    uint64_t n;        // elements
};

constexpr size_t kSuperblock = 96, kOhPrefix = 16;
constexpr size_t kBtreeNode = 24 + 32 * 8 + 33 * 8;  // group node, K = 16
constexpr size_t kSnod = 8 + 8 * 40;                 // symbol table node, leaf K = 4

size_t oh_size(int rank) { return kOhPrefix + (8 + 8 + 8 * rank) + (8 + 24) + (8 + 24); }

std::vector<unsigned char> h5_image_header(const Dataset* ds, int nds, std::vector<uint64_t>& data_addr) {
    // names in the local heap: "" at 0, then each name NUL-terminated, padded to 8
    std::vector<uint64_t> name_off(nds);
    size_t heap_size = 8;
    for (int d = 0; d < nds; ++d) {
        name_off[d] = heap_size;
        heap_size += (std::strlen(ds[d].name) + 1 + 7) / 8 * 8;
    }
    const size_t root_oh = kSuperblock, heap = root_oh + kOhPrefix + 8 + 16, heap_data = heap + 32;
    const size_t btree = heap_data + heap_size, snod = btree + kBtreeNode;
    std::vector<size_t> oh(nds);
    size_t p = snod + kSnod;
    for (int d = 0; d < nds; ++d) {
        oh[d] = p;
        p += oh_size(ds[d].rank);
    }
    data_addr.resize(nds);
    for (int d = 0; d < nds; ++d) {
        data_addr[d] = p;
        p += 8 * ds[d].n;
    }
    const uint64_t eof = p;

    Out o;
    // superblock, version 0
    o.raw(kSig, 8);
    o.u8(0), o.u8(0), o.u8(0), o.u8(0), o.u8(0), o.u8(8), o.u8(8), o.u8(0);
    o.u16(4), o.u16(16), o.u32(0);
    o.u64(0), o.u64(kUndef), o.u64(eof), o.u64(kUndef);
    sym_entry(o, 0, root_oh, 1, btree, heap);  // root group: cache type 1 holds the B-tree and heap
    // root group object header: one symbol table message
    o.u8(1), o.u8(0), o.u16(1), o.u32(1), o.u32(8 + 16), o.u32(0);
    msg_header(o, 0x0011, 16);
    o.u64(btree), o.u64(heap);
    // local heap (no free block: the HDF5 library's end-of-free-list marker is 1)
    o.raw("HEAP", 4), o.u8(0), o.zeros(3), o.u64(heap_size), o.u64(1), o.u64(heap_data);
    o.zeros(8);
    for (int d = 0; d < nds; ++d) {
        o.pad_to(heap_data + name_off[d]);
        o.raw(ds[d].name, std::strlen(ds[d].name));
    }
    o.pad_to(heap_data + heap_size);
    // symbol table entries sorted by name (byte order, as strcmp)
    std::vector<int> order(nds);
    for (int d = 0; d < nds; ++d) order[d] = d;
    for (int a = 0; a < nds; ++a)
        for (int b = a + 1; b < nds; ++b)
            if (std::strcmp(ds[order[b]].name, ds[order[a]].name) < 0) std::swap(order[a], order[b]);
    // B-tree: one leaf node, one child (the symbol table node); key 0 is the
    // empty name, key 1 the last name of the child
    o.raw("TREE", 4), o.u8(0), o.u8(0), o.u16(1), o.u64(kUndef), o.u64(kUndef);
    o.u64(0), o.u64(snod), o.u64(name_off[order[nds - 1]]);
    o.pad_to(btree + kBtreeNode);
    // symbol table node
    o.raw("SNOD", 4), o.u8(1), o.u8(0), o.u16(nds);
    for (int a = 0; a < nds; ++a) sym_entry(o, name_off[order[a]], oh[order[a]], 0);
    o.pad_to(snod + kSnod);
    // dataset object headers
    for (int d = 0; d < nds; ++d) {
        const int r = ds[d].rank;
        o.u8(1), o.u8(0), o.u16(3), o.u32(1), o.u32((uint32_t)(oh_size(r) - kOhPrefix)), o.u32(0);
        msg_header(o, 0x0001, 8 + 8 * r);  // dataspace, version 1 (rank 0: scalar)
        o.u8(1), o.u8(r), o.u8(0), o.u8(0), o.u32(0);
        for (int a = 0; a < r; ++a) o.u64(ds[d].dims[a]);
        msg_header(o, 0x0003, 24);  // datatype: IEEE 754 binary64, little-endian
        o.u8(0x11), o.u8(0x20), o.u8(63), o.u8(0), o.u32(8);
        o.u16(0), o.u16(64), o.u8(52), o.u8(11), o.u8(0), o.u8(52), o.u32(1023);
        o.zeros(4);
        msg_header(o, 0x0008, 24);  // data layout, version 3, contiguous
        o.u8(3), o.u8(1), o.u64(data_addr[d]), o.u64(8 * ds[d].n);
        o.zeros(6);
    }
    return o.b;
}

// ------------------------------------------------------------------ reader
struct In {
    FILE* f = nullptr;
    uint64_t size = 0;
    ~In() {
        if (f) std::fclose(f);
    }
    bool at(uint64_t addr, void* p, size_t n) const {
        if (addr > size || n > size - addr) return false;
        return std::fseek(f, (long)addr, SEEK_SET) == 0 && std::fread(p, 1, n, f) == n;
    }
    std::vector<unsigned char> block(uint64_t addr, size_t n) const {
        std::vector<unsigned char> v(n);
        if (!at(addr, v.data(), n)) throw ht3d_error(HT3D_ERR_IO, "HDF5 file truncated or inconsistent");
        return v;
    }
};

uint64_t le(const unsigned char* p, int n) {
    uint64_t v = 0;
    for (int i = n - 1; i >= 0; --i) v = (v << 8) | p[i];
    return v;
}

[[noreturn]] void bad(const char* what) { throw ht3d_error(HT3D_ERR_IO, std::string("HDF5: ") + what); }

struct Found {
    int rank = -1;
    uint64_t dims[8] = {};
    bool f64le = false;
    int layout = -1;  // 0 compact, 1 contiguous
    uint64_t addr = kUndef, bytes = 0;
    std::vector<unsigned char> compact;
};

// messages of a version-1 object header (following continuation blocks)
Found read_object(const In& in, uint64_t oh) {
    const auto pre = in.block(oh, 16);
    if (pre[0] != 1) bad("only version-1 object headers are supported");
    const unsigned nmsg = (unsigned)le(&pre[2], 2);
    std::vector<std::pair<uint64_t, uint64_t>> chunks{{oh + 16, le(&pre[8], 4)}};
    Found r;
    unsigned seen = 0;
    for (size_t c = 0; c < chunks.size() && c < 64; ++c) {
        const auto ch = in.block(chunks[c].first, (size_t)chunks[c].second);
        size_t p = 0;
        while (p + 8 <= ch.size() && seen < nmsg) {
            const unsigned type = (unsigned)le(&ch[p], 2), sz = (unsigned)le(&ch[p + 2], 2);
            if (p + 8 + sz > ch.size()) bad("object header message overruns its block");
            const unsigned char* m = &ch[p + 8];
            ++seen;
            if (type == 0x0001) {  // dataspace
                const int ver = m[0];
                r.rank = m[1];
                if (r.rank > 8) bad("dataspace rank");
                const int off = ver == 1 ? 8 : 4;
                if (ver == 2 && m[3] == 2) bad("null dataspace");
                for (int a = 0; a < r.rank; ++a) r.dims[a] = le(m + off + 8 * a, 8);
            } else if (type == 0x0003) {  // datatype
                const int cls = m[0] & 0x0f;
                r.f64le = cls == 1 && (m[1] & 1) == 0 && le(m + 4, 4) == 8 && le(m + 10, 2) == 64;
            } else if (type == 0x0008) {  // data layout
                const int ver = m[0];
                if (ver == 3) {
                    r.layout = m[1];
                    if (r.layout == 1) {
                        r.addr = le(m + 2, 8);
                        r.bytes = le(m + 10, 8);
                    } else if (r.layout == 0) {
                        const size_t n = (size_t)le(m + 2, 2);
                        if (4 + n > sz) bad("compact data overruns its message");
                        r.compact.assign(m + 4, m + 4 + n);
                    } else {
                        bad("chunked or virtual storage is not supported");
                    }
                } else if (ver == 1 || ver == 2) {
                    const int nd = m[1];
                    r.layout = m[2];
                    if (r.layout != 1) bad("only contiguous storage is supported in layout versions 1-2");
                    r.addr = le(m + 8, 8);
                    uint64_t n = 1;
                    for (int a = 0; a < nd; ++a) n *= le(m + 16 + 4 * a, 4);
                    r.bytes = n;  // the last dimension is the element size
                } else {
                    bad("unknown data layout version");
                }
            } else if (type == 0x0010) {  // continuation
                chunks.push_back({le(m, 8), le(m + 8, 8)});
            }
            p += 8 + sz;
        }
    }
    return r;
}

// names and object headers of the root group's links
void list_group(const In& in, uint64_t btree, uint64_t heap_data, uint64_t heap_size,
                std::vector<std::pair<std::string, uint64_t>>& out, int depth) {
    if (depth > 32) bad("group B-tree too deep");
    const auto h = in.block(btree, 24);
    if (std::memcmp(h.data(), "TREE", 4) != 0 || h[4] != 0) bad("expected a group B-tree node");
    const int level = h[5];
    const unsigned used = (unsigned)le(&h[6], 2);
    const auto kc = in.block(btree + 24, (size_t)(8 + 16 * used));
    for (unsigned c = 0; c < used; ++c) {
        const uint64_t child = le(&kc[8 + 16 * c], 8);
        if (level > 0) {
            list_group(in, child, heap_data, heap_size, out, depth + 1);
            continue;
        }
        const auto sn = in.block(child, 8);
        if (std::memcmp(sn.data(), "SNOD", 4) != 0) bad("expected a symbol table node");
        const unsigned ns = (unsigned)le(&sn[6], 2);
        const auto ent = in.block(child + 8, (size_t)40 * ns);
        for (unsigned e = 0; e < ns; ++e) {
            const uint64_t off = le(&ent[40 * e], 8), oh = le(&ent[40 * e + 8], 8);
            if (off >= heap_size) bad("link name outside the local heap");
            const auto nm = in.block(heap_data + off, (size_t)std::min<uint64_t>(256, heap_size - off));
            const size_t len = strnlen((const char*)nm.data(), nm.size());
            out.push_back({std::string((const char*)nm.data(), len), oh});
        }
    }
}

std::vector<std::pair<std::string, uint64_t>> root_links(const In& in) {
    const auto sb = in.block(0, 24);
    if (std::memcmp(sb.data(), kSig, 8) != 0) bad("not an HDF5 file (no signature at offset 0)");
    const int ver = sb[8];
    if (ver > 1) bad("superblock versions 2 and 3 are not supported");
    if (sb[13] != 8 || sb[14] != 8) bad("only 8-byte offsets and lengths are supported");
    const uint64_t entry = ver == 0 ? 56 : 60;  // root group symbol table entry
    const auto re = in.block(entry, 40);
    uint64_t btree = le(&re[24], 8), heap = le(&re[32], 8);
    if (le(&re[16], 4) != 1) {  // no cached scratch-pad: the root object header's symbol table message
        const uint64_t oh = le(&re[8], 8);
        const auto pre = in.block(oh, 16);
        const auto ch = in.block(oh + 16, (size_t)le(&pre[8], 4));
        bool found = false;
        for (size_t p = 0; p + 8 <= ch.size();) {
            const unsigned type = (unsigned)le(&ch[p], 2), sz = (unsigned)le(&ch[p + 2], 2);
            if (type == 0x0011 && sz >= 16 && p + 24 <= ch.size()) {
                btree = le(&ch[p + 8], 8);
                heap = le(&ch[p + 16], 8);
                found = true;
                break;
            }
            p += 8 + sz;
        }
        if (!found) bad("the root group has no symbol table (newer group format)");
    }
    const auto hp = in.block(heap, 32);
    if (std::memcmp(hp.data(), "HEAP", 4) != 0) bad("expected a local heap");
    std::vector<std::pair<std::string, uint64_t>> links;
    list_group(in, btree, le(&hp[24], 8), le(&hp[8], 8), links, 0);
    return links;
}

// the dataset's FP64 values; dims (HDF5 order) must match `want` (rank 0 = scalar, or 1 element)
std::vector<double> read_dataset(const In& in, uint64_t oh, int rank, const uint64_t* want) {
    const Found f = read_object(in, oh);
    if (!f.f64le) bad("dataset is not IEEE little-endian float64");
    uint64_t n = 1;
    for (int a = 0; a < f.rank; ++a) n *= f.dims[a];
    if (rank == 0) {
        if (n != 1) throw ht3d_error(HT3D_ERR_ARG, "HDF5: time/dt is not a scalar");
    } else {
        if (f.rank != rank) throw ht3d_error(HT3D_ERR_ARG, "breakpoint grid differs from nx, ny, nz");
        for (int a = 0; a < rank; ++a)
            if (f.dims[a] != want[a]) throw ht3d_error(HT3D_ERR_ARG, "breakpoint grid differs from nx, ny, nz");
    }
    std::vector<double> v((size_t)n);
    if (f.layout == 0) {
        if (f.compact.size() != 8 * n) bad("compact data size");
        std::memcpy(v.data(), f.compact.data(), 8 * n);
    } else if (f.layout == 1) {
        if (f.addr == kUndef) {  // storage never allocated: the fill value (0)
            return v;
        }
        if (f.bytes < 8 * n || !in.at(f.addr, v.data(), (size_t)(8 * n))) bad("dataset data truncated");
    } else {
        bad("dataset has no data layout message");
    }
    return v;
}

}  // namespace

extern "C" {

int ht3d_breakpoint_write_h5(ht3d_ctx* ctx, const char* path, const double* Tc_ex, const double* Pc_ex, double time,
                             double dt, int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(path, Tc_ex, Pc_ex), "null argument");
        ht3d_check_dims(nx, ny, nz, 1);
        const uint64_t nex = (uint64_t)(nx + 2) * (ny + 2) * (nz + 2);
        std::vector<double> h(2 * nex);
        HT3D_CUDA(cudaMemcpyAsync(h.data(), Tc_ex, 8 * nex, cudaMemcpyDeviceToHost, ctx->stream));
        HT3D_CUDA(cudaMemcpyAsync(h.data() + nex, Pc_ex, 8 * nex, cudaMemcpyDeviceToHost, ctx->stream));
        HT3D_CUDA(cudaStreamSynchronize(ctx->stream));
        // the reference's write order: Tc_ex, Pc_ex, time, dt (v18.jl:583-586)
        const Dataset ds[4] = {
            {"Tc_ex", 3, {(uint64_t)nz + 2, (uint64_t)ny + 2, (uint64_t)nx + 2}, h.data(), nex},
            {"Pc_ex", 3, {(uint64_t)nz + 2, (uint64_t)ny + 2, (uint64_t)nx + 2}, h.data() + nex, nex},
            {"time", 0, {}, &time, 1},
            {"dt", 0, {}, &dt, 1}};
        std::vector<uint64_t> addr;
        const std::vector<unsigned char> head = h5_image_header(ds, 4, addr);
        FILE* f = std::fopen(path, "wb");
        if (!f) throw ht3d_error(HT3D_ERR_IO, std::string("cannot write ") + path);
        bool ok = std::fwrite(head.data(), 1, head.size(), f) == head.size();
        for (int d = 0; d < 4 && ok; ++d) ok = std::fwrite(ds[d].data, 8, (size_t)ds[d].n, f) == ds[d].n;
        ok = (std::fclose(f) == 0) && ok;
        if (!ok) throw ht3d_error(HT3D_ERR_IO, std::string("cannot write ") + path);
        return HT3D_OK;
    });
}

int ht3d_breakpoint_read_h5(ht3d_ctx* ctx, const char* path, double* Tc_ex, double* Pc_ex, double* time, double* dt,
                            int nx, int ny, int nz) {
    return ht3d_guard(ctx, [&]() {
        HT3D_REQUIRE(all_nonnull(path, Tc_ex, Pc_ex, time, dt), "null argument");
        ht3d_check_dims(nx, ny, nz, 1);
        In in;
        in.f = std::fopen(path, "rb");
        if (!in.f) throw ht3d_error(HT3D_ERR_IO, std::string("cannot open ") + path);
        if (std::fseek(in.f, 0, SEEK_END) != 0) throw ht3d_error(HT3D_ERR_IO, "cannot seek");
        in.size = (uint64_t)std::ftell(in.f);
        const auto links = root_links(in);
        auto find = [&](const char* name) {
            for (const auto& l : links)
                if (l.first == name) return l.second;
            throw ht3d_error(HT3D_ERR_IO, std::string("HDF5: no dataset ") + name + " in " + path);
        };
        const uint64_t want[3] = {(uint64_t)nz + 2, (uint64_t)ny + 2, (uint64_t)nx + 2};
        const std::vector<double> T = read_dataset(in, find("Tc_ex"), 3, want);
        const std::vector<double> P = read_dataset(in, find("Pc_ex"), 3, want);
        const double t = read_dataset(in, find("time"), 0, nullptr)[0];
        const double d = read_dataset(in, find("dt"), 0, nullptr)[0];
        HT3D_CUDA(cudaMemcpyAsync(Tc_ex, T.data(), 8 * T.size(), cudaMemcpyHostToDevice, ctx->stream));
        HT3D_CUDA(cudaMemcpyAsync(Pc_ex, P.data(), 8 * P.size(), cudaMemcpyHostToDevice, ctx->stream));
        HT3D_CUDA(cudaStreamSynchronize(ctx->stream));  // T and P are released on return
        *time = t;
        *dt = d;
        return HT3D_OK;
    });
}

// the file image without touching a device: for the CPU tests of the format
int ht3d_h5_breakpoint_image(const char* path, const double* Tc_ex, const double* Pc_ex, double time, double dt,
                             int nx, int ny, int nz) {
    if (!path || !Tc_ex || !Pc_ex || nx < 1 || ny < 1 || nz < 1) return HT3D_ERR_ARG;
    const uint64_t nex = (uint64_t)(nx + 2) * (ny + 2) * (nz + 2);
    const Dataset ds[4] = {{"Tc_ex", 3, {(uint64_t)nz + 2, (uint64_t)ny + 2, (uint64_t)nx + 2}, Tc_ex, nex},
                           {"Pc_ex", 3, {(uint64_t)nz + 2, (uint64_t)ny + 2, (uint64_t)nx + 2}, Pc_ex, nex},
                           {"time", 0, {}, &time, 1},
                           {"dt", 0, {}, &dt, 1}};
    std::vector<uint64_t> addr;
    const std::vector<unsigned char> head = h5_image_header(ds, 4, addr);
    FILE* f = std::fopen(path, "wb");
    if (!f) return HT3D_ERR_IO;
    bool ok = std::fwrite(head.data(), 1, head.size(), f) == head.size();
    for (int d = 0; d < 4 && ok; ++d) ok = std::fwrite(ds[d].data, 8, (size_t)ds[d].n, f) == ds[d].n;
    ok = (std::fclose(f) == 0) && ok;
    return ok ? HT3D_OK : HT3D_ERR_IO;
}

// reads a file's four items into HOST arrays (the CPU tests' reader)
int ht3d_h5_breakpoint_parse(const char* path, double* Tc_ex, double* Pc_ex, double* time, double* dt, int nx, int ny,
                             int nz) {
    if (!path || !Tc_ex || !Pc_ex || !time || !dt || nx < 1 || ny < 1 || nz < 1) return HT3D_ERR_ARG;
    try {
        In in;
        in.f = std::fopen(path, "rb");
        if (!in.f) return HT3D_ERR_IO;
        if (std::fseek(in.f, 0, SEEK_END) != 0) return HT3D_ERR_IO;
        in.size = (uint64_t)std::ftell(in.f);
        const auto links = root_links(in);
        auto find = [&](const char* name) {
            for (const auto& l : links)
                if (l.first == name) return l.second;
            throw ht3d_error(HT3D_ERR_IO, "missing dataset");
        };
        const uint64_t want[3] = {(uint64_t)nz + 2, (uint64_t)ny + 2, (uint64_t)nx + 2};
        const std::vector<double> T = read_dataset(in, find("Tc_ex"), 3, want);
        const std::vector<double> P = read_dataset(in, find("Pc_ex"), 3, want);
        *time = read_dataset(in, find("time"), 0, nullptr)[0];
        *dt = read_dataset(in, find("dt"), 0, nullptr)[0];
        std::memcpy(Tc_ex, T.data(), 8 * T.size());
        std::memcpy(Pc_ex, P.data(), 8 * P.size());
        return HT3D_OK;
    } catch (const ht3d_error& e) {
        return e.code;
    }
}

}  // extern "C"
