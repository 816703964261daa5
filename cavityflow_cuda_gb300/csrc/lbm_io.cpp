// lbm_io.cpp -- checkpoint/resume and VTK output of a solver.
//
// Checkpoint file (little-endian):
//   char[16]  "LBMGB300CKPT" padded with zeros
//   uint32    version (2; version-1 files, without the lid record, are read
//             as the injection lid)
//   int32     storage, nx, ny, nz
//   int64     step counter
//   int32     last step was alpha, FP64 fused multiply-adds (0/1)
//   double    inv_tau, lid velocity, gravity x, y, z
//   int32     boundary[6]
//   uint64    flag bytes, population bytes
//   int32     lid mode, moving wall (0/1)            -- version 2 only
//   uint8     flags of the (nx+2)(ny+2)(nz+2) cells, x fastest
//   raw       populations: 19 slots of the same cells in the storage type
//             (16-bit storage: the stored deviations, bit for bit)
// The step parity is part of the state: after an alpha step the populations
// sit in swapped slots, so a resumed run continues exactly where it stopped.
//
// VTK: the legacy structured-grid file of the reference's
// CLbmVisualizationVTK (src/libvis/CLbmVisualizationVTK.cpp:69-205): points at
// the cell corners, then CELL_DATA with flags, densities and velocities of
// the interior, ASCII as the reference writes it or legacy big-endian binary.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/lbm_gb300.h"
#include "lbm_internal.h"
#include "lbm_kernels.h"

using namespace lbm_detail;

namespace {

const char kMagic[16] = {'L', 'B', 'M', 'G', 'B', '3', '0', '0', 'C', 'K', 'P', 'T', 0, 0, 0, 0};

#pragma pack(push, 1)
struct CkptHeader {
    char magic[16];
    uint32_t version;
    int32_t storage, nx, ny, nz;
    int64_t counter;
    int32_t last_alpha, fma;
    double inv_tau, lid_u, gx, gy, gz;
    int32_t boundary[6];
    uint64_t flag_bytes, pop_bytes;
};
// Appended by version 2.
struct CkptLid {
    int32_t lid_mode, moving_wall;
};
#pragma pack(pop)

// Raw copy of all 19 slots of the full (halo-included) domain between the
// padded device layout and a packed host buffer in the storage type.
int raw_populations(lbm_solver* s, void* host, bool to_host)
{
    const size_t eb = (size_t)elem_bytes(s->storage);
    const lbm::Grid& g = s->g;
    const size_t cells = (size_t)g.cells();
    for (int k = 0; k < lbm::Q; ++k) {
        cudaMemcpy3DParms m = {};
        char* base = static_cast<char*>(s->dd) + (size_t)k * g.S * eb;
        cudaPitchedPtr dptr = make_cudaPitchedPtr(base, (size_t)g.P * eb, (size_t)g.P, (size_t)(g.ny + 2));
        cudaPitchedPtr hptr =
            make_cudaPitchedPtr(static_cast<char*>(host) + (size_t)k * cells * eb, (size_t)(g.nx + 2) * eb,
                                (size_t)(g.nx + 2), (size_t)(g.ny + 2));
        const cudaPos dpos = make_cudaPos((size_t)g.xoff * eb, 0, 0);
        if (to_host) {
            m.srcPtr = dptr; m.srcPos = dpos; m.dstPtr = hptr; m.kind = cudaMemcpyDeviceToHost;
        } else {
            m.srcPtr = hptr; m.dstPtr = dptr; m.dstPos = dpos; m.kind = cudaMemcpyHostToDevice;
        }
        m.extent = make_cudaExtent((size_t)(g.nx + 2) * eb, (size_t)(g.ny + 2), (size_t)(g.nz + 2));
        const cudaError_t e = cudaMemcpy3D(&m);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy3D checkpoint populations");
    }
    return LBM_OK;
}

struct File {
    FILE* f = nullptr;
    ~File()
    {
        if (f) std::fclose(f);
    }
};

void be32(unsigned char* p, uint32_t v)
{
    p[0] = (unsigned char)(v >> 24); p[1] = (unsigned char)(v >> 16);
    p[2] = (unsigned char)(v >> 8); p[3] = (unsigned char)v;
}

void be64(unsigned char* p, uint64_t v)
{
    for (int i = 0; i < 8; ++i) p[i] = (unsigned char)(v >> (56 - 8 * i));
}

}  // namespace

extern "C" {

static int save_checkpoint_unguarded(lbm_solver* s, const char* path)
{
    if (!s || !path) return fail(LBM_ERR_INVALID_ARGUMENT, "NULL argument");
    if (int r = lbm_synchronize(s)) return r;
    const lbm::Grid& g = s->g;
    const size_t cells = (size_t)g.cells();
    CkptHeader h;
    std::memset(&h, 0, sizeof(h));
    std::memcpy(h.magic, kMagic, 16);
    h.version = 2;
    const CkptLid lid = {s->lid_mode, s->p.wall_y > 0 ? 1 : 0};
    h.storage = s->storage;
    h.nx = g.nx; h.ny = g.ny; h.nz = g.nz;
    h.counter = s->counter;
    h.last_alpha = s->last_alpha ? 1 : 0;
    h.fma = s->fma ? 1 : 0;
    h.inv_tau = s->p.inv_tau; h.lid_u = s->p.lid_u;
    h.gx = s->p.gx; h.gy = s->p.gy; h.gz = s->p.gz;
    for (int f = 0; f < 6; ++f) h.boundary[f] = s->bc[f];
    h.flag_bytes = cells;
    h.pop_bytes = (uint64_t)lbm::Q * cells * (uint64_t)elem_bytes(s->storage);
    std::vector<unsigned char> flags(cells);
    const cudaError_t e = cudaMemcpy(flags.data(), s->flags, cells, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy checkpoint flags");
    std::vector<unsigned char> pops((size_t)h.pop_bytes);
    if (int r = raw_populations(s, pops.data(), true)) return r;
    const std::string tmp = std::string(path) + ".tmp";
    {
        File out;
        out.f = std::fopen(tmp.c_str(), "wb");
        if (!out.f) return fail(LBM_ERR_IO, "cannot write checkpoint \"%s\"", tmp.c_str());
        if (std::fwrite(&h, sizeof(h), 1, out.f) != 1 || std::fwrite(&lid, sizeof(lid), 1, out.f) != 1 ||
            std::fwrite(flags.data(), 1, cells, out.f) != cells ||
            std::fwrite(pops.data(), 1, pops.size(), out.f) != pops.size())
            return fail(LBM_ERR_IO, "short write to \"%s\"", tmp.c_str());
        if (std::fflush(out.f) != 0) return fail(LBM_ERR_IO, "cannot flush \"%s\"", tmp.c_str());
    }
    if (std::rename(tmp.c_str(), path) != 0) return fail(LBM_ERR_IO, "cannot rename to \"%s\"", path);
    return LBM_OK;
}

// Reads the header and validates it against a solver (or returns it).
static int read_header(FILE* f, const char* path, CkptHeader& h, CkptLid& lid)
{
    if (std::fread(&h, sizeof(h), 1, f) != 1) return fail(LBM_ERR_IO, "\"%s\": truncated header", path);
    if (std::memcmp(h.magic, kMagic, 16) != 0 || (h.version != 1 && h.version != 2))
        return fail(LBM_ERR_IO, "\"%s\" is not a version-1 or -2 checkpoint of this solver", path);
    lid = {LBM_LID_INJECTION, 0};
    if (h.version == 2) {
        if (std::fread(&lid, sizeof(lid), 1, f) != 1) return fail(LBM_ERR_IO, "\"%s\": truncated header", path);
        if ((lid.lid_mode != LBM_LID_INJECTION && lid.lid_mode != LBM_LID_MOVING_WALL) ||
            (lid.moving_wall != 0 && lid.moving_wall != 1) || (lid.moving_wall && !lid.lid_mode))
            return fail(LBM_ERR_IO, "\"%s\": corrupt header", path);
    }
    // each axis within lbm_create's limit [1, 2^20], so the products below
    // are exact in 64 bits
    const auto axis_ok = [](int32_t n) { return n > 0 && n <= (1 << 20); };
    if (h.storage < LBM_STORAGE_F64 || h.storage > LBM_STORAGE_F16SR || !axis_ok(h.nx) || !axis_ok(h.ny) ||
        !axis_ok(h.nz) || (h.fma != 0 && h.fma != 1))
        return fail(LBM_ERR_IO, "\"%s\": corrupt header", path);
    const uint64_t cells = ((uint64_t)h.nx + 2) * ((uint64_t)h.ny + 2) * ((uint64_t)h.nz + 2);
    if (h.flag_bytes != cells || h.pop_bytes != (uint64_t)lbm::Q * cells * (uint64_t)elem_bytes(h.storage))
        return fail(LBM_ERR_IO, "\"%s\": sizes do not match the header", path);
    return LBM_OK;
}

static int load_checkpoint_unguarded(lbm_solver* s, const char* path)
{
    if (!s || !path) return fail(LBM_ERR_INVALID_ARGUMENT, "NULL argument");
    File in;
    in.f = std::fopen(path, "rb");
    if (!in.f) return fail(LBM_ERR_IO, "cannot read checkpoint \"%s\"", path);
    CkptHeader h;
    CkptLid lid;
    if (int r = read_header(in.f, path, h, lid)) return r;
    if (h.storage != s->storage || h.nx != s->g.nx || h.ny != s->g.ny || h.nz != s->g.nz)
        return fail(LBM_ERR_INVALID_ARGUMENT, "\"%s\" holds a %dx%dx%d domain of storage %d", path, h.nx, h.ny, h.nz,
                    h.storage);
    if (lid.lid_mode != s->lid_mode)
        return fail(LBM_ERR_INVALID_ARGUMENT, "\"%s\" was written with lid mode %d, the solver has %d", path,
                    lid.lid_mode, s->lid_mode);
    std::vector<unsigned char> flags((size_t)h.flag_bytes);
    std::vector<unsigned char> pops((size_t)h.pop_bytes);
    if (std::fread(flags.data(), 1, flags.size(), in.f) != flags.size() ||
        std::fread(pops.data(), 1, pops.size(), in.f) != pops.size())
        return fail(LBM_ERR_IO, "\"%s\": truncated data", path);
    if (int r = lbm_synchronize(s)) return r;
    std::vector<int32_t> f32(flags.begin(), flags.end());
    const int32_t origin[3] = {0, 0, 0};
    const int32_t size[3] = {h.nx + 2, h.ny + 2, h.nz + 2};
    if (int r = lbm_set_flags(s, origin, size, f32.data())) return r;
    if (int r = raw_populations(s, pops.data(), false)) return r;
    s->counter = h.counter;
    s->last_alpha = h.last_alpha != 0;
    s->macros_fresh = false;
    if ((s->p.wall_y > 0) != (lid.moving_wall != 0)) {  // the wall's state as saved; graphs hold the old one
        s->p.wall_y = lid.moving_wall ? s->g.ny : 0;
        if (s->graph) {
            cudaGraphExecDestroy(s->graph);
            s->graph = nullptr;
        }
    }
    return LBM_OK;
}

static int create_from_checkpoint_unguarded(const char* path, int32_t device, lbm_solver** out)
{
    if (!path || !out) return fail(LBM_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = nullptr;
    CkptHeader h;
    CkptLid lid;
    {
        File in;
        in.f = std::fopen(path, "rb");
        if (!in.f) return fail(LBM_ERR_IO, "cannot read checkpoint \"%s\"", path);
        if (int r = read_header(in.f, path, h, lid)) return r;
    }
    lbm_params p;
    std::memset(&p, 0, sizeof(p));
    p.size[0] = h.nx; p.size[1] = h.ny; p.size[2] = h.nz;
    p.storage = h.storage;
    for (int f = 0; f < 6; ++f) p.boundary[f] = h.boundary[f];
    p.inv_tau = h.inv_tau;
    p.lid_velocity = h.lid_u;
    p.gravity[0] = h.gx; p.gravity[1] = h.gy; p.gravity[2] = h.gz;
    p.device = device;
    p.fused_multiply_add = h.fma;  // resume with the arithmetic that wrote the checkpoint
    p.lid_mode = lid.lid_mode;
    lbm_solver* s = nullptr;
    if (int r = lbm_create(&p, &s)) return r;
    if (int r = lbm_load_checkpoint(s, path)) {
        lbm_destroy(s);
        return r;
    }
    *out = s;
    return LBM_OK;
}

static int write_vtk_unguarded(lbm_solver* s, const char* path, const double length[3], int32_t binary)
{
    if (!s || !path) return fail(LBM_ERR_INVALID_ARGUMENT, "NULL argument");
    const int nx = s->g.nx, ny = s->g.ny, nz = s->g.nz;
    const size_t n = (size_t)nx * ny * nz;
    const bool dbl = s->storage == LBM_STORAGE_F64;
    const double L[3] = {length ? length[0] : (double)nx, length ? length[1] : (double)ny,
                         length ? length[2] : (double)nz};
    std::vector<int32_t> flags(n);
    std::vector<double> rho(n), u(3 * n);
    std::vector<float> rho_f, u_f;
    if (int r = lbm_get_flags(s, nullptr, nullptr, flags.data())) return r;
    if (dbl) {
        if (int r = lbm_get_densities(s, nullptr, nullptr, rho.data())) return r;
        if (int r = lbm_get_velocities(s, nullptr, nullptr, u.data())) return r;
    } else {
        rho_f.resize(n);
        u_f.resize(3 * n);
        if (int r = lbm_get_densities(s, nullptr, nullptr, rho_f.data())) return r;
        if (int r = lbm_get_velocities(s, nullptr, nullptr, u_f.data())) return r;
        for (size_t i = 0; i < n; ++i) rho[i] = rho_f[i];
        for (size_t i = 0; i < 3 * n; ++i) u[i] = u_f[i];
    }
    File out;
    out.f = std::fopen(path, "wb");
    if (!out.f) return fail(LBM_ERR_IO, "cannot write \"%s\"", path);
    FILE* f = out.f;
    const char* type = dbl ? "double" : "float";
    std::fprintf(f, "# vtk DataFile Version 3.0\nGB300 D3Q19 lid-driven cavity, step %lld\n%s\n",
                 (long long)s->counter, binary ? "BINARY" : "ASCII");
    std::fprintf(f, "DATASET STRUCTURED_GRID\nDIMENSIONS %d %d %d\nPOINTS %lld %s\n", nx + 1, ny + 1, nz + 1,
                 (long long)(nx + 1) * (ny + 1) * (nz + 1), type);
    unsigned char b[8];
    auto put = [&](double v) {
        if (!binary) {
            std::fprintf(f, "%g", v);
            return;
        }
        if (dbl) {
            uint64_t x;
            std::memcpy(&x, &v, 8);
            be64(b, x);
            std::fwrite(b, 1, 8, f);
        } else {
            const float fv = (float)v;
            uint32_t x;
            std::memcpy(&x, &fv, 4);
            be32(b, x);
            std::fwrite(b, 1, 4, f);
        }
    };
    auto sep = [&](char c) {
        if (!binary) std::fputc(c, f);
    };
    // (origin + i) * length / size in the value type, as the reference
    // computes the corner coordinates (origin 0: one subdomain)
    auto corner = [&](int i, int d, int n) -> double {
        if (dbl) return (double)i * L[d] / (double)n;
        return (double)((float)i * (float)L[d] / (float)n);
    };
    for (int k = 0; k <= nz; ++k)
        for (int j = 0; j <= ny; ++j)
            for (int i = 0; i <= nx; ++i) {
                put(corner(i, 0, nx)); sep(' ');
                put(corner(j, 1, ny)); sep(' ');
                put(corner(k, 2, nz)); sep('\n');
            }
    if (binary) std::fputc('\n', f);
    std::fprintf(f, "CELL_DATA %lld\nSCALARS flags INT 1\nLOOKUP_TABLE default\n", (long long)n);
    for (size_t i = 0; i < n; ++i) {
        if (binary) {
            be32(b, (uint32_t)flags[i]);
            std::fwrite(b, 1, 4, f);
        } else {
            std::fprintf(f, "%d\n", flags[i]);
        }
    }
    if (binary) std::fputc('\n', f);
    std::fprintf(f, "SCALARS densities %s 1\nLOOKUP_TABLE default\n", type);
    for (size_t i = 0; i < n; ++i) {
        put(rho[i]);
        sep('\n');
    }
    if (binary) std::fputc('\n', f);
    std::fprintf(f, "VECTORS velocities %s\n", type);
    for (size_t i = 0; i < n; ++i) {
        put(u[i]); sep(' ');
        put(u[n + i]); sep(' ');
        put(u[2 * n + i]); sep('\n');
    }
    if (std::ferror(f)) return fail(LBM_ERR_IO, "error writing \"%s\"", path);
    return LBM_OK;
}

int lbm_save_checkpoint(lbm_solver* s, const char* path)
{
    return guarded("lbm_save_checkpoint", [&] { return save_checkpoint_unguarded(s, path); });
}

int lbm_load_checkpoint(lbm_solver* s, const char* path)
{
    return guarded("lbm_load_checkpoint", [&] { return load_checkpoint_unguarded(s, path); });
}

int lbm_create_from_checkpoint(const char* path, int32_t device, lbm_solver** out)
{
    return guarded("lbm_create_from_checkpoint", [&] { return create_from_checkpoint_unguarded(path, device, out); });
}

int lbm_write_vtk(lbm_solver* s, const char* path, const double length[3], int32_t binary)
{
    return guarded("lbm_write_vtk", [&] { return write_vtk_unguarded(s, path, length, binary); });
}

}  // extern "C"
