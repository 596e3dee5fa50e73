// io.cu -- restart and visualisation files written from device snapshots.
//
// PETSc binary Vec records: what the reference's MonitorFunction writes every
// RestartInterval steps and reads back at start-up (3d/weno3/Euler/monitor_function.c:46-62,
// hype.c:147-155: PetscViewerBinaryOpen + VecView / VecLoad).  The record is the
// int32 class id 1211214, the int32 length and the entries as big-endian IEEE
// doubles; for a single-rank DMDA vector the entries are in the DMDA's natural
// order, [k][j][i][c] with the components interleaved, and PETSc writes the
// block size of a multi-component vector into a companion "<file>.info"
// (-vecload_block_size <dof>).  Legacy VTK 2.0 ASCII files (the format of the
// reference's PETSC_VIEWER_ASCII_VTK output, hype.c:202-208) carry one SCALARS
// section per component on the cell-centre lattice.
//
// Host code only: the state comes to the host through hype_euler_download /
// hype_mp2d_download (one device->host copy) and goes back through the uploads.
#include <errno.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <string>
#include <vector>

#include "hype_common.cuh"

namespace {

constexpr int32_t kVecClassId = 1211214;

void be32(unsigned char* b, int32_t x) {
    const uint32_t u = (uint32_t)x;
    b[0] = (unsigned char)(u >> 24);
    b[1] = (unsigned char)(u >> 16);
    b[2] = (unsigned char)(u >> 8);
    b[3] = (unsigned char)u;
}

int32_t rd_be32(const unsigned char* b) {
    return (int32_t)(((uint32_t)b[0] << 24) | ((uint32_t)b[1] << 16) | ((uint32_t)b[2] << 8) | (uint32_t)b[3]);
}

void be64(unsigned char* b, double d) {
    uint64_t u;
    memcpy(&u, &d, 8);
    for (int k = 0; k < 8; ++k) b[k] = (unsigned char)(u >> (56 - 8 * k));
}

double rd_be64(const unsigned char* b) {
    uint64_t u = 0;
    for (int k = 0; k < 8; ++k) u = (u << 8) | b[k];
    double d;
    memcpy(&d, &u, 8);
    return d;
}

int io_error(const char* what, const char* path) {
    std::string m = std::string(what) + ": " + (path ? path : "(null)") + ": " + strerror(errno);
    hype::set_last_error(m.c_str(), cudaSuccess);
    return HYPE_ERR_ARG;
}

}  // namespace

extern "C" int hype_write_petsc_vec(const char* path, const double* v, long long n, int block_size) {
    if (!path || (!v && n > 0) || n < 0 || n > 0x7fffffffLL || block_size < 1) return HYPE_ERR_ARG;
    FILE* f = fopen(path, "wb");
    if (!f) return io_error("hype_write_petsc_vec: cannot open", path);
    unsigned char h[8];
    be32(h, kVecClassId);
    be32(h + 4, (int32_t)n);
    bool ok = fwrite(h, 1, 8, f) == 8;
    std::vector<unsigned char> buf(8 * 65536);
    for (long long i0 = 0; ok && i0 < n; i0 += 65536) {
        const long long m = (n - i0) < 65536 ? (n - i0) : 65536;
        for (long long i = 0; i < m; ++i) be64(&buf[8 * i], v[i0 + i]);
        ok = fwrite(buf.data(), 1, (size_t)(8 * m), f) == (size_t)(8 * m);
    }
    if (fclose(f) != 0) ok = false;
    if (!ok) return io_error("hype_write_petsc_vec: write failed", path);
    if (block_size > 1) {
        const std::string info = std::string(path) + ".info";
        FILE* g = fopen(info.c_str(), "w");
        if (!g) return io_error("hype_write_petsc_vec: cannot open", info.c_str());
        fprintf(g, "-vecload_block_size %d\n", block_size);
        if (fclose(g) != 0) return io_error("hype_write_petsc_vec: write failed", info.c_str());
    }
    return HYPE_OK;
}

extern "C" int hype_read_petsc_vec(const char* path, double* v, long long n) {
    if (!path || !v || n < 0) return HYPE_ERR_ARG;
    FILE* f = fopen(path, "rb");
    if (!f) return io_error("hype_read_petsc_vec: cannot open", path);
    unsigned char h[8];
    if (fread(h, 1, 8, f) != 8 || rd_be32(h) != kVecClassId || rd_be32(h + 4) != n) {
        fclose(f);
        hype::set_last_error("hype_read_petsc_vec: not a PETSc Vec record of the expected length", cudaSuccess);
        return HYPE_ERR_ARG;
    }
    std::vector<unsigned char> buf(8 * 65536);
    bool ok = true;
    for (long long i0 = 0; ok && i0 < n; i0 += 65536) {
        const long long m = (n - i0) < 65536 ? (n - i0) : 65536;
        ok = fread(buf.data(), 1, (size_t)(8 * m), f) == (size_t)(8 * m);
        for (long long i = 0; ok && i < m; ++i) v[i0 + i] = rd_be64(&buf[8 * i]);
    }
    fclose(f);
    if (!ok) {
        hype::set_last_error("hype_read_petsc_vec: file shorter than its header says", cudaSuccess);
        return HYPE_ERR_ARG;
    }
    return HYPE_OK;
}

// Legacy VTK 2.0 ASCII: STRUCTURED_POINTS on the cell centres (origin + h/2),
// one SCALARS section per component of the interleaved [k][j][i][c] array.
extern "C" int hype_write_vtk(const char* path, const char* title, int nx, int ny, int nz, double x0, double y0, double z0,
                              double h, int ncomp, const char* const* names, const double* aos) {
    if (!path || !aos || !names || nx < 1 || ny < 1 || nz < 1 || ncomp < 1 || !(h > 0)) return HYPE_ERR_ARG;
    FILE* f = fopen(path, "w");
    if (!f) return io_error("hype_write_vtk: cannot open", path);
    const long long n = (long long)nx * ny * nz;
    fprintf(f, "# vtk DataFile Version 2.0\n%s\nASCII\nDATASET STRUCTURED_POINTS\n", title ? title : "HyPE solution");
    fprintf(f, "DIMENSIONS %d %d %d\n", nx, ny, nz);
    fprintf(f, "ORIGIN %.17g %.17g %.17g\n", x0 + 0.5 * h, y0 + 0.5 * h, nz > 1 ? z0 + 0.5 * h : z0);
    fprintf(f, "SPACING %.17g %.17g %.17g\n", h, h, h);
    fprintf(f, "POINT_DATA %lld\n", n);
    for (int c = 0; c < ncomp; ++c) {
        fprintf(f, "SCALARS %s double 1\nLOOKUP_TABLE default\n", names[c] ? names[c] : "field");
        for (long long q = 0; q < n; ++q) fprintf(f, "%.17g\n", aos[q * ncomp + c]);
    }
    if (ferror(f)) {
        fclose(f);
        return io_error("hype_write_vtk: write failed", path);
    }
    if (fclose(f) != 0) return io_error("hype_write_vtk: write failed", path);
    return HYPE_OK;
}

// ---------------------------------------------------------------- solver snapshots
extern "C" int hype_euler_write_restart(hype_euler* e, const char* path) {
    hype_euler_params p;
    int rc = hype_euler_get_params(e, &p);
    if (rc || !path) return rc ? rc : HYPE_ERR_ARG;
    std::vector<double> u((size_t)p.nx * p.ny * p.nz * 5);
    if ((rc = hype_euler_download(e, u.data()))) return rc;
    return hype_write_petsc_vec(path, u.data(), (long long)u.size(), 5);
}

extern "C" int hype_euler_read_restart(hype_euler* e, const char* path) {
    hype_euler_params p;
    int rc = hype_euler_get_params(e, &p);
    if (rc || !path) return rc ? rc : HYPE_ERR_ARG;
    std::vector<double> u((size_t)p.nx * p.ny * p.nz * 5);
    if ((rc = hype_read_petsc_vec(path, u.data(), (long long)u.size()))) return rc;
    return hype_euler_upload(e, u.data());
}

extern "C" int hype_euler_write_vtk(hype_euler* e, const char* path) {
    hype_euler_params p;
    int rc = hype_euler_get_params(e, &p);
    if (rc || !path) return rc ? rc : HYPE_ERR_ARG;
    std::vector<double> u((size_t)p.nx * p.ny * p.nz * 5);
    if ((rc = hype_euler_download(e, u.data()))) return rc;
    static const char* const names[5] = {"density", "x-momentum", "y-momentum", "z-momentum", "energy"};
    return hype_write_vtk(path, "HyPE 3D Euler conserved variables", p.nx, p.ny, p.nz, p.x_min, p.y_min, p.z_min, p.h, 5,
                          names, u.data());
}

extern "C" int hype_mp2d_write_restart(hype_mp2d* m, const char* path) {
    hype_mp2d_params p;
    int rc = hype_mp2d_get_params(m, &p);
    if (rc || !path) return rc ? rc : HYPE_ERR_ARG;
    const int nv = p.model == HYPE_MP_DI4 ? 5 : 6;
    std::vector<double> u((size_t)p.nx * p.ny * nv);
    if ((rc = hype_mp2d_download(m, u.data()))) return rc;
    return hype_write_petsc_vec(path, u.data(), (long long)u.size(), nv);
}

extern "C" int hype_mp2d_read_restart(hype_mp2d* m, const char* path) {
    hype_mp2d_params p;
    int rc = hype_mp2d_get_params(m, &p);
    if (rc || !path) return rc ? rc : HYPE_ERR_ARG;
    const int nv = p.model == HYPE_MP_DI4 ? 5 : 6;
    std::vector<double> u((size_t)p.nx * p.ny * nv);
    if ((rc = hype_read_petsc_vec(path, u.data(), (long long)u.size()))) return rc;
    return hype_mp2d_upload(m, u.data());
}

extern "C" int hype_mp2d_write_vtk(hype_mp2d* m, const char* path) {
    hype_mp2d_params p;
    int rc = hype_mp2d_get_params(m, &p);
    if (rc || !path) return rc ? rc : HYPE_ERR_ARG;
    const int nv = p.model == HYPE_MP_DI4 ? 5 : 6;
    std::vector<double> u((size_t)p.nx * p.ny * nv);
    if ((rc = hype_mp2d_download(m, u.data()))) return rc;
    static const char* const di4[5] = {"rho", "rho_u", "rho_v", "E", "phi"};
    static const char* const kap[6] = {"alpha1_rho1", "alpha2_rho2", "rho_u", "rho_v", "E", "alpha1"};
    return hype_write_vtk(path, "HyPE 2D multiphase conserved variables", p.nx, p.ny, 1, p.x_min, p.y_min, 0.0, p.h, nv,
                          nv == 5 ? di4 : kap, u.data());
}
