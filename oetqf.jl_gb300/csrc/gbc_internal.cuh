// Internal declarations shared by the libgbcycle translation units.
#pragma once
#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "gbcycle.h"

namespace gbc {

// thread-local last-error message, returned by gbc_last_error()
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

#define GBC_CUDA(call)                                       \
    do {                                                     \
        cudaError_t _e = (call);                             \
        if (_e != cudaSuccess) return ::gbc::cuda_fail(_e, #call); \
    } while (0)

constexpr int kSMs = 152;  // GB300: 2 dies x 76 SMs (grids are sized from the live count)
int sm_count();
// raises a kernel's dynamic shared-memory limit on the current device (the attribute is per
// device; thread-safe, set once per kernel, device and size)
int set_smem_limit(const void* fn, int bytes);

// adds n to the library's kernel-launch counter (gbc_kernel_launches)
void count_launches(long long n);

// 2-D tiled TMA descriptor (CUtensorMap, 128 bytes at tmap_out) over a row-major rows x cols array
// of esize-byte elements of CUtensorMapDataType dtype, box box_rows x box_cols; swizzle128 selects
// the 128-byte swizzle (box_cols * esize must then be 128)
int encode_tmap_2d(void* base, int dtype, int esize, long long rows, long long cols, int box_cols, int box_rows,
                   bool swizzle128, void* tmap_out);

// Gauss-Legendre tables for the strain-volume stacks (4, 8, 12, 16 nodes), in constant memory.
void gl_rule(int n, double* x, double* w);
int upload_gl_tables();

// ---- Green's-function assembly launches (gf_kernels.cu) -------------------------------------
struct FaultDev {       // device copy of a fault mesh
    int nx, nxi;
    const double *x, *y, *z, *ax, *axi;  // ax: (nx,2) interleaved, axi: (nxi,2)
    double dx, dep, dip;
};
struct HexDev {
    int ne;
    const double *cx, *cy, *cz, *qx, *qy, *qz, *dx, *dy, *dz;
};
// st (nx,nxi,nxi) column-major real Toeplitz kernel
int launch_gf_ff(const FaultDev& f, double lambda, double mu, int ftype, int nrept,
                 double buffer_ratio, double* st, cudaStream_t s);
// rFFT of the circulant embedding, complex interleaved (nx,nxi,nxi)
int launch_gf_ff_dft(int nx, int nxi, const double* st, double* st_dft, cudaStream_t s);
// inverse: recover the real Toeplitz kernel from the reference's complex (nx,nxi,nxi) form
int launch_gf_ff_idft(int nx, int nxi, const double* st_dft, double* st, cudaStream_t s);
// fault -> mantle: rows (k*ne + i), cols j; written into a row-major matrix with leading dim ld
int launch_gf_fm(const FaultDev& f, const HexDev& m, double lambda, double mu, int ftype,
                 int nrept, double buffer_ratio, const double* qc, const double* qw, int nq,
                 double* out, size_t ld, cudaStream_t s);
// mantle -> fault: rows i (fault patch), cols (p*ne + j), row-major with leading dim ld
int launch_gf_mf(const HexDev& m, const FaultDev& f, double lambda, double mu, int ftype,
                 double* out, size_t ld, cudaStream_t s);
// structured mantle boxes: per-cell grid indices (see mm_grid)
struct MMGrid {
    int nX = 0, nY = 0, nZ = 0;
    std::vector<int> ix, iy, iz, cell;
};
bool mm_grid(const gbc_hex_mesh* ma, MMGrid& g);
// mantle-mantle: rows (k*ne + j), cols (p*ne + i), row-major with leading dim ld; with a grid, one
// evaluation per distinct (offset, layers) key
int launch_gf_mm(const HexDev& m, double lambda, double mu, const double* qc, const double* qw,
                 int nq, double* out, size_t ld, cudaStream_t s, const MMGrid* grid = nullptr);

}  // namespace gbc
