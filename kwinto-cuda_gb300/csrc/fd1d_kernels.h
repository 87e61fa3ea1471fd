// fd1d_kernels.h -- host-visible launch interface of the FD1D kernels (internal to
// libkwg.so; the public boundary is include/kwg.h).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace kwg {

constexpr int kTile = 32;  // PDEs per tile: one warp, one PDE per lane

// One PDE per distinct option key (t, r, q, z, e, w), structure-of-arrays in device
// memory; m PDEs, padded to m_pad = a multiple of 32 (padding lanes replicate PDE m-1).
struct PdeBatch {
    const double* t;
    const double* z;
    const double* r;
    const double* q;
    const int8_t* w;
    const uint8_t* e;
    int m;
    int m_pad;
};

// Assets to price: spot, strike and the PDE slot each one reads its value from.
struct AssetBatch {
    const double* s;
    const double* k;
    const int32_t* pde;
    int n;
};

// Thomas-kernel tile of an uneven batch: 32 PDE slots sharing one node count.
struct TileDesc {
    int n;          // nodes of every PDE in the tile
    int t_max;      // largest time-level count among the tile's PDEs
    long long off;  // offset of the tile's first node-lane (arrays hold node-lanes)
};

// Grid shape and scheme parameters shared by a batch.  A uniform batch uses x_dim
// and t_dim; an uneven batch gives every PDE slot its own node count (pde_x) and
// time levels (pde_t), and the layout of its work arrays (tiles for the Thomas
// kernel, row_off for the kernels that write one row of final values per PDE).
struct Fd1dShape {
    int x_dim;
    int t_dim;
    double theta;
    double c;  // (1 - theta) / theta
    double scale;
    double density;
    bool uniform;
    const int32_t* pde_x = nullptr;
    const int32_t* pde_t = nullptr;
    const TileDesc* tiles = nullptr;
    const long long* row_off = nullptr;
    long long node_lanes = 0;  // Thomas work arrays: sum over tiles of 32 * n
    // per-PDE shapes only: every PDE of the launch has x_dim == 32 x its nodes per
    // lane (no padded nodes), which the warp-per-PDE uniform-grid kernels require
    bool full_lanes = false;
    // resolved launch shapes: warps per block of the streaming FP64 solver (1, 2, 4;
    // 32 options each) and warps per option of the FP32 solver (1, 2)
    int block_warps = 1;
    int option_warps = 1;
    int sm_blocks = 0;  // FP64 streaming solver: resident blocks per SM (0: as many as fit)
    int keep_nodes = 0;  // FP64 streaming solver: nodes at each sweep's end stored evict-last in L2 (set by the launch)
    // FP64 streaming solver, uniform batches: tiles [0, twin_tiles) hold 16 twin pairs
    // each -- an American PDE in the even lane, its European copy (same t, r, q, z, w)
    // in the odd lane -- which read one shared record of coefficients and payoff
    int twin_tiles = 0;
};

__host__ __device__ inline int shape_x(const Fd1dShape& sh, int pde) { return sh.pde_x ? sh.pde_x[pde] : sh.x_dim; }
__host__ __device__ inline int shape_t(const Fd1dShape& sh, int pde) { return sh.pde_t ? sh.pde_t[pde] : sh.t_dim; }
__host__ __device__ inline long long shape_row(const Fd1dShape& sh, int pde)
{
    return sh.row_off ? sh.row_off[pde] : (long long)pde * sh.x_dim;
}

// Device bytes of the FP64 Thomas work arrays of a uniform batch (coefficients +
// state), and of an uneven batch with the given node-lane count.
size_t fd1d_fp64_work_bytes(int m_pad, int x_dim);
size_t fd1d_fp64_work_bytes_nl(int m_pad, long long node_lanes);

// Optional CUDA events recorded immediately before and after the solve kernel.
struct SolveEvents {
    cudaEvent_t start = nullptr, stop = nullptr;
    unsigned long long* bytes = nullptr;  // pinned host slot for the launch's byte count
};

// Launches setup, solve and interpolation on `stream`; returns the launch count.
// counters: 4 ints, [0] tile queue, [1] device-timeout flag, [2..3] a 64-bit count
// of the bytes the solve reads and writes (all zeroed here).
int fd1d_fp64_launch(const PdeBatch& b, const AssetBatch& a, const Fd1dShape& sh, double* rec, int32_t* pde_status,
                     int* counters, double* prices, int32_t* status, int solve_blocks, cudaStream_t stream,
                     const SolveEvents* ev);

// FP32 stepping (one, two, four or eight warps per PDE, on chip; sh.option_warps).  Nodes per
// lane M of the one-warp layout for an x-grid of x_dim nodes (the grid is padded to
// 32*M with decoupled identity rows; W warps take M/W each); -1 if x_dim > 2048.
// The work buffer holds the final V of every PDE, [m][x_dim] doubles.
int fd1d_fp32_nodes_per_lane(int x_dim);
size_t fd1d_fp32_work_bytes(int m, int x_dim);
int fd1d_fp32_launch(const PdeBatch& b, const AssetBatch& a, const Fd1dShape& sh, double* vout, int32_t* pde_status,
                     int* counters, double* prices, int32_t* status, int device, cudaStream_t stream,
                     const SolveEvents* ev);

// FP64 warp-per-PDE on-chip solve (x_dim <= 1024).  Same work buffer as FP32.
int fd1d_pcr64_nodes_per_lane(int x_dim);
int fd1d_pcr64_launch(const PdeBatch& b, const AssetBatch& a, const Fd1dShape& sh, double* vout, int32_t* pde_status,
                      int* counters, double* prices, int32_t* status, int device, cudaStream_t stream,
                      const SolveEvents* ev);

// Device options (56-byte kw::Option records) -> the SoA arrays of a PdeBatch and
// an AssetBatch, every option its own PDE, the PDEs grouped by exercise / put-call
// class (European puts, European calls, American puts, American calls) so that the
// streaming FP64 solver's tiles are homogeneous; the slot order inside a class is
// arrival order.  counts: 8 ints (per-class counts, cursors), zeroed here on
// `stream`.  Two launches; returns the first CUDA error.
cudaError_t unpack_by_class(const void* d_opts, int n, int* counts, double* t, double* z, double* r, double* q,
                            double* s, double* k, int32_t* pde, int8_t* w, uint8_t* e, cudaStream_t stream);

// Interpolation over a [m][x_dim] array of final values (FP32 and PCR paths).
__global__ void fd1d_interp_rows(const PdeBatch b, const AssetBatch a, Fd1dShape sh, const double* __restrict__ vrow,
                                 const int32_t* __restrict__ pde_status, double* __restrict__ prices,
                                 int32_t* __restrict__ status);

// One-time per-device set-up of every kernel's shared-memory limit and occupancy, so
// that launches (also inside a stream capture) make no attribute calls.  Safe to call
// from several threads: the first call for a device does the work under a lock, later
// ones return after one atomic load.  fd1d_fp32_prepare and fd1d_pcr64_prepare run
// only inside it.
void fd1d_prepare_kernels(int device);
void fd1d_fp32_prepare(int device);
void fd1d_pcr64_prepare(int device);

// Occupancy-derived persistent grid size (blocks of block_warps warps) for the FP64
// solve kernel.
int fd1d_fp64_solve_blocks(int ntiles, int device, int block_warps = 1, int sm_blocks = 0);

}  // namespace kwg
