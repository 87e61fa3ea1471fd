/*
 * kwg.h -- C ABI of the GB300 batched finite-difference American-option pricer.
 *
 * This is the drop-in boundary for the FD1D solve of gituliar/kwinto-cuda.  The
 * reference exposes it as the C++ interface
 *     kw::Pricer::init(const Config&)                                src/Pricer/kwPricer.h:14-16
 *     kw::Pricer::price(const vector<Option>&, vector<double>&)      src/Pricer/kwPricer.h:18-20
 *     kw::PricerFactory::create(config, pricer)  (PRICER=FD1D)       src/Pricer/kwPricerFactory.h:15-41
 * over the solver
 *     kw::Fd1d::solve / kw::Fd1d::value                              src/Math/kwFd1d.h:49-52
 * Every entry point below takes plain pointers and sizes; errors are returned as an
 * int status (0 = success) with the message in kwg_last_error(), the C form of the
 * reference's kw::Error string (src/Core/kwTypes.h:15, empty = OK).
 *
 * Threading: a kwg_ctx owns device buffers and one CUDA stream; like a reference
 * pricer object (src/Pricer/kwFd1d.h:22-30) it is stateful and not re-entrant --
 * use one context per calling thread.
 */
#ifndef KWG_H
#define KWG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- return codes ---------------------------------------------------------------- */
#define KWG_OK 0
#define KWG_ERR_INVALID 1     /* bad argument (null pointer, grid too small, theta out of range) */
#define KWG_ERR_CUDA 2        /* a CUDA call failed; message has the CUDA error string */
#define KWG_ERR_OUT_OF_GRID 3 /* strict mode: an asset's log(s/k) lies outside its x-grid */
#define KWG_ERR_SOLVER 4      /* strict mode: a tridiagonal pivot was zero or not finite */

/* ---- per-option status (status[i]) --------------------------------------------------- */
#define KWG_STATUS_OK 0
#define KWG_STATUS_OUT_OF_GRID 1 /* price is NaN; the reference fails the whole batch here */
#define KWG_STATUS_SOLVER 2      /* price is NaN; zero/non-finite pivot in the factorisation, or a non-finite
                                    value where the price is read (FP32: values beyond its range) */
#define KWG_STATUS_BAD_INPUT 3   /* price is NaN; t<=0, z<=0, k<=0 or s<=0 */
#define KWG_STATUS_DEVICE_TIMEOUT 4 /* price is NaN; a bounded device-side wait expired */

/* ---- numeric modes ------------------------------------------------------------------- */
#define KWG_FP64 0 /* all stepping in FP64: parity with the reference to <= 1e-10 relative */
#define KWG_FP32 1 /* FP32 stepping: FP64 setup and interpolation, float-float state and residual */

#define KWG_SOLVER_AUTO 0   /* the autotuned choice for this shape, else a cost model */
#define KWG_SOLVER_THOMAS 1 /* FP64: thread per option, option-interleaved streaming layout */
#define KWG_SOLVER_PCR 2    /* warp per option, partitioned solve with warp-shuffle cyclic
                               reduction, state on chip (FP64: x_dim <= 1024; FP32: <= 2048) */

/* Same field order, types and 56-byte layout as kw::Option (src/Core/kwAsset.h:12-22). */
typedef struct kwg_option {
    double t; /* time to maturity, years          */
    double k; /* strike                           */
    double z; /* volatility                       */
    double r; /* interest rate                    */
    double q; /* dividend rate                    */
    double s; /* spot                             */
    uint8_t e; /* early exercise: 0 European, 1 American */
    int8_t w;  /* -1 put, +1 call                 */
} kwg_option;

/* The FD1D.* config keys of the reference (src/Pricer/kwFd1d.cpp:12-16) plus the
 * GPU knobs.  Defaults (kwg_fd1d_params_default) are the reference defaults. */
typedef struct kwg_fd1d_params {
    int32_t t_dim;     /* FD1D.T_GRID_SIZE, default 512 (>= 2) */
    int32_t x_dim;     /* FD1D.X_GRID_SIZE, default 512 (>= 3) */
    double theta;      /* theta of the scheme, default 0.5 (the reference hard-codes it,
                          src/Math/kwFd1d.h:31); any value in (0, 1]        */
    double scale;      /* FD1D.SCALE, default 50: half-width scale*z*sqrt(t) */
    double density;    /* FD1D.DENSITY, default 0.25; +INFINITY = uniform grid (the
                          density -> infinity limit of the sinh grid)        */
    int32_t precision; /* KWG_FP64 (default) or KWG_FP32 */
    int32_t solver;    /* KWG_SOLVER_AUTO (default), _THOMAS or _PCR */
    int32_t strict;    /* blocking host calls (kwg_fd1d_price, kwg_fd1d_bs_price,
                          kwg_fd1d_price_uneven): 1 returns an error for the first
                          bad option, like the reference
                          (src/Pricer/kwFd1d.cpp:154-155); 0 (default): per-option
                          status and NaN, the batch still succeeds.  The
                          asynchronous device calls reject 1 (KWG_ERR_INVALID): their
                          caller reads d_status */
    int32_t device_dedup; /* kwg_fd1d_price_device only: 1 deduplicates the options on
                          the device by (t,r,q,z,e,w) like the host path (one stream
                          synchronisation reads the PDE count); 0 (default) solves every
                          option as its own PDE, fully asynchronously */
    int32_t block_warps;  /* FP64 streaming solver: warps (32 options each) per thread
                             block, 1, 2 or 4; 0 (default) = tuned or 1 */
    int32_t option_warps; /* warp-per-PDE FP32 solver: warps (32 threads each) per
                             option, 1, 2, 4 or 8 (grids of more than 1024 nodes at
                             least 2; at least 2 nodes per lane); 0 (default) = tuned or 1 */
    int32_t sm_blocks;    /* FP64 streaming solver: resident blocks per SM, 0 (default) =
                             tuned or as many as fit (two 4-warp blocks).  With
                             block_warps 4 and sm_blocks 1 each of an SM's four warp
                             schedulers runs one tile, whose FP64 pipe it then has to
                             itself: it shortens the longest tiles of an uneven batch */
} kwg_fd1d_params;

typedef struct kwg_ctx kwg_ctx;

/* Fills p with the reference defaults (src/Pricer/kwFd1d.cpp:12-16, kwFd1d.h:31). */
void kwg_fd1d_params_default(kwg_fd1d_params* p);

/* The grouping of options into PDEs that every pricing call uses
 * (src/Pricer/kwFd1d.cpp:28-65): options with equal (t, r, q, z, e, w) -- and, when
 * x_dims and t_dims are given (uneven batches), equal grid shape -- share one PDE.
 * Writes asset2pde[n] (each option's PDE; PDEs are numbered in order of their first
 * option) and, unless pde2asset is NULL, pde2asset[m] (each PDE's first option; room
 * for n entries); returns m.  Keys compare by value (+0 == -0); a NaN field matches
 * nothing, so such an option keeps its own PDE.  Host only: no context, no GPU.
 * O(n) (the reference sorts, O(n log n)). */
size_t kwg_fd1d_dedup(const kwg_option* opts, const int32_t* x_dims, const int32_t* t_dims, size_t n,
                      int32_t* asset2pde, uint32_t* pde2asset);

/* Creates a context on CUDA device `device`; NULL on failure (no GPU, bad id). */
kwg_ctx* kwg_create(int device);
void kwg_destroy(kwg_ctx* ctx);

/* Message of the last failed call on ctx ("" if it succeeded). */
const char* kwg_last_error(const kwg_ctx* ctx);

/* Prices n options given in HOST memory; writes n prices (and, if status is not
 * NULL, n per-option status codes) to HOST memory.  Blocking.
 * Replaces kw::Fd1d_Pricer::price (src/Pricer/kwFd1d.cpp:21-160): the options are
 * deduplicated by (t,r,q,z,e,w) on the host exactly like the reference
 * (src/Pricer/kwFd1d.cpp:28-65), one PDE is solved per distinct key on the GPU, and
 * prices[i] = k * V(log(s/k)) by linear interpolation (src/Math/kwFd1d.cpp:139-158).
 * n == 0 succeeds and writes nothing. */
int kwg_fd1d_price(kwg_ctx* ctx, const kwg_option* opts, size_t n, const kwg_fd1d_params* p,
                   double* prices, int32_t* status);

/* FD1D-BS control variate: prices[i] = FD(opts[i]) + BS(e) - FD(e), e = opts[i] with
 * European exercise, all FD prices on p's grid.  Replaces
 * kw::Fd1d_BlackScholes_Pricer::price (src/Pricer/kwFd1d_BlackScholes.cpp:15-42) and
 * its Black-Scholes leg (src/Pricer/kwBlackScholes.cpp:27-49).  The n options and
 * their European copies are deduplicated together and solved in one batch; the
 * combination runs on the GPU.  Status, strict mode and n == 0 as kwg_fd1d_price. */
int kwg_fd1d_bs_price(kwg_ctx* ctx, const kwg_option* opts, size_t n, const kwg_fd1d_params* p,
                      double* prices, int32_t* status);

/* Same computation with inputs and outputs already in DEVICE memory.  Asynchronous
 * on `stream` (a cudaStream_t; NULL = the context's stream).  For callers that keep
 * portfolios resident in HBM.  Without p->device_dedup every option is solved as its
 * own PDE; with it the options are deduplicated on the device (hash table on the key
 * of src/Pricer/kwFd1d.cpp:28-65; the call then waits once for the PDE count).
 * Per-option results are in d_status; p->strict = 1 is rejected (KWG_ERR_INVALID).
 * Replaces kw::Fd1d::solve + kw::Fd1d::value (src/Math/kwFd1d.cpp:11-58, 139-158). */
int kwg_fd1d_price_device(kwg_ctx* ctx, const kwg_option* d_opts, size_t n,
                          const kwg_fd1d_params* p, double* d_prices, int32_t* d_status,
                          void* stream);

/* No counterpart in the reference.  The FP64 device call for callers that cannot
 * allocate device memory -- for example a pricing step inside a host application
 * whose device memory belongs to another allocator or is held to a fixed budget, or
 * a latency-critical path where cudaMalloc's implicit synchronisation is not allowed.
 * It needs no context and allocates nothing: all scratch is one 64 MiB __device__
 * array inside the library (about 80 bytes per option and grid node: roughly 800
 * options at x_dim 1024), held by every GPU that loads the library until the process
 * exits.  Larger batches are rejected with KWG_ERR_INVALID and a message.
 * It always runs the streaming Thomas solver (solver AUTO or THOMAS; PCR is
 * rejected) and solves every option as its own PDE, so its prices are bit-identical
 * to kwg_fd1d_price_device's with solver THOMAS, and equal to the FP64 parity
 * tolerance otherwise.  block_warps and sm_blocks apply as there; option_warps (an
 * FP32 knob) is ignored; strict = 1 and device_dedup = 1 are rejected: read d_status.
 * Set-up: the first call on a device looks up the array's address with that device
 * current and caches it with the device's context id; a call that finds another
 * context (after a device reset) or none current on its thread repeats the look-up.
 * Make the first call on each device, and from each host thread, before any stream
 * capture.  Calls share the array: calls that overlap on the GPU race, so serialise
 * them.  `stream` is a cudaStream_t (NULL = the legacy default stream); `err` (may
 * be NULL) receives the error message.  Asynchronous like kwg_fd1d_price_device. */
int kwg_fd1d_price_device_static(const kwg_option* d_opts, size_t n, const kwg_fd1d_params* p,
                                 double* d_prices, int32_t* d_status, void* stream, char* err,
                                 size_t errlen);

/* Prices n options in HOST memory, option i on its own grid of x_dims[i] nodes and
 * t_dims[i] time levels (p's x_dim and t_dim are ignored; its other fields apply).
 * The reference prices one grid shape per Fd1d_Pricer::init
 * (src/Pricer/kwFd1d.cpp:15-16), so a mixed portfolio needs one reference call per
 * shape; here the whole batch is one persistent launch (FP64 Thomas) or one launch
 * per nodes-per-lane bucket (PCR and FP32), replayed from a CUDA graph while the
 * batch layout is unchanged.  Dedup key: (t, r, q, z, e, w, x_dim, t_dim).
 * Results and status as kwg_fd1d_price.  Blocking. */
int kwg_fd1d_price_uneven(kwg_ctx* ctx, const kwg_option* opts, const int32_t* x_dims,
                          const int32_t* t_dims, size_t n, const kwg_fd1d_params* p,
                          double* prices, int32_t* status);

/* Result of the autotuner: the launch shape it picked and the solve-kernel time of
 * every candidate (-1: not timed or not applicable). */
typedef struct kwg_tuning {
    int32_t solver;       /* KWG_SOLVER_THOMAS or KWG_SOLVER_PCR (FP64); KWG_SOLVER_PCR (FP32) */
    int32_t block_warps;  /* warps (32 options each) per block of the streaming FP64 solver */
    int32_t option_warps; /* warps (32 threads each) per option of the FP32 solver */
    int32_t sm_blocks;    /* resident blocks per SM of the streaming FP64 solver (0: as many as fit) */
    double thomas_ms[3];  /* streaming FP64 solver with 1, 2, 4 warps per block */
    double pcr_ms;        /* FP64 warp-per-PDE solver */
    double fp32_ms[3];    /* FP32 solver with 1, 2, 4 warps per option (the launch may
                             use fewer: at least 2 nodes per lane, and at least 2 warps
                             for grids of more than 1024 nodes) */
    double spread_ms;     /* streaming FP64 solver, 4 warps per block, one block per SM */
    double fp32_8w_ms;    /* FP32 solver with 8 warps per option (same caveat) */
} kwg_tuning;

/* Autotuner (no counterpart in the reference): on a synthetic batch of m options of
 * p's shape and precision, times options-per-block (1, 2, 4 warps of 32 per block, and
 * one 4-warp block per SM) and Thomas vs PCR for FP64, threads-per-option (1, 2, 4 or 8 warps) for FP32, and records
 * the fastest for later calls of that shape whose p leaves the choices at 0 / AUTO.
 * `out` may be NULL. */
int kwg_autotune_ex(kwg_ctx* ctx, const kwg_fd1d_params* p, size_t m, kwg_tuning* out);

/* The same for an uneven batch (kwg_fd1d_price_uneven's arguments): times the
 * candidates on these options and records the fastest for uneven calls of p's
 * precision and this batch size. */
int kwg_autotune_uneven(kwg_ctx* ctx, const kwg_option* opts, const int32_t* x_dims, const int32_t* t_dims,
                        size_t n, const kwg_fd1d_params* p, kwg_tuning* out);

/* Compact form of kwg_autotune_ex for FP64: tunes and records the same choices and
 * writes the best streaming (Thomas) solve time over the block sizes and residencies and the
 * warp-per-PDE (PCR) solve time (ms; negative if not applicable).  The choice is kept
 * for calls of the same shape (precision, x_dim, t_dim, m rounded to a power of two)
 * on this context.  No counterpart in the reference, which has one CPU solver. */
int kwg_autotune(kwg_ctx* ctx, const kwg_fd1d_params* p, size_t m, double* thomas_ms, double* pcr_ms);

/* Tensor-core GEMM used by the MLP surrogate: C[m][n] = sum_k A[m][k] B[n][k] with
 * A, B row-major BF16 in device memory and C row-major FP32, computed by tcgen05
 * MMAs with an FP32 accumulator in tensor memory.  k must be a multiple of 64.
 * Asynchronous on `stream` (a cudaStream_t; NULL = legacy default stream).
 * No counterpart in the reference. */
int kwg_gemm_bf16(const void* d_a, const void* d_b, float* d_c, int m, int n, int k, void* stream);

/* ---- learned surrogate ------------------------------------------------------------
 * No counterpart in the reference (it has no learned component).  An MLP
 * 5 -> 128 -> 128 -> 128 -> 128 -> 1 with SiLU, BF16 weights and FP32 accumulation on
 * the tcgen05 tensor cores maps (log K/S, vol sqrt T, r T, q T, put/call), normalised
 * by a training box, to the early-exercise premium over an analytic base:
 * (FD American price - base)/K, base = the Barone-Adesi-Whaley quadratic
 * approximation.  Price = max(intrinsic, base + K * premium).  Trained on FD prices.
 * Layer inputs enter the tensor cores as BF16 pairs (hi + lo, a 16-bit mantissa:
 * plain BF16 inputs would move log K/S by ~4e-4 and the price by ~0.02); the
 * 128 -> 1 output layer is an FP32 dot product with BF16 weights. */
typedef struct kwg_mlp kwg_mlp;

/* Parameters: 5 weight matrices of 128 x 128 (row-major [out][in]; the first layer
 * uses inputs 0..4, the output layer row 0) followed by 5 bias vectors of 128. */
#define KWG_MLP_PARAMS (5 * 128 * 128 + 5 * 128)

typedef struct kwg_audit {
    int64_t audited;       /* options priced by both the network and FD */
    int64_t out_of_box;    /* options outside the training box, priced by FD */
    double audit_abs_max;  /* max |network - FD| over the audited options */
    double audit_abs_sum;
} kwg_audit;

kwg_mlp* kwg_mlp_create(int device, uint64_t seed); /* He-uniform initial weights */
void kwg_mlp_destroy(kwg_mlp* h);
const char* kwg_mlp_last_error(const kwg_mlp* h);
/* box_lo/box_hi (5 each, raw feature units) may be NULL to keep the current box. */
int kwg_mlp_set_params(kwg_mlp* h, const float* params, const double* box_lo, const double* box_hi,
                       float y_scale);
int kwg_mlp_get_params(kwg_mlp* h, float* params, double* box_lo, double* box_hi, float* y_scale);
/* Device features [n][5] (normalised, FP32) -> n outputs (the scaled premium). */
int kwg_mlp_forward(kwg_mlp* h, const float* d_x, int n, float* d_y);
/* One forward + backward of the loss mean(e^2) on n rows: e = y - t, except where
 * d_floor[i] > -1e30 (an early-exercise row, whose price is the intrinsic value):
 * there e = max(0, y - floor).  d_floor may be NULL (no floors).  Gradients of all
 * KWG_MLP_PARAMS parameters to d_grad (device), loss to *loss (host). */
int kwg_mlp_gradients(kwg_mlp* h, const float* d_x, const float* d_t, const float* d_floor, int n, float* d_grad,
                      double* loss);
/* Device options -> device features [n][5] (FP32, normalised by the training box),
 * in-box flags and analytic base prices (any output may be NULL): the Barone-Adesi-
 * Whaley approximation for American options, Black-Scholes for European ones. */
int kwg_mlp_featurize(kwg_mlp* h, const kwg_option* d_opts, int n, float* d_x, uint8_t* d_inside, double* d_base);
/* Trains on device options with their FD prices (device): premium targets scaled to
 * unit standard deviation, exercise-region floors, Adam with a cosine learning-rate
 * schedule, shuffled minibatches.  The network keeps the parameters of the epoch with
 * the lowest mean minibatch loss (the initial ones until an epoch's loss is finite);
 * an epoch whose mean loss is not finite or exceeds 3x that best returns to those
 * parameters with fresh Adam moments and halves the learning rate for the remaining
 * epochs.  *final_loss = the kept epoch's mean loss (the last epoch's when none was
 * finite). */
int kwg_mlp_train(kwg_mlp* h, const kwg_option* d_opts, const double* d_prices, int n, int epochs, int batch,
                  float lr, uint64_t seed, double* final_loss);
/* The last kwg_mlp_train run of h: copies min(epochs, cap) per-epoch mean losses to
 * losses, the kept epoch to *best_epoch (-1 if none) and the number of returns after
 * a loss spike to *restarts (either may be NULL); returns the epoch count, or -1 for
 * invalid arguments.  Host only, no device work. */
int kwg_mlp_train_history(kwg_mlp* h, double* losses, int cap, int* best_epoch, int* restarts);
/* Network prices of device options (no fallback): max(intrinsic, base + K *
 * premium) for American options; d_inside (may be NULL) flags options inside the
 * training box. */
int kwg_mlp_price_device(kwg_mlp* h, const kwg_option* d_opts, int n, double* d_prices, uint8_t* d_inside);
/* Surrogate pricing of host options: the network for options inside the training
 * box, the FD solver (fd's grid and precision) for options outside it and for a
 * seeded random audit fraction, whose network-vs-FD error is reported.  route[i]:
 * 0 network, 1 audited (FD price returned), 2 out of box (FD), 3 FD failed. */
int kwg_surrogate_price(kwg_ctx* ctx, kwg_mlp* h, const kwg_option* opts, size_t n, const kwg_fd1d_params* fd,
                        double audit_frac, uint64_t seed, double* prices, int32_t* route, kwg_audit* audit);

/* Self-test of the bounded device waits (no counterpart in the reference): one
 * kernel waits on an mbarrier that nothing arrives on and must give up after a few
 * thousand polls (*timed_out = 1), then waits on one it arrived on and must pass
 * (*completed = 1).  Nothing faults or hangs; the context stays usable. */
int kwg_selftest_waits(kwg_ctx* ctx, int32_t* timed_out, int32_t* completed);

/* Number of kernel launches the last pricing call made (for launch accounting). */
int kwg_last_launch_count(const kwg_ctx* ctx);

/* Kernel timing for roofline accounting.  With profiling on, every pricing call
 * records CUDA events around its solve kernel on the stream it launches on, and the
 * FP64 solve counts the bytes it reads and writes.  kwg_profile_read waits for
 * them, returns the summed solve-kernel time (ms), the number of launches and the
 * summed bytes since the last read (any output may be NULL), and starts a new
 * accumulation. */
int kwg_set_profiling(kwg_ctx* ctx, int enable);
int kwg_profile_read(kwg_ctx* ctx, double* solve_ms, int* solve_launches, double* solve_bytes);

#ifdef __cplusplus
}
#endif

#endif /* KWG_H */
