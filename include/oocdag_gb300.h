/*
 * oocdag_gb300 -- GB300 (sm_103a) out-of-core left-looking tiled Cholesky.
 *
 * C-ABI of the library.  Plain pointers and sizes only; every entry point returns an
 * int status (OOC_OK = 0, negative = error) unless stated otherwise.  Matrices are
 * column-major; only the lower triangle is read and written ('L').
 *
 * Each entry point names the reference interface it replaces (paths relative to the
 * efdazedo/oocdag project).
 */
#ifndef OOCDAG_GB300_H
#define OOCDAG_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------------ */
/* -1 .. -99: the k-th argument is invalid (LAPACK convention, -k).                 */
#define OOC_OK 0
#define OOC_ERR_NOMEM (-101)     /* device or pinned-host allocation failed          */
#define OOC_ERR_CUDA (-102)      /* a CUDA call failed; see ooc_last_error_string()  */
#define OOC_ERR_TIMEOUT (-103)   /* a bounded host wait on the device ran out        */
#define OOC_ERR_BUDGET (-104)    /* device budget too small for one panel column     */
#define OOC_ERR_INTERNAL (-105)  /* internal limit exceeded                          */
#define OOC_ERR_NODEVICE (-106)  /* no CUDA device / device index out of range       */
#define OOC_ERR_UNSUPPORTED (-107)

typedef struct ooc_handle ooc_handle;

/* Statistics of one factorization (filled when the caller passes a non-NULL pointer). */
typedef struct ooc_stats {
  double seconds;          /* factorization wall time (allocation excluded, as
                              oocdag.cpp:41,51,90 measures it)                       */
  double flops;            /* n^3/3                                                  */
  double h2d_bytes;        /* host -> device bytes scheduled                         */
  double d2h_bytes;        /* device -> host bytes scheduled                         */
  int npanels;             /* left-looking panels (1 = in-core)                     */
  int info;                /* LAPACK info                                           */
  int64_t kernel_launches; /* kernels launched by the library for this call         */
  /* Per-kernel device time, recorded with CUDA events on the compute stream when
     OOC_OPT_PROFILE is set (0 otherwise).                                          */
  double update_ms;        /* panel-update (syrk+gemm) kernels                       */
  int64_t update_launches;
  double update_flops;     /* algorithmic flops of those launches                    */
  double factor_ms;        /* diagonal factor + column solve                         */
  double h2d_ms;           /* host-to-device copies of a streamed host matrix: first
                              copy's start to last copy's end on the copy stream
                              (OOC_OPT_PROFILE; 0 otherwise)                        */
} ooc_stats;

/* Options (ooc_set_option). */
enum {
  OOC_OPT_X_BUFFERS = 1,   /* 1 = the reference's single X buffer, 2 = double-buffered
                              X (default 2; copy of column k+1 overlaps update k)    */
  OOC_OPT_TIMEOUT_MS = 2,  /* bound on every host wait for the device (default 6 h)  */
  OOC_OPT_PROFILE = 3,     /* 1 = time kernels with CUDA events into ooc_stats       */
  OOC_OPT_PIN_HOST = 4,    /* 1 = page-lock a pageable host matrix for the call
                              (cudaHostRegister; default 1)                          */
  OOC_OPT_REF_SCHEDULE = 5, /* 1 = panel widths exactly as oocdag.cpp:478-492 with one
                              X buffer counted (default 0: two X buffers counted)     */
  OOC_OPT_KEEP_A = 6,      /* 1 = a reduced-precision factor created from a HOST matrix
                              keeps the FP64 lower triangle it copied to the device
                              (8 n^2 more device bytes), and ooc_solve_refine given the
                              same host pointer and lda uses it instead of copying A
                              again (default 0)                                       */
  OOC_OPT_TAIL_ORDER = 7,  /* split-BF16 factors with nb a multiple of 256: the last
                              panels, from the first multiple of nb at or after order
                              n - value, are nb/2 wide (their one-CTA diagonal tiles are
                              ~3x cheaper where the trailing update no longer hides
                              them); 0 = uniform nb-wide panels.  Default 24576.      */
  OOC_OPT_POOL_BYTES = 8,  /* device bytes the handle may keep cached from destroyed
                              factor objects for reuse by later ones of the same sizes
                              (freeing multi-GB buffers costs ~0.4 ms per GB and
                              synchronises the device); released by ooc_destroy, or when
                              an allocation fails.  Default 40 % of device memory, 0 =
                              no caching.                                             */
  OOC_OPT_BLOCK_COLS = 9,  /* split-BF16 factors of a stored matrix (nb a multiple of
                              128): width, in columns (rounded up to whole panels), of the
                              left-looking column blocks.  A block is caught up with every
                              finished panel by long-K tensor-core updates, then factored
                              right-looking inside itself in nb/2-wide panels; for a
                              page-locked host matrix each block is copied to the device
                              while earlier ones are factored (the reference's panel
                              streaming, oocdag.cpp:59-87).  0 = right-looking over the
                              whole matrix (a host matrix is copied first); -1 (default)
                              = 4096 for device and page-locked host matrices with
                              n > 8192, 0 otherwise.  Needs a plane store of 4 n^2
                              device bytes while the factor is computed.              */
  OOC_OPT_COPY_STREAMS = 10 /* host-to-device streams that a host matrix streamed into a
                              split-BF16 factor with a kept copy alternates its column
                              chunks over (1 or 2; default 2): two copy engines in
                              flight on the group of columns needed next             */
};

/* Handles: one per thread of control; reentrant across handles. */
int ooc_create(ooc_handle** h, int device);
int ooc_destroy(ooc_handle* h);
int ooc_set_option(ooc_handle* h, int key, int64_t value);
int ooc_get_option(ooc_handle* h, int key, int64_t* value);
const char* ooc_last_error_string(void);
/* LAPACK info of the last factorization run on the handle. */
int ooc_last_info(ooc_handle* h);
/* The handle's CUDA streams (which: 0 = compute, 1 = host-to-device copies,
 * 2 = device-to-host copies, 3 = a second host-to-device copy stream that streamed host
 * matrices use beside the first), as a cudaStream_t, so that a caller can order its own
 * work or timing events against the library's.
 * Device-pointer arguments are read on these streams (compute and host-to-device)
 * from the moment of the call: data still being produced on another stream must be
 * finished, or those two streams made to wait for it (cudaStreamWaitEvent), before
 * the call.  Every call returns after its own work on the device is done.           */
int ooc_get_stream(ooc_handle* h, int which, void** stream);

/* Lower Cholesky A = L L^T in place, out of core.
 * Replaces: double Cholesky(Quark*, double *A, int N, int NB, int LDA, size_t memsize)
 *           (oocdag.cpp:18-112) together with its task generators A2Y/A2X/ooc_syrk/
 *           ooc_incore (oocquark.cpp:253-421, prototypes oocdag.h:119-123).
 * A: host memory (pageable or pinned; streamed through a device budget of dev_budget
 *    bytes) or device memory (factored in place, in core).  Upper triangle untouched.
 * *info: 0, or k > 0 if the leading minor of order k is not positive definite.      */
int ooc_dpotrf_L(ooc_handle* h, double* A, int64_t n, int64_t lda, int nb, size_t dev_budget,
                 int* info, ooc_stats* stats);

/* FP32 Cholesky A = L L^T in place (lower; upper triangle untouched).  The reference has
 * no FP32 entry (LIN/psmatgen.f exists but nothing binds it).  A on the device: factored
 * in place (FP32 diagonal tiles, column solves and FP32 trailing updates, nb <= 512).
 * A on the host: on a device copy when it fits dev_budget bytes (0 = 3/4 of free device
 * memory); otherwise out of core, left-looking over panels of W columns with
 * 3 n W floats <= dev_budget (the panel and two buffers of earlier columns streamed from
 * the host, oocdag.cpp:59-87), OOC_ERR_BUDGET if not even W = nb fits.
 * *info as for ooc_dpotrf_L.                                                          */
int ooc_spotrf_L(ooc_handle* h, float* A, int64_t n, int64_t lda, int nb, size_t dev_budget,
                 int* info, ooc_stats* stats);

/* B := A^{-1} B with the lower factor L of A as ooc_dpotrf_L leaves it, host or device
 * (ld ldl): the reference's VERIFY solve, dpotrs on the factored matrix
 * (oocdag.cpp:436-439).  A host L is streamed through the device twice (forward and
 * backward sweeps over nb-wide column panels, two panel buffers of n x nb doubles);
 * dev_budget (0 = no limit) caps the device bytes, else OOC_ERR_BUDGET.  B: host or
 * device, n x nrhs (ld ldb), nrhs <= 16, overwritten by the solution.                 */
int ooc_dpotrs_L(ooc_handle* h, const double* L, int64_t n, int64_t ldl, int nb, size_t dev_budget, double* B,
                 int64_t ldb, int nrhs);

/* Drop-in for the reference driver entry (oocdag.cpp:18): same argument order, the
 * QUARK context replaced by an ooc_handle (NULL = a per-process handle on the current
 * device).  Returns the factorization time in seconds, or a negative status code.  */
double Cholesky(void* handle, double* A, int N, int NB, int LDA, size_t memsize);

/* ScaLAPACK-style entry (pdpotrf_ argument order) on a 1 x 1 process grid, as the
 * reference's test matrices are described (desc layout DTYPE_,CTXT_,M_,N_,MB_,NB_,
 * RSRC_,CSRC_,LLD_, LIN/pdpotrrv.f:118-120).  Only uplo = 'L'.  The tile size is
 * desca[5] (NB_), the leading dimension desca[8] (LLD_).  The device budget is the
 * OOC_DEVICE_BUDGET_MB environment variable, else 3/4 of free device memory.      */
void ooc_pdpotrf_(const char* uplo, const int* n, double* a, const int* ia, const int* ja,
                  const int* desca, int* info);

/* FP32 ScaLAPACK-style entry (pspotrf_ argument order, same descriptor and budget rules as
 * ooc_pdpotrf_): ooc_spotrf_L on the sub-matrix; a host matrix larger than the budget is
 * factored out of core.  No FP32 entry exists in the reference; this mirrors its
 * descriptor form for the single-precision ScaLAPACK routine.                         */
void ooc_pspotrf_(const char* uplo, const int* n, float* a, const int* ia, const int* ja, const int* desca,
                  int* info);

/* Panel plan of the left-looking loop: writes (jb, Ym, Yn) triples for an n x n matrix,
 * tile nb and a budget of memBlock tiles, counting nx X buffers (nx = 1 reproduces
 * find_Yn and the panel loop of oocdag.cpp:59-66,478-492).  Host only, no GPU.
 * Returns the number of panels, OOC_ERR_BUDGET, or -5 if cap triples do not suffice. */
int ooc_panel_plan(int64_t n, int nb, int64_t memBlock, int nx, int* out, int cap);

/* ---- mixed precision: factor once, solve with FP64 iterative refinement -------- */
/* Precision of the trailing syrk/gemm updates.  OOC_PREC_FP64 factors the diagonal
 * tiles (potrf and inverse) and solves the column panels in FP64.  The reduced-precision
 * factors work in an FP32 matrix: FP32 diagonal tiles; the column solve (a product with
 * the tile's inverse) in FP32 for OOC_PREC_FP32 and with the update's three BF16 tensor
 * products for OOC_PREC_BF16X3 (nb a multiple of 128).                               */
enum {
  OOC_PREC_FP64 = 0,  /* FP64 DMMA updates (the plain path)                        */
  OOC_PREC_FP32 = 1,  /* FP32 operands, FP32 FFMA accumulation                      */
  OOC_PREC_BF16X3 = 2 /* hi/lo BF16 splits, 3 tensor-core products, FP32 accumulate */
};

typedef struct ooc_factor ooc_factor;

/* Factor an SPD matrix in core (A: host or device, lower triangle read; A is not
 * modified) with trailing updates in `prec`; keeps L, the inverses of its diagonal
 * tiles and (for prec != FP64) FP32 copies for refinement.  No reference counterpart:
 * the reference only factors (oocdag.cpp:18) and checks with dpotrs (oocdag.cpp:439). */
int ooc_factor_create(ooc_handle* h, const double* A, int64_t n, int64_t lda, int nb, int prec,
                      ooc_factor** F, int* info, ooc_stats* stats);
int ooc_factor_destroy(ooc_factor* F);
/* Copy the factor (lower triangle = L; the upper triangle holds A's values) out.      */
int ooc_factor_copy_L(ooc_factor* F, double* L, int64_t ldl);
/* B := A^{-1} B with the factor (FP64 triangular solves), B on the device, nrhs <= 16.
 * The dpotrs of the reference's VERIFY block (oocdag.cpp:439).                       */
int ooc_factor_solve(ooc_handle* h, ooc_factor* F, double* B, int64_t ldb, int nrhs);
/* Solve A X = B by iterative refinement: X0 from the factor, then R = B - A X in FP64
 * with the original A, correction with the factor (FP32 copy for a reduced-precision
 * factor), until the normwise backward error ||R||_inf/(||A||_inf ||X||_inf + ||B||_inf)
 * <= tol or maxiter corrections.  A: device or host, lower triangle read (the residual
 * and the norm use A's symmetry; a host A is copied to the device, lower triangle only,
 * unless the factor kept it, OOC_OPT_KEEP_A).  B, X: device, nrhs <= 16.            */
int ooc_solve_refine(ooc_handle* h, ooc_factor* F, const double* A, int64_t lda, const double* B,
                     int64_t ldb, double* X, int64_t ldx, int nrhs, double tol, int maxiter, int* iters,
                     double* berr);

/* The same for the uniform test matrix A = (R + R^T)/2 + alpha I of seed `seed`
 * (ooc_dmatgen_uniform), generated straight into the factor's storage: no copy of A is
 * kept.  The refinement below regenerates A's elements inside its FP64 residual, so a
 * seeded system needs only the factor's memory (8 n^2 bytes, 12 n^2 for a reduced-
 * precision factor).                                                                 */
int ooc_factor_create_gen(ooc_handle* h, int64_t n, uint64_t seed, double alpha, int nb, int prec,
                          ooc_factor** F, int* info, ooc_stats* stats);
int ooc_solve_refine_gen(ooc_handle* h, ooc_factor* F, uint64_t seed, double alpha, const double* B,
                         int64_t ldb, double* X, int64_t ldx, int nrhs, double tol, int maxiter, int* iters,
                         double* berr);
/* Device bytes a factor object of order n, tile nb and precision prec holds.         */
int64_t ooc_factor_bytes(int64_t n, int nb, int prec);
/* B (n x nrhs, device) := N(0,1) samples of stream `seed` (Box-Muller on SplitMix64).  */
int ooc_gen_normal(ooc_handle* h, double* B, int64_t n, int64_t ldb, int nrhs, uint64_t seed);

/* C := C - A A^T on the lower triangle (device pointers; A n x k), with the trailing-
 * update kernel of precision `prec`: the dsyrk('L','N',-1,A,1,C) task body of the
 * reference (oocquark.cpp:176, cublasDsyrk_v2) as a tile call.                       */
int ooc_dsyrk_ln(ooc_handle* h, int prec, int n, int k, const double* A, int64_t lda, double* C,
                 int64_t ldc);

/* ---- batched small systems ---------------------------------------------------- */
/* Factor and solve `count` SPD systems (orders 1..512) in ONE persistent launch: matrix i
 * is column-major with ld = n[i] at element offset a_off[i] of A (device; its lower
 * triangle is replaced by L_i), its right-hand side at b_off[i] of B (device; replaced
 * by the solution).  info[i] (host) receives LAPACK info; a failed matrix is not solved.
 * blk_table (host, 16 entries, may be NULL): panel width per size bucket n/32, from
 * the autotuner.  ctas_per_sm: resident CTAs per SM (0 = occupancy limit).  *seconds:
 * kernel time.  The per-matrix work restates the reference's tile bodies at small n
 * (dpotrf oocquark.cpp:87, dtrsm :130, dsyrk/dgemm :176,222) and its dpotrs check
 * (oocdag.cpp:439).                                                                   */
int ooc_batched_dposv(ooc_handle* h, int count, const int* n, const int64_t* a_off, const int64_t* b_off,
                      double* A, double* B, int* info, const int* blk_table, int ctas_per_sm, double* seconds);
int ooc_batched_sposv(ooc_handle* h, int count, const int* n, const int64_t* a_off, const int64_t* b_off,
                      float* A, float* B, int* info, const int* blk_table, int ctas_per_sm, double* seconds);

/* ---- serving: continuous batching of factor + solve requests ------------------- */
/* A request loop with no counterpart in the reference (which factors one matrix per
 * process).  Requests are admitted in arrival order against a device-memory budget
 * (least-recently-used resident factors are evicted when nobody uses them); systems with
 * n <= small_max_n are gathered by a batcher into one persistent batched launch, larger
 * ones run on `workers` concurrent pipelines (own streams each) as a factor with
 * trailing updates in `prec` plus FP64 refinement to `tol`; factors stay resident under
 * the request's key for repeat solves.  Matrices are the uniform test matrices
 * (R + R^T)/2 + n I of the request's seed, right-hand sides N(0,1) of its rhs seed.    */
typedef struct ooc_server ooc_server;
typedef struct ooc_server_config {
  int device;
  int workers;             /* concurrent pipelines for the larger systems (default 4)     */
  int small_max_n;         /* n <= this goes to the batched kernel (<= 512, default 512)  */
  int nb;                  /* tile size of the larger systems (default 512)              */
  int prec;                /* OOC_PREC_* of their trailing updates                       */
  double tol;              /* backward-error target (default 1e-14)                      */
  double batch_window_ms;  /* the batcher waits this long for more small requests        */
  int64_t hbm_budget;      /* device bytes the server may hold (0 = 90% of free memory)  */
  int64_t ooc_min_n;       /* new factors of order >= this are computed out of core: FP64
                              ooc_dpotrf_L of a host-resident copy of the matrix through
                              ooc_budget device bytes, solved with ooc_dpotrs_L (completion
                              path 2), one at a time; <= 0 = never (every factor in HBM)  */
  int64_t ooc_budget;      /* device panel budget of those factorizations (0 = 24 GiB)    */
} ooc_server_config;
typedef struct ooc_request {
  int kind;                /* 0: factor + solve, 1: solve with the factor resident under key */
  int64_t n;
  uint64_t matrix_seed;
  uint64_t rhs_seed;
  int64_t key;
  int keep_solution;       /* 1: keep x until ooc_server_solution fetches it             */
} ooc_request;
typedef struct ooc_completion {
  int64_t id;
  int status;              /* OOC_OK or an error (OOC_ERR_BUDGET: never fits the budget) */
  int info;                /* LAPACK info                                                 */
  int path;                /* 0: batched kernel, 1: factor + refinement pipeline, 2: out
                              of core (host-resident factor)                             */
  int factor_reused;       /* 1: solved with a resident factor                            */
  int iterations;          /* refinement steps                                            */
  double backward_error;   /* ||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf)           */
  double t_submit, t_admit, t_done;  /* seconds on the server clock                       */
  double x_sum;            /* sum of the solution's entries                               */
} ooc_completion;
int ooc_server_create(const ooc_server_config* cfg, ooc_server** s);
int ooc_server_submit(ooc_server* s, const ooc_request* r, int64_t* id);
/* Up to `max` completions; waits up to wait_ms for the first one.                    */
int ooc_server_poll(ooc_server* s, ooc_completion* out, int max, int* count, int wait_ms);
int ooc_server_solution(ooc_server* s, int64_t id, double* x, int64_t n);
int ooc_server_status(ooc_server* s, int64_t* pending, int64_t* running, int64_t* resident_bytes,
                      int64_t* reserved_bytes);
double ooc_server_now(ooc_server* s);
/* Description of the last failed request (empty if none).                            */
const char* ooc_server_last_error(ooc_server* s);
int ooc_server_destroy(ooc_server* s);

/* Size of the device array that ooc_dpotrf_L_static uses as its panel buffer.      */
#define OOC_STATIC_PANEL_BYTES (64u << 20)

/* Out-of-core lower Cholesky that allocates nothing.  No counterpart in the reference.
 * For callers that cannot call cudaMalloc: processes whose device memory belongs to
 * another allocator (a framework's caching pool that has reserved the GPU, where a new
 * allocation fails or fragments it), and servers that must not let an allocation or a
 * free synchronize the device under their other streams.  The panel buffer and status
 * word live in the library's static device memory (OOC_STATIC_PANEL_BYTES, held by every
 * GPU that loads the library until exit); all work runs on `stream` (a cudaStream_t,
 * NULL = the legacy default stream).  A: host (pageable or page-locked) or device,
 * column-major, lower triangle factored in place as ooc_dpotrf_L does.
 * - Limit: the matrix must fit the reference's panel rule in OOC_STATIC_PANEL_BYTES with
 *   one X buffer: at least 2*ceil(n/nb) tiles of nb*nb doubles (n <= 16384 at nb = 256);
 *   larger sizes return OOC_ERR_BUDGET, before any device call, with a message in
 *   ooc_last_error_string().
 * - The first call on a device looks up the array's device address (set-up); make that
 *   first call before any stream capture.  The lookup is kept per device context, so it
 *   runs again after the device or its primary context has been reset.
 * - The call waits (bounded) until its work on `stream` has finished, then reads the
 *   status word, so it returns with A factored and *info set.
 * - Calls share the array: the status word is cleared at the start of each call; calls
 *   whose GPU work overlaps (e.g. two threads on two streams) race and must be
 *   serialized by the caller.                                                        */
int ooc_dpotrf_L_static(double* A, int64_t n, int64_t lda, int nb, void* stream, int* info);

/* ---- test matrices (the reference's generator, and the uniform generator) ------ */
/* pdmatgen('Symm','Diag') on a 1 x 1 grid (LIN/pdmatgen.f, called at oocdag.cpp:298-302):
 * A(i,j) = 1 - 2 u[min(i,j) n + max(i,j)], A(i,i) = |A(i,i)| + n, u from the 31-bit LCG
 * x <- 1103515245 x + 12345 mod 2^31 started at x0 = 1103515245 seed + 12345.
 * A: host or device.                                                               */
int ooc_dmatgen_pdmatgen(ooc_handle* h, double* A, int64_t n, int64_t lda, int seed);
/* A = (R + R^T)/2 + alpha I, R(i,j) = u - 1/2 with u the top 53 bits of SplitMix64
 * output number i + j n (state started at mix(seed)).  Exact in binary64.  No
 * reference counterpart (the uniform test matrix of the benchmark configurations).  */
int ooc_dmatgen_uniform(ooc_handle* h, double* A, int64_t n, int64_t lda, uint64_t seed,
                        double alpha);

/* Scaled residual ||A - L L^T||_F / (n eps ||A||_F), eps = 2^-53, with A regenerated
 * from its seed tile by tile (kind 0: uniform with alpha; kind 1: pdmatgen with seed)
 * as LIN/pdlaschk.f:238-250 regenerates it.  L: lower triangle, host or device.     */
int ooc_dresidual(ooc_handle* h, const double* L, int64_t n, int64_t lda, int kind, uint64_t seed,
                  double alpha, double* resid);

/* FP64 DMMA issue-rate probe: runs an MMA-only loop on every SM for about `ms`
 * milliseconds and returns the achieved FP64 tensor rate in TFLOP/s (the FP64 peak
 * used as the roofline denominator).  No reference counterpart.                     */
int ooc_fp64_peak_probe(ooc_handle* h, double ms, double* tflops);

#ifdef __cplusplus
}
#endif

#endif /* OOCDAG_GB300_H */
