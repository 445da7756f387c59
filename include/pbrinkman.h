/*
 * pbrinkman.h -- C ABI of the GB300 periodic regularized Brinkman evaluator.
 *
 * Plain pointers and sizes only.  Layouts follow the reference project
 * hoangngan82/periodicBrinkman: a "3 x N column-major matrix" is an array of N
 * xyz triples (cuda/periodicBrinkman.h:16-17); the mobility matrix A is
 * 3m x 3n column-major with the (r, c) entry of the block of target i and
 * source j at A[(3j + c) * 3m + 3i + r] (cuda/periodicBrinkman.h:304).
 *
 * Every function returns PB_OK (0) or a negative PB_ERR_* code;
 * pb_last_error() gives a one-line message for the calling thread.
 * Nothing falls back to the CPU: without a CUDA device every compute entry
 * point returns PB_ERR_CUDA.
 */
#ifndef PBRINKMAN_H
#define PBRINKMAN_H

#ifdef __cplusplus
extern "C" {
#endif

#define PB_OK 0
#define PB_ERR_INVALID -1     /* bad argument (sizes, NaN, L <= 0, alpha <= 0, ...) */
#define PB_ERR_CUDA -2        /* CUDA runtime error or no device */
#define PB_ERR_NOMEM -3       /* device allocation failed */
#define PB_ERR_UNSUPPORTED -4 /* valid but outside what this build supports */
#define PB_ERR_BUDGET -5      /* request exceeds the memory budget of a server */
#define PB_ERR_BUSY -6        /* server queue full */

/* precision */
#define PB_PREC_FP64 0  /* all FP64 ("plain"): reference closed forms, FP64 grids */
#define PB_PREC_MIXED 1 /* FP32 bulk: polynomial pair kernel, FP32 grids; FP64 series/self/sum */

/* flags */
#define PB_REAL_SPACE 1 /* real-space sum (incl. self term) */
#define PB_KSPACE 2     /* k-space sum (k != 0) */
#define PB_ZERO_MODE 4  /* add the k = 0 mean-flow mode  sum_j f_j / (alpha^2 tau) */
#define PB_FLAGS_DEFAULT (PB_REAL_SPACE | PB_KSPACE)

/* memory location of user buffers */
#define PB_HOST 0        /* host memory; the call returns when U is written (a non-finite
                            input is found on the device: PB_ERR_INVALID, U unspecified) */
#define PB_DEVICE 1      /* device memory; ordered on the given stream */
#define PB_HOST_PINNED 2 /* page-locked host memory; ordered on the given stream, no wait */

/* One solve: velocities at n_tgt targets induced by n_src point forces in the
 * periodic box L with Brinkman alpha (inverse permeability length) and blob
 * width eps (eps = 0: singular point forces).  Zero-valued tuning fields are
 * chosen by the autotuner from (n, L, tol). */
typedef struct pb_solve_params {
    int n_src;     /* number of point forces */
    int n_tgt;     /* number of targets; 0 = the targets are the sources */
    double L[3];   /* box */
    double alpha;  /* Brinkman alpha > 0 */
    double eps;    /* blob width >= 0 */
    double tol;    /* target max relative velocity error (autotuner); 0 -> 1e-6 */
    double d;      /* Ewald splitting blob width d = 1/xi; 0 = autotune */
    double rc;     /* real-space cutoff; 0 = autotune */
    int M[3];      /* FFT grid (powers of two >= 8); 0 = autotune */
    int P;         /* Gaussian support points per axis (even, 4..32); 0 = autotune */
    double m_std;  /* support half-width in Gaussian standard deviations; 0 = from tol */
    int precision; /* PB_PREC_FP64 or PB_PREC_MIXED */
    int flags;     /* PB_REAL_SPACE | PB_KSPACE | PB_ZERO_MODE; 0 = default */
} pb_solve_params;

/* Resolved parameters of one instance (d, rc, grid, support, cells). */
typedef struct pb_instance_info {
    double d, rc, eta, m_std;
    int M[3];
    int P;
    int ncell[3];
    int npoly;            /* polynomial terms of the FP32 pair kernel */
    long long pairs_est;  /* estimated real-space pairs inside rc */
} pb_instance_info;

/* Capacity of a serving slot: a plan whose instances are bound per use. */
typedef struct pb_slot_config {
    int M[3];          /* FFT grid of every instance bound to the slot */
    int max_instances; /* instances per execution */
    int max_src;       /* total sources over the bound instances */
    int max_tgt;       /* total targets (an instance whose targets are its sources counts n_src) */
    int max_cells;     /* total real-space cells over the bound instances */
    int precision;     /* PB_PREC_FP64 or PB_PREC_MIXED */
    int npoly;         /* terms of the FP32 far-piece polynomial (16..28; 0 = 18; longer fits are truncated) */
} pb_slot_config;

typedef struct pb_plan_s* pb_plan;

/* ---- reference-facing entry points ------------------------------------ */

/* Replaces periodicBrinkman(dA, dx, dx0, a, d, e, M, N, L, maxBlockSize)
 * (cuda/periodicBrinkman.h:432-513).  DEVICE pointers: dA (3m x 3n,
 * column-major) is ACCUMULATED into (A += real + k-space sums); dx is 3 x m
 * targets, dx0 is 3 x n sources; L has 3 entries (host).  Real images over
 * [-M,M]^3 and wave vectors over [-N,N]^3 \ {0}, both rescaled per axis from
 * the sorted box as the reference does (cuda/periodicBrinkman.h:457-487).
 * M < 0 skips the real part, N <= 0 skips the k part.  The k-space sum is
 * divided by tau = Lx Ly Lz like the reference's host twin fourierShells
 * (cuda/periodicBrinkman.h:745); the reference's GPU kernelFourier omits it,
 * the two agree for L = (1,1,1).  maxBlockSize must be > 0 (it tuned the
 * reference's block size; it has no effect here).  Runs on the current
 * stream 0 and synchronises before returning. */
int pb_periodic_brinkman(double* dA, const double* dx, int m, const double* dx0, int n, double a, double d,
                         double e, int M, int N, const double* L, int maxBlockSize);

/* As pb_periodic_brinkman with explicit per-axis shell counts Mx[3], Nx[3]
 * and tau_scaled = 0 to reproduce kernelFourier's missing 1/tau. */
int pb_periodic_brinkman_ex(double* dA, const double* dx, int m, const double* dx0, int n, double a, double d,
                            double e, const int* Mx, const int* Nx, const double* L, int tau_scaled, void* stream);

/* Replaces fftBrinkman(U, y, f, xn, L, M, P, m, C, e, tol, d, alpha)
 * (cuda/fftBrinkman.h:34-50).  HOST pointers: U (3 x m_tgt, overwritten),
 * y (3 x m_tgt targets), f (3 x n forces), xn (3 x n force locations),
 * L[3], grid M[3], support P[3] (P[0] used for all axes, as the reference's
 * eta uses P[0]), msd = support half-width in standard deviations, C unused
 * (as in the reference), e = blob width, tol only reported, d = splitting
 * blob width, alpha.  Computes, like the reference, the k-space part only
 * (k != 0), but with a centred support window, no conjugation of the scaled
 * spectrum (cuda/fftBrinkman.h:209-216) and a gather over each target's own
 * support instead of the whole grid (cuda/fftBrinkman.h:253-272). */
int pb_fft_brinkman(double* U, const double* y, int m_tgt, const double* f, const double* xn, int n,
                    const double* L, const int* M, const int* P, int msd, int C, double e, double tol, double d,
                    double alpha);

/* No counterpart in the reference.  pb_fft_brinkman's k-space velocities for
 * callers that cannot allocate device memory: code that runs where
 * cudaMalloc/cudaFree would block or synchronise the device (a real-time
 * loop), or a host program whose device memory is all owned by its own pool.
 * Same arguments and results as pb_fft_brinkman, minus C and tol, but U, y,
 * f and xn are DEVICE pointers and the work is queued on `stream` (NULL =
 * legacy default stream) without a synchronise.  Allocates nothing: all
 * intermediates live in one fixed array of 21.2 MB (20.2 MiB) compiled into the
 * library, which every GPU that loads the library holds until the process
 * exits.  Limits: M[a] <= 64, n <= 65536, m_tgt <= 65536; larger sizes return
 * PB_ERR_UNSUPPORTED.  Nothing is autotuned: M[a] and P[0] must be given
 * (> 0, else PB_ERR_INVALID).  The descriptor and twiddles travel as a
 * kernel launch parameter, so no host memory is read after the call
 * returns.  The first call on a device looks up the array's
 * device address for that device (make it before any stream capture).  All
 * calls share the array, so calls that overlap on the GPU race: serialise
 * them on one stream. */
int pb_fft_brinkman_static(double* U, const double* y, int m_tgt, const double* f, const double* xn, int n,
                           const double* L, const int* M, const int* P, int msd, double e, double d, double alpha,
                           void* stream);

/* Free-space (non-periodic) Brinkmanlet, the GPU counterpart of the
 * reference's Brinkmanlet() (cuda/periodicBrinkman.h:119-141): the
 * regularized R_eps of regH (53-78) for eps > 0, the singular S of singH
 * (31-46) for eps = 0.  Velocities U (3 x m) at targets y (3 x m) of forces
 * f (3 x n) at x (3 x n), overwritten; a direct FP64 sum (O(m n)).  where =
 * PB_HOST (copies in and out, synchronous) or PB_DEVICE (queued on stream).
 * With eps = 0 a coincident pair (r <= 1e-12) has no finite velocity and is
 * skipped. */
int pb_brinkmanlet(double* U, const double* y, int m, const double* x, const double* f, int n, double alpha,
                   double eps, int where, void* stream);
/* The dense form: dA (DEVICE, 3m x 3n column-major, the layout of
 * pb_periodic_brinkman) += the Brinkmanlet tensor of every (target, source)
 * pair, queued on stream.  A coincident singular pair gets singH's sentinel
 * 1.79e308 on its diagonal, as the reference's Brinkmanlet does. */
int pb_brinkmanlet_matrix(double* dA, const double* dx, int m, const double* dx0, int n, double alpha, double eps,
                          void* stream);

/* ---- evaluator ----------------------------------------------------------- */

/* One-shot solve.  x, f: 3 x n_src; y: 3 x n_tgt (NULL when n_tgt == 0);
 * U: 3 x n_tgt (or 3 x n_src), overwritten.  where = PB_HOST or PB_DEVICE for
 * all four buffers.  stream: cudaStream_t or NULL (default stream). */
int pb_solve(const pb_solve_params* p, const double* x, const double* f, const double* y, double* U, int where,
             void* stream);

/* A plan holds device buffers, kernel tables and FFT twiddles for `count`
 * instances solved together (a batch; count = 1 for a single solve).  Its
 * execution is captured into a CUDA graph on the second call and replayed. */
int pb_plan_create(const pb_solve_params* p, int count, pb_plan* out);
/* Packed inputs: instances back to back in the order of creation. */
int pb_plan_execute(pb_plan plan, const double* x, const double* f, const double* y, double* U, int where,
                    void* stream);
/* The same plan applied to new forces at the positions (and targets) of its
 * last successful pb_plan_execute: a matrix-free mobility product for
 * iterative solves.  Only f (3 x n_src) is read; the cell lists and work
 * items are reused, so the sorting stage is skipped.  PB_ERR_INVALID if no
 * execution with positions has succeeded since creation or the last bind. */
int pb_plan_execute_forces(pb_plan plan, const double* f, double* U, int where, void* stream);
int pb_plan_instance_info(pb_plan plan, int i, pb_instance_info* info);
/* A capacity plan (serving slot) with no instances bound yet. */
int pb_plan_create_slot(const pb_slot_config* cfg, pb_plan* out);
long long pb_slot_estimate_bytes(const pb_slot_config* cfg);
/* Bind `count` instances (<= the plan's instances) to the plan; the next
 * pb_plan_execute solves them (packed inputs in this order).  Each instance
 * keeps the grid of its position; the autotuner picks d and rc for it.  The
 * captured CUDA graph is reused: kernels read the bound sizes from device
 * memory.  PB_ERR_BUDGET if the totals exceed the capacity. */
int pb_plan_bind(pb_plan plan, const pb_solve_params* p, int count);
/* The autotuner's choice for one parameter block, on the host (no GPU). */
int pb_resolve(const pb_solve_params* p, pb_instance_info* info);
/* Device bytes held by the plan. */
long long pb_plan_device_bytes(pb_plan plan);
/* CUDA kernels one execution launches (kernel nodes of the captured graph;
 * 0 before the graph exists, i.e. before the second pb_plan_execute). */
int pb_plan_kernel_count(pb_plan plan);
/* One row of pb_tune_report. */
typedef struct pb_tune_row {
    int status;              /* PB_OK, or the error this candidate met (then max_err = rms_err = -1) */
    double d, rc;            /* splitting blob width and real-space cutoff it resolved to */
    int M[3], P;             /* grid and Gaussian support it resolved to */
    long long pairs_est;     /* estimated real-space pairs inside rc */
    double max_err, rms_err; /* against the reference solution: max_i |u_i - u*_i| / max_i |u*_i|, ||u - u*|| / ||u*|| */
    double ms;               /* device time of one execution (CUDA events, median of three replays) */
} pb_tune_row;

/* Error-versus-parameter report and splitting-independence study, the
 * concept of the reference's optimalNumShells (cuda/periodicBrinkman.h:
 * 836-1015, commented out there) and of its driver's d study
 * (cuda/periodicBrinkman.cu:139-203): the instance p with x, f (and y when
 * p->n_tgt > 0; where = PB_HOST or PB_DEVICE) is solved once per candidate
 * splitting width d_values[k] (0 = the autotuner's choice; p's other tuning
 * fields kept, 0 = autotuned for that d), and each result is compared with
 * a reference solution of the same instance: the FP64 path at tolerance
 * ref_tol (0 = 1e-12) with every tuning field autotuned.  The Ewald total
 * does not depend on d, so a row whose error exceeds p->tol marks a
 * parameter choice that misses the tolerance.  Allocates; synchronous. */
int pb_tune_report(const pb_solve_params* p, const double* x, const double* f, const double* y, int where,
                   const double* d_values, int nd, double ref_tol, pb_tune_row* rows);
/* Bytes a plan for these parameters would hold (for admission control). */
long long pb_plan_estimate_bytes(const pb_solve_params* p, int count);
/* Per-stage device time of the last pb_plan_execute (ms), if timing was
 * enabled with pb_plan_set_timing: [0] sort, [1] real space, [2] spread,
 * [3] FFT + Green, [4] gather, [5] combine. */
int pb_plan_set_timing(pb_plan plan, int enable);
/* Waits for the plan's last execution and returns its device-side status:
 * PB_ERR_INVALID if an input was not finite (those inputs were computed as
 * 0), PB_ERR_UNSUPPORTED if a capacity was exceeded (results incomplete),
 * else PB_OK.  Executions with PB_HOST buffers check this themselves. */
int pb_plan_status(pb_plan plan);
/* Testing aid: lowers the plan's real-space work-item capacity to `cap`
 * (at most what the plan allocated), so that the overflow check can be
 * exercised; drops the captured graphs. */
int pb_plan_set_item_capacity(pb_plan plan, int cap);
int pb_plan_stage_ms(pb_plan plan, double* ms6);
int pb_plan_destroy(pb_plan plan);

/* ---- continuous-batching server ------------------------------------------- */

typedef struct pb_server_config {
    long long budget_bytes; /* device memory for all slots, resident and dynamic (0: 150 GiB) */
    int precision;          /* PB_PREC_MIXED or PB_PREC_FP64 */
    int max_batch;          /* instances per slot execution (0: 4) */
    int slots_per_grid;     /* resident slots per grid size, created with the server (0: 4) */
    int n_grids;            /* grid sizes provisioned (0: 8, 16, ..., 256) */
    int grids[8];
    int max_src;            /* source capacity of a resident slot (0: 262144) */
    int max_tgt;            /* target capacity of a resident slot (0: max_src) */
    int queue_capacity;     /* pending requests before PB_ERR_BUSY (0: unbounded) */
    int linger_us;          /* an idle slot waits up to this long for a fuller batch (0: dispatch at once) */
    int max_dynamic_per_grid; /* dynamic slots per grid made from the unused budget (0: slots_per_grid; < 0: none) */
    int dynamic_idle_ms;    /* an idle dynamic slot is released after this long (0: 1000) */
} pb_server_config;

typedef struct pb_server_counters {
    long long submitted, completed, failed, rejected, batches;
    double mean_batch;      /* instances per slot execution */
    long long device_bytes; /* held by the slots now */
    int slots;              /* slots now (resident + dynamic) */
    long long kernels;      /* kernel launches of the slot executions (graph kernel nodes) */
    double scheduler_busy_s; /* time the scheduler thread spent binding, staging and launching */
    long long peak_device_bytes; /* most device memory the slots held at once */
    long long slots_created, slots_released; /* dynamic slots made and given back */
    long long memory_waits; /* times a request waited for device memory to free up */
} pb_server_counters;

typedef struct pb_server_s* pb_server;

/* Creates the resident slots within the budget and starts the scheduler.
 * Admission is by device-memory budget: a request that no slot of its grid
 * can hold gets a dynamic slot sized for it, and a grid whose queue backs up
 * while its slots are busy gets extra dynamic slots, both from the part of
 * the budget the slots do not hold; when the budget is taken, the request
 * waits in its queue while idle dynamic slots are released, and is admitted
 * as memory frees up.  Idle dynamic slots are also released after
 * dynamic_idle_ms. */
int pb_server_create(const pb_server_config* cfg, pb_server* out);
/* Queue one solve (HOST buffers the caller keeps alive until it completes;
 * U receives 3 x n_tgt, or 3 x n_src when n_tgt = 0).  The request is
 * autotuned here and assigned to the smallest provisioned grid that holds
 * its k-space resolution.  PB_ERR_BUDGET: even a slot of its own would not
 * fit the budget (larger than the largest grid, or too many points). */
int pb_server_submit(pb_server s, const pb_solve_params* p, const double* x, const double* f, const double* y,
                     double* U, long long* ticket);
/* state: 0 queued, 1 on the GPU, 2 done (then status and latency are set). */
int pb_server_poll(pb_server s, long long ticket, int* state, int* status, double* latency_s);
int pb_server_wait(pb_server s, long long ticket, double timeout_s, int* status, double* latency_s);
/* Forget a finished request. */
int pb_server_release(pb_server s, long long ticket);
/* Wait until every submitted request has finished. */
int pb_server_drain(pb_server s, double timeout_s);
int pb_server_stats(pb_server s, pb_server_counters* out);
int pb_server_destroy(pb_server s);

/* ---- parameter files --------------------------------------------------- */

/* Mirrors readData's array twin (cuda/periodicBrinkman.h:524-554): reads the
 * text file's lines, splits each at any character of `delimiters` (NULL =
 * ": "), and where the first token equals names[k] stores the second token,
 * converted as atof does, in values[k]; other lines are ignored and values
 * of names absent from the file are left as they are.  PB_ERR_INVALID if the
 * file cannot be opened (the reference returns 1) or a line has a name but
 * no value. */
int pb_read_params(const char* file_name, const char* delimiters, const char* const* names, double* values,
                   int numel);
/* Mirrors readData's map form (cuda/periodicBrinkman.cu:44-70): every name
 * of the file with its value (a later line overrides an earlier one), in
 * order of first appearance.  Writes up to max_keys names (NUL-terminated,
 * at most 63 characters) and values; returns the number of distinct names
 * (which may exceed max_keys: call again with more room) or an error. */
int pb_read_param_file(const char* file_name, const char* delimiters, char (*keys)[64], double* values,
                       int max_keys);

/* ---- misc ----------------------------------------------------------------- */
const char* pb_last_error(void);
const char* pb_version(void);
/* Build the FP32 real-space tables of one instance on the host and evaluate
 * the pair kernel H1, H2 at n radii exactly as the GPU polynomial path does
 * (FP32 Horner), for testing the tables without a GPU. */
int pb_debug_pair_kernel(double alpha, double d, double eps, double rc, int n, const double* r, double* H1,
                         double* H2);
/* The same for the FP64 path: its FP64 Chebyshev far series beyond r_mid,
 * the closed forms below it, evaluated on the host as the GPU does. */
int pb_debug_pair_kernel64(double alpha, double d, double eps, double rc, int n, const double* r, double* H1,
                           double* H2);
/* The k-space grid operator alone, for checking the hand-written FFT passes
 * against a library FFT: forward 3D real FFT of the three components of a
 * DEVICE grid, the Green-tensor multiply with Gaussian deconvolution (the
 * instance's kfac (1 + (1 - e^{-alpha^2 d^2/4}) k^2/alpha^2)
 * e^{-k^2 (d^2/4 - eta/2)} / (k^2 (k^2 + alpha^2)) (k^2 I - k k^T); Nyquist
 * planes and k = 0 zeroed) and the unnormalised inverse FFT, in place.  The
 * grid M and the splitting of `p` are resolved as a solve resolves them (M
 * must be given).  Layout: PB_PREC_MIXED, M^3 float4 (x, y, z, unused);
 * PB_PREC_FP64, four planes of M^3 doubles (x, y, z, unused).  Allocates a
 * temporary spectrum and synchronises `stream`. */
int pb_debug_fft_green(const pb_solve_params* p, void* grid, void* stream);
/* Number of CUDA devices visible (0 without a GPU). */
int pb_device_count(void);

#ifdef __cplusplus
}
#endif
#endif
