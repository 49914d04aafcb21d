/*
 * subby_gb300 — C ABI of the GB300 (sm_103a) eigensubstitution backend.
 *
 * One call computes, for every alignment column independently, the
 * Felsenstein inside pass, the outside pass and the eigenbasis J(t) count
 * accumulation of ihh/subby, on one GPU.  Inputs are the reference's
 * (alignment, parentIndex, distanceToParent, eigenvalues, eigenvectors, pi)
 * as flat arrays; outputs use the reference layouts (column last):
 *
 *   logLike   (C,)        float32     subby/jax/__init__.py:207-291
 *   counts    (A, A, C)   float32     subby/jax/__init__.py:338-447
 *             diagonal = dwell times, off-diagonal = substitution counts
 *   rootProb  (A, C)      float32     subby/jax/__init__.py:543-650
 *
 * The flat-array argument convention (R = len(parentIndex), C = columns,
 * A = len(pi), eigenvectors row-major v[a*A + k]) is that of the reference's
 * Rust/WASM exports subby/wasm/src/lib.rs:622-760, which every entry point
 * below mirrors; the reference's Python API the host shim reproduces is
 * subby/jax/__init__.py.
 *
 * Conventions
 *  - alignment is (R, C) int32 row-major; tokens 0..A-1 observed, A
 *    ungapped-unobserved, A+1 gapped, -1 legacy gap; any other value is
 *    treated as unobserved (subby/oracle/oracle.py:69-96).
 *  - parentIndex[0] < 0, 0 <= parentIndex[n] < n, every node has 0 or 2
 *    children (subby/oracle/oracle.py:52-62); violations return
 *    SUBBY_ERR_TREE.
 *  - Tree and model arrays are always host pointers (FP64 preparation stays
 *    on the host, as in the reference).
 *  - alignment, mask and output pointers are host pointers unless
 *    SUBBY_DEVICE_PTRS is set in `flags`, in which case they are device
 *    pointers on the current device.  With host pointers the call copies in
 *    and out on `stream` and returns after the results are in host memory;
 *    with device pointers it only enqueues work on `stream` (NULL = legacy
 *    default stream).
 *  - Every function returns 0 (SUBBY_OK) or a negative SUBBY_ERR_* code;
 *    subby_strerror() names it and subby_last_error() gives details of the
 *    most recent failure on the calling thread.
 */
#ifndef SUBBY_GB300_H
#define SUBBY_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SUBBY_OK               0
#define SUBBY_ERR_ARG         -1   /* null pointer / bad size / bad enum      */
#define SUBBY_ERR_TREE        -2   /* parentIndex is not a binary preorder tree */
#define SUBBY_ERR_UNSUPPORTED -3   /* alphabet size or tree too large          */
#define SUBBY_ERR_CUDA        -4   /* CUDA runtime failure                     */
#define SUBBY_ERR_NOMEM       -5   /* device or pinned allocation failed       */
#define SUBBY_ERR_TIMEOUT     -6   /* a bounded device wait gave up            */

/* flags */
#define SUBBY_DEVICE_PTRS   1      /* alignment/mask/outputs are device pointers */
#define SUBBY_BT_FP32       2      /* back-transform in FP32 (default: FP64 for A <= 8) */
#define SUBBY_BT_FP64       4      /* force FP64 back-transform for any A          */
#define SUBBY_IRREV_EXACT   8      /* irreversible models: counts of M(t) = e^{Qt}
                                      itself (D~ = D V, U~ = V^-1 U, V^-T C V^T)
                                      instead of the reference's formula       */

/* mask_mode */
#define SUBBY_MASK_NONE   0        /* every branch n >= 1 counts                 */
#define SUBBY_MASK_AUTO   1        /* Steiner tree of ungapped leaves (default)  */
#define SUBBY_MASK_GIVEN  2        /* (R, C) uint8 mask supplied by the caller   */

/* Counts variants */
#define SUBBY_COUNTS_EIGEN 0       /* general eigensubstitution path            */
#define SUBBY_COUNTS_F81   1       /* O(A^2) F81/JC closed form (f81_fast_flag) */

typedef struct subby_plan subby_plan;

/* Library version string. */
const char *subby_version(void);
/* Human-readable name of a status code. */
const char *subby_strerror(int status);
/* Details of the last failure on the calling thread ("" if none). */
const char *subby_last_error(void);

/*
 * Prepare a (tree, model) pair once: validates the tree, builds the
 * postorder schedule, computes M(t) in FP64 on the host and J(t) on the GPU
 * (FP64 only for near-degenerate eigenvalue pairs), and keeps every table
 * resident on the current device.  Replaces the per-call model preparation
 * of subby/jax/__init__.py:285-289 / 431-435 (compute_sub_matrices,
 * subby/jax/diagonalize.py:141-172; compute_J, subby/jax/eigensub.py:7-50).
 */
int subby_plan_create(const int32_t *parent_index, const double *distances,
                      const double *eigenvalues, const double *eigenvectors,
                      const double *pi, int R, int A, subby_plan **out);
/*
 * The same for an irreversible model (subby.jax IrrevDiagModel,
 * subby/jax/types.py:14-18): eigenvalues (A complex), eigenvectors V and
 * eigenvectors_inv V^-1 (A x A complex, row-major), each complex value as
 * two doubles (re, im) — the memory layout of numpy complex128.  M(t) =
 * Re V diag(e^{mu t}) V^-1 and the complex J(t) are formed in FP64 on the
 * host (subby/oracle/oracle.py:474-534).  LogLike, RootProb, posteriors,
 * Counts and per-branch counts (complex accumulation and back-transform,
 * oracle.py:537-740) and the distance gradient (subby_plan_grad; dldS
 * is zeros) then run on this plan; the F81 fast path returns an error (the
 * reference's F81 path is reversible-only).
 * Counts are implemented for A = 4, 8, 16, 20, 32, 64.
 */
int subby_plan_create_irrev(const int32_t *parent_index, const double *distances, const double *eigenvalues,
                            const double *eigenvectors, const double *eigenvectors_inv, const double *pi, int R,
                            int A, subby_plan **out);
/*
 * Per-branch models (the reference's (1, R) model grid,
 * subby/jax/__init__.py:74-152): node n's reversible system
 * eigenvalues[n*A ..], eigenvectors[n*A*A ..] (row-major), pi[n*A ..] gives
 * M_n; the root prior is node 0's pi.  LogLike, RootProb and posteriors run
 * the usual kernels on the per-node M(t); Counts and per-branch counts run
 * the complex accumulation once per group of branches sharing a system
 * (each branch projected and back-transformed in its own eigenbasis); the
 * distance gradient (subby_plan_grad) uses each node's dM/dt.  The F81
 * fast path returns an error.
 */
int subby_plan_create_rows(const int32_t *parent_index, const double *distances, const double *eigenvalues,
                           const double *eigenvectors, const double *pi, int R, int A, subby_plan **out);
int subby_plan_destroy(subby_plan *plan);
/* Bytes of device memory the plan currently holds (tables + workspace). */
size_t subby_plan_device_bytes(const subby_plan *plan);
/*
 * Per-branch counts: branchCounts (R, A, A, C) — for each branch n (the
 * branch above node n; n = 0, the root, is zeros) the dwell times (diagonal)
 * and substitution counts (off-diagonal) per column.  counts_kind, mask_mode
 * and mask as for subby_plan_run (subby.jax.BranchCounts does not mask: pass
 * SUBBY_MASK_NONE for its semantics).  Implemented for A = 4, 16, 20, 32
 * and 64; other alphabets return SUBBY_ERR_UNSUPPORTED.  Replaces subby.jax BranchCounts
 * (subby/jax/__init__.py:450-540) and the oracle's BranchCounts
 * (subby/oracle/oracle.py:1517-1568).
 */
int subby_plan_branch_counts(subby_plan *plan, const int32_t *alignment, int C, float *branchCounts,
                             int counts_kind, int mask_mode, const uint8_t *mask, int flags, void *stream);
/*
 * Posteriors of the inside-outside tables.  node = -1: nodePost (R, A, C) is
 * the posterior state distribution of every node (row 0, the root, equals
 * RootProb) and branchPost (R, A, A, C) the joint posterior of (parent state
 * i, child state j) on every branch (branch 0 zeros).  node = n >= 0: the
 * same for node n only, nodePost (A, C) and branchPost (A, A, C) (n > 0 for
 * branchPost).  Either output may be NULL.  Implemented for A = 4, 8, 16,
 * 20, 32 and 64.  Replaces subby.jax InsideOutside.node_posterior /
 * branch_posterior (subby/jax/__init__.py:868-1040) and the oracle's
 * (subby/oracle/oracle.py:1755-1905).
 */
int subby_plan_posteriors(subby_plan *plan, const int32_t *alignment, int C, int node, float *nodePost,
                          float *branchPost, int flags, void *stream);
/*
 * Posterior over mixture components per column: out[k][c] = softmax_k of
 * logL[k][c] + log_weights[k] (logL, out (K, C) float32; log_weights (K,)
 * host float64).  Replaces MixturePosterior's final step
 * (subby/jax/mixture.py:6-28, subby/jax/__init__.py:653-678; oracle
 * subby/oracle/oracle.py:1334-1365); the K log-likelihoods come from one
 * plan per component.
 */
int subby_mixture_posterior(const float *logL, const double *log_weights, int K, int C, float *out, int flags,
                            void *stream);
/*
 * Tokenise n characters on the device: out[i] = lut[chars[i]] (lut: 256
 * device int32 entries, -1 = not in the alphabet); *first_bad (device int64,
 * preset to -1 by the caller) receives the smallest index of a byte mapped
 * to -1.  chars and out 16-byte aligned, device pointers; enqueued on
 * `stream`.  The character tokenisation of subby/formats.py:228-625 for
 * large alignments (1 byte per cell over the host link instead of 4).
 */
int subby_tokenize(const uint8_t *chars, int64_t n, const int32_t *lut, int32_t *out, int64_t *first_bad,
                   void *stream);
/*
 * Gather token rows into a contiguous (R, C) int32 device array on
 * `stream`: dst[r*C + c] = src[map(r)*pitch + c] with map(r) = rowmap[r]
 * (a device array of R row indices) or r when rowmap is NULL.  src may be
 * pinned host memory (the SMs read it over the host link) or device memory;
 * pitch >= C is its row length in elements; R <= 65535.  The serving loop
 * uploads each job's alignment with it from a window of a larger host
 * buffer.  No reference counterpart (the reference builds its inputs on the
 * host).
 */
int subby_gather_rows(const int32_t *src, int64_t pitch, const int32_t *rowmap, int R, int C,
                      int32_t *dst, void *stream);
/* Wait for the plan's enqueued work and report SUBBY_ERR_TIMEOUT if a
 * bounded device wait (tensor-core kernels) gave up since the last check
 * (device-pointer runs return before their kernels finish, so they report
 * it here); clears the record.  No counterpart in the reference. */
int subby_plan_status(subby_plan *plan);
/* Replace the root prior (A positive values, host FP64) of a reversible
 * plan; the model's pi still defines M(t) and the eigenbasis.  This is the
 * root prior of subby.jax InsideOutside over a per-column model list, which
 * takes the first model's pi for every column (subby/jax/__init__.py:
 * 721-731, rootProb = stacked.pi[0]); the posteriors, LogLike and RootProb
 * of later runs use it.  Ordered after the plan's enqueued work. */
int subby_plan_set_root_prior(subby_plan *plan, const double *root_prior);
/* Release the plan's workspace (staging, scratch, host-call buffers) in
 * stream order after its last enqueued kernel; the tables stay.  The next
 * run allocates again (from the library pool).  For servers that keep many
 * plans resident.  No counterpart in the reference (it holds no device
 * state between calls). */
int subby_plan_trim(subby_plan *plan);

/*
 * Run the hot path of a prepared plan on a (R, C) alignment.
 *   logLike : (C,) or NULL
 *   counts  : (A, A, C) or NULL (NULL skips the outside pass)
 *   rootProb: (A, C) or NULL
 *   counts_kind: SUBBY_COUNTS_EIGEN or SUBBY_COUNTS_F81
 *   mask_mode / mask: as above (mask ignored unless SUBBY_MASK_GIVEN)
 * Replaces subby.jax LogLike (subby/jax/__init__.py:207), Counts (:338) and
 * RootProb (:543) for a single reversible DiagModel.
 */
int subby_plan_run(subby_plan *plan, const int32_t *alignment, int C,
                   float *logLike, float *counts, float *rootProb,
                   int counts_kind, int mask_mode, const uint8_t *mask,
                   int flags, void *stream);

/*
 * Gradient of sum_c g_c * logLike_c (g NULL = all ones) with respect to the
 * branch lengths (dldt, (R,), root entry 0) and to the symmetrised rate
 * matrix S (dldS, (A, A), FP64, = sum_c g_c V C_c V^T with the unmasked
 * eigenbasis counts C_c).  The distance part is the Fisher-identity rule of
 * subby/jax/vjp.py:62-133; the rate part has no reference counterpart beyond
 * jax.grad and is checked against finite differences.  logLike (C,) may be
 * NULL.  Always synchronous.
 */
int subby_plan_grad(subby_plan *plan, const int32_t *alignment, int C,
                    const float *g, float *logLike, double *dldt, double *dldS,
                    int flags, void *stream);

/* One-shot conveniences (plan create + run + destroy), mirroring the
 * reference Rust/WASM exports wasm_log_like / wasm_counts / wasm_root_prob
 * (subby/wasm/src/lib.rs:628-734) with explicit output buffers. */
int subby_loglike(const int32_t *alignment, const int32_t *parent_index,
                  const double *distances, const double *eigenvalues,
                  const double *eigenvectors, const double *pi,
                  int R, int C, int A, float *logLike, int flags, void *stream);
int subby_counts(const int32_t *alignment, const int32_t *parent_index,
                 const double *distances, const double *eigenvalues,
                 const double *eigenvectors, const double *pi,
                 int R, int C, int A, int counts_kind, int mask_mode,
                 const uint8_t *mask, float *counts, int flags, void *stream);
int subby_rootprob(const int32_t *alignment, const int32_t *parent_index,
                   const double *distances, const double *eigenvalues,
                   const double *eigenvectors, const double *pi,
                   int R, int C, int A, float *rootProb, int flags, void *stream);

/*
 * Counts (and optionally LogLike) for A = 4 without allocating anything: no
 * cudaMalloc / cudaFree and no host heap allocation.  For callers that
 * cannot allocate device memory — a framework whose caching allocator owns
 * the device heap, a plugin or callback that must not allocate, a service
 * that fixes its device footprint at start-up.  Every table the kernel reads
 * lives in one file-scope device array of 1 MiB that each GPU loading the
 * library holds until exit; slot state stays in tensor / shared memory.
 *   alignment (R, C) int32, mask (R, C) uint8 (SUBBY_MASK_GIVEN only),
 *   counts (A*A*C) and logLike (C, may be NULL): DEVICE pointers.
 *   Tree and model arrays: host pointers, as elsewhere.
 * Limits: A = 4, R <= 1023 nodes, and the tree program must fit the A = 4
 * kernel's on-chip budget; larger inputs return SUBBY_ERR_UNSUPPORTED.
 * The first call on a device resolves the array's device address with that
 * device current and loads the kernels; make that first call before any
 * stream capture.  A call with C = 0 validates its arguments and does only
 * this set-up: it is the warm-up step.  The tables are uploaded from a host
 * staging buffer that the next call rewrites, so a call on a stream that is
 * capturing returns SUBBY_ERR_UNSUPPORTED.  Each call rewrites every table it
 * uses, so nothing needs clearing between calls, but calls that overlap on
 * the GPU share the array and race.  A rejection's reason is a fixed string
 * returned by subby_last_error().  Work is enqueued on `stream`.  No
 * counterpart in the reference.
 */
int subby_counts_noalloc(const int32_t *alignment, const int32_t *parent_index,
                         const double *distances, const double *eigenvalues,
                         const double *eigenvectors, const double *pi,
                         int R, int C, int counts_kind, int mask_mode,
                         const uint8_t *mask, float *counts, float *logLike,
                         void *stream);

/*
 * Serving engine: continuous batching of jobs of uneven R, C and A on the
 * current device.  An engine thread admits submitted jobs as slots and the
 * device-memory budget free up (shortest estimated job first, aged by its
 * wait; two slots kept for short jobs), runs short A = 4 jobs that wait
 * together as one launch of a persistent kernel over their flattened
 * (job, column-tile) queue, keeps prepared plans resident in an LRU cache
 * keyed by tree and model, gathers each job's alignment rows from host
 * memory on the job's own stream, runs long jobs as column slices so that
 * short ones are not held behind them, and copies results into pinned host
 * blocks that the caller hands back with subby_server_release.  The
 * reference has no server (its batching is jax.vmap over same-shaped trees,
 * scripts/batch_eigensub_maf.py:527-532); the per-job computation is
 * subby_plan_run's.  Reversible models only.
 */
typedef struct subby_server subby_server;

#define SUBBY_WANT_LOGLIKE  1
#define SUBBY_WANT_COUNTS   2
#define SUBBY_WANT_ROOTPROB 4

typedef struct subby_job {
  /* tree and model, host memory, copied by subby_server_submit */
  const int32_t *parent_index;
  const double *distances;
  int R;
  const double *eigenvalues, *eigenvectors, *pi;
  int A;
  /* alignment: row r of the job is alignment + map(r) * pitch (C int32
   * tokens), map(r) = row_map[r] (host, R entries, copied) or r.  Pinned
   * host memory (read by the GPU over the host link) or device memory; it
   * must stay valid until the job completes. */
  const int32_t *alignment;
  int64_t pitch;
  const int32_t *row_map;
  int C;
  int want;          /* SUBBY_WANT_* bits */
  int counts_kind;   /* SUBBY_COUNTS_EIGEN / SUBBY_COUNTS_F81 */
  int mask_mode;     /* SUBBY_MASK_NONE / SUBBY_MASK_AUTO */
  double arrival;    /* arrival time on the server clock, or < 0 for now */
  int64_t tag;       /* caller's identifier, returned with the result */
} subby_job;

typedef struct subby_job_result {
  int64_t tag, handle;
  int status;        /* SUBBY_OK, SUBBY_ERR_TIMEOUT (a bounded device wait gave up), ... */
  const float *logLike, *counts, *rootProb;  /* pinned host, (C,), (A,A,C), (A,C) or NULL */
  double t_arrival, t_start, t_finish;       /* server clock, seconds */
} subby_job_result;

/* Create an engine on the current device with max_inflight slots (2..64),
 * a device-memory budget for admitted jobs, and pinned result blocks
 * allocated up front (two of every power-of-two size up to
 * pinned_prewarm_bytes). */
int subby_server_create(int max_inflight, size_t device_budget, size_t pinned_prewarm_bytes,
                        subby_server **out);
/* Queue a job (thread-safe; returns at once). */
int subby_server_submit(subby_server *server, const subby_job *job);
/* Collect up to max completed jobs, waiting up to timeout_ms for the first;
 * *n receives how many.  Each result's buffers stay valid until
 * subby_server_release(handle). */
int subby_server_wait(subby_server *server, subby_job_result *out, int max, int timeout_ms, int *n);
int subby_server_release(subby_server *server, int64_t handle);
/* Scheduling parameters, before the first submission: "short_ms" (jobs up
 * to this estimated device time take the high-priority streams and the
 * reserved slots; 5), "slice_ms" (long jobs run as column slices of about
 * this device time; 8), "wave_cols" (slice granularity in columns; 0 = one
 * wave of the kernels' grids), "aging" (ms of estimated cost forgiven per ms
 * waited; 0.2), "short_slots" (2), "plan_cache" (resident plans; 64),
 * "pack" (1: short A = 4 jobs waiting together run as one launch of the
 * persistent packed kernel over their (job, column-tile) queue; 0: one
 * launch per job), "pack_max_jobs" (64), "pack_tiles_r64",
 * "pack_tiles_r256", "pack_tiles_big" (256-column tiles per packed work item
 * for trees of up to 64, up to 256 and more nodes; 1; the shape
 * subby_gb300.serve.autotune_packed chooses). */
int subby_server_set(subby_server *server, const char *key, double value);
/* Seconds since the engine was created (the clock of arrival / finish). */
double subby_server_clock(subby_server *server);
/* Engine-thread busy time, cached plans, in-flight runs, waiting jobs, and
 * the jobs / launches of the packed A = 4 kernel so far (any may be NULL). */
int subby_server_stats(subby_server *server, double *engine_busy_s, int *plans_cached, int *inflight,
                       int *waiting, long long *packed_jobs, long long *packed_launches);
/* Finish every queued job, then free the engine and everything it holds. */
int subby_server_destroy(subby_server *server);
/* Test hook of the packed kernel's bounded queue wait: launches it on `grid`
 * CTAs over an open queue with nothing published; every CTA's claim waits
 * `polls` polls, gives up and counts itself in the status word (*gave_up).
 * Returns SUBBY_ERR_TIMEOUT when any wait gave up.  Synchronous; no
 * reference counterpart. */
int subby_debug_packed_queue_wait(int polls, int grid, int *gave_up);

/* Test hook selecting the kernel so that every code path can be checked
 * against the oracle: 0 automatic (A = 4 tree kernel with tensor-memory
 * slots when it fits; A = 64 tree walk on the tensor cores), 1
 * thread-per-column kernel (A <= 8) / warp-per-column kernel (larger A), 2
 * tree program with shared-memory slots (A <= 8) / FP32 CUDA-core tree walk
 * (larger A), 3 tree program with global-memory slots, 4 generic tree
 * program with tensor-memory slots, 5 (A = 64) tensor-core walk with the
 * CUDA-core back-transform, 6 (A = 64) CUDA-core walk with the tensor-core
 * back-transform.  No reference counterpart. */
int subby_debug_set_kernel(int which);

/* Test hook of the bounded-wait failure path: with polls > 0, every
 * tensor-core tree walk (A = 64) launched afterwards first waits on an
 * mbarrier that nothing arms, while no copy or MMA is in flight, gives up
 * after `polls` polls, frees its tensor memory and skips its work, so that
 * subby_plan_status (device pointers) or the call itself (host pointers)
 * reports SUBBY_ERR_TIMEOUT and the outputs are left unwritten.  0 (the
 * default) turns it off; polls must be 0..4096.  No reference
 * counterpart. */
int subby_debug_fail_waits(int polls);

/* Number of kernel launches the most recent subby_plan_run /
 * subby_plan_grad on this thread enqueued (for launch accounting). */
int subby_last_launch_count(void);

#ifdef __cplusplus
}
#endif

#endif /* SUBBY_GB300_H */
