// Shared definitions of the subby_gb300 kernels and host plan.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace subby {

// Step of the node schedule: one internal node p with children l < r.
// Steps are stored in postorder (children before parents); the outside pass
// walks them backwards (preorder).
//   step.x = p, step.y = l, step.z = r, step.w = flags (bit0 l is leaf,
//   bit1 r is leaf, bit2 p is the root)
//   slot.x = scratch slot of p (-1 root), slot.y = of l, slot.z = of r
//            (-1 for leaves: leaves are recomputed from their token)
enum : int { kLeafL = 1, kLeafR = 2, kRoot = 4 };

enum : int {
  kModeLogLike = 1,      // write logLike
  kModeRootProb = 2,     // write rootProb
  kModeCounts = 4,       // outside pass + counts
  kModeF81 = 8,          // F81 closed form instead of the eigenbasis path
  kModeBT64 = 16,        // FP64 back-transform
  kModeGrad = 32,        // gradient accumulation instead of counts output
  kModeBranch = 64,      // per-branch counts (R, A, A, C) instead of their sum
  kModeIrrevExact = 128, // irreversible counts of M(t) itself, not the reference's formula
};

enum : int { kMaskNone = 0, kMaskAuto = 1, kMaskGiven = 2 };

// Offsets (in floats) of the per-plan tables inside the packed FP32 buffer.
struct TableOffsets {
  int MT;    // R x (A+1) x A : MT[n][j][b] = M_n[b][j] (j<A), MT[n][A][b] = sum_j M_n[b][j]
  int MN;    // R x A x A     : MN[n][i][a] = M_n[i][a]
  int J;     // R x A x A     : J[n][k][l]
  int JT;    // R x A x A     : JT[n][l][k] = J[n][k][l]
  int F81;   // R x 4         : alpha, beta, gamma, t
  int Vu;    // A x A         : Vu[b][l] = sqrt(pi_b) V[b][l]
  int Vd;    // A x A         : Vd[a][k] = V[a][k] / sqrt(pi_a)
  int Ut;    // (A+1) x A     : Ut[tok][l] = Vu[tok][l], Ut[A][l] = sum_b Vu[b][l]
  int pi0;   // A             : root prior (pi unless subby_plan_set_root_prior set another);
             //                 follows V in the small block
  int pi;    // A
  int V;     // A x A         : V[i][k] (FP32 copy)
  int S;     // A x A         : S[i][j] = sum_k V_ik mu_k V_jk
  int ME;    // R x A         : mu_k e^{mu_k t_n} (distance gradient)
  int K;     // R x (A+1) x A x A (A <= 8 only): K[n][code][k][l] = J[n][k][l] Ut[code][l]
  int EF;    // R x 2         : e^{-mu t_n}, 1 - e^{-mu t_n} (F81 closed form of M(t))
  int total;
};

// A table copied into shared memory at kernel start.
struct SmemTable {
  int gofs;   // offset in the packed buffer (floats)
  int sofs;   // offset in shared memory (floats)
  int n;      // floats
};

constexpr int kMaxSmemTables = 8;

struct KParams {
  const int32_t *aln;     // (R, C)
  int C, R, A, nInt;
  int mode;
  int mask_mode;
  const uint8_t *mask;    // (R, C) when mask_mode == kMaskGiven
  const float *tab;       // packed FP32 tables (device)
  const double *tab64;    // V (A x A), S (A x A) in FP64
  TableOffsets off;
  const int4 *steps;      // (nInt,) device
  const int4 *slots;      // (nInt,) device
  int root_is_leaf;
  float f81_mu;
  // scratch: vectors [slot][worker][A] floats, words [slot][worker][2] ints
  float *scrV;
  int *scrW;
  int nworkers;           // threads (small kernel) or warps (warp kernel) in the grid
  // outputs
  float *logL;
  float *counts;
  float *rootp;
  // gradient outputs (kModeGrad): per-block partial sums
  const float *g;         // (C,) cotangent or NULL (= ones)
  double *grad_t;         // (gridDim.x, R)  partial d/dt
  double *grad_C;         // (gridDim.x, A, A) partial sum_c g_c C_c (eigenbasis)
  // shared-memory tables
  int ntab;
  SmemTable stab[kMaxSmemTables];
  int smem_steps;         // sofs of steps (ints) in shared memory, -1 = read from global
  int smem_slots;
  // tree-program kernel (k_tree.cu)
  const int4 *prog;       // (nsteps, 4) int4
  int nsteps;
  int nslots;
  int smem_words;         // sofs of the slot words (k_tree, shared-memory slots)
  // tensor-core walk (A = 64): three-term BF16 operand tiles in the
  // canonical K-major layout; per node n at n*24576: [M 1|2|3 | M^T 1|2|3]
  // (4096 elements each), then [Vd^T 1|2|3 | Vu^T 1|2|3] at R*24576
  const uint16_t *tab16;
  int *err;               // device status: bounded waits that gave up (tensor-core walk)
  int noderiv;            // the walk's program has no derived nodes (every internal node stored)
  int dbg_wait_polls;     // test hook: > 0 makes the tensor-core walk's prologue wait
                          // on an unarmed mbarrier for that many polls and give up
  // the model is F81 / JC: M_n = e_n I + (1 - e_n) 1 pi^T, so the walk's
  // products take the closed form (tables EF) instead of A x A products
  int f81_model;
  // F81 staging (k_walk MODE 2): per branch and column (pi . U, sum s D), or null
  float2 *stage_c;
  // node posteriors (k_walk MODE 3): (R, A, C) for npost_node < 0, else the
  // (A, C) of node npost_node
  float *npost;
  int npost_node;
  // branch joint posteriors (k_tree4, A = 4): (R, 4, 4, C) or the (4, 4, C)
  // of node npost_node
  float *bpost;
  // irreversible models: complex tables (k_acccx.cu) and the choice of the
  // reference's formula (0) or the expected counts of M(t) itself (1)
  const float2 *cx;
  int cx_exact;
  const float2 *cx_tab;   // the system's tables (V, Vinv, rate, Vinv^T, V^T, FP64 copies)
  const int *cx_br;       // branches of this system; the kernels take list slots [n_lo, n_hi)
  int cx_accum;           // add the summed counts to the output instead of storing
};

// launchers (k_small.cu / k_warp.cu)
int launch_small(const KParams &p, int A, int grid, int block, size_t smem, cudaStream_t s);
int launch_warp(const KParams &p, int A, int grid, int block, size_t smem, cudaStream_t s);
// store: 0 shared-memory slots, 1 global-memory slots, 2 tensor-memory slots (A = 4)
int launch_tree(const KParams &p, int A, int store, int grid, int block, size_t smem,
                cudaStream_t s);
bool tree_supported(int A);
// large-alphabet walk + accumulation (k_big.cu)
bool big_supported(int A);
int big_tile();
int big_acc_group(int A);
// mode: 0 inside pass only (LogLike / RootProb), 1 stage eigen vectors, 2 stage F81 vectors
int launch_walk(const KParams &p, int A, int mode, bool tc, float *sa, float *sb, int c_base, int c_count,
                int grid, cudaStream_t s);
// the walk of the posteriors (k_walkpost.cu) at A = 4, 8 and the large
// alphabets: mode 0 (inside only: the root's posterior) or 3 (node
// posteriors, and D_n s_n, U_n staged in the original basis when sa is given)
int launch_walk_post(const KParams &p, int A, int mode, bool tc, float *sa, float *sb, int c_base, int c_count,
                     int grid, cudaStream_t s);
// branch posteriors of branches [n_lo, n_hi) from the raw staging
// (k_post.cu); output row = n - row_off
bool post_supported(int A);
int post_tile();
int launch_post(const KParams &p, int A, const float *sa, const float *sb, int c_base, int c_count, int n_lo,
                int n_hi, int row_off, float *br_out, int grid, cudaStream_t s);
// tc: A = 64 eigen back-transform on the tensor cores
int launch_acc(const KParams &p, int A, bool f81, bool tc, const float *sa, const float *sb, int c_base,
               int c_count, int grid, cudaStream_t s);
int launch_tree4(const KParams &p, bool f81, int mask_mode, int grid, int block, size_t smem,
                 cudaStream_t s);
// Packed queue of (job, column range) work items of the A = 4 serving
// kernel (k_tree4_packed): jobs[j] are the tree-kernel parameters of job j,
// items are (job, first column, end column) of a run of whole tiles of
// blockDim.x columns (how many tiles an item spans is the work-item shape
// the serving autotuner picks).  CTAs claim items with an atomic counter; an
// item at or past *published is waited for (at most wait_polls polls) until
// *closed is set, and a wait that gives up increments *err and ends the CTA.
struct T4Queue {
  const KParams *jobs;
  const int4 *items;
  int *head;
  const int *published;
  const int *closed;
  int wait_polls;
  int *err;
};
int launch_tree4_packed(const T4Queue &q, bool f81, int mask_mode, int grid, int block, size_t smem,
                        cudaStream_t s);
// Row-strided copy by the SMs (k_token.cu): rows x width bytes (width a
// multiple of 4), e.g. device results into pinned host memory.
int launch_copy_rows(void *dst, size_t dpitch, const void *src, size_t spitch, size_t width, int rows,
                     cudaStream_t s);
// Load the counts variants of the A = 4 kernel into the current context
// (cudaFuncGetAttributes), so that a later launch needs no module loading.
int preload_tree4();
// Record a fixed failure reason for subby_last_error without allocating
// (plan.cu); nullptr or "" clears it.
void set_static_error(const char *why);
// irreversible counts (k_acccx.cu): complex accumulation + back-transform
// over the walk's raw staging; pb: per-branch counts
bool cx_supported(int A);
int cx_columns_per_cta(int A);
bool cx_bt64(int A);  // C buffered and back-transformed in FP64 (k_bt_cx)
int launch_acc_cx(const KParams &p, int A, bool pb, const float *sa, const float *sb, int c_base, int c_count,
                  int n_lo, int n_hi, float2 *cbuf, int grid, cudaStream_t s);
int launch_bt_cx(const KParams &p, int A, const float2 *cbuf, int c_base, int c_count, int row, int grid,
                 cudaStream_t s);
// reversible large-alphabet gradient (k_grad.cu): X_n += sum_c g_c D~_nc (x) U~_nc
// from the walk's eigen staging, X (R x A x A) FP64
int xgram_items(int R, int c_count);
int launch_xgram(int A, const float *sa, const float *sb, const float *g, int c_base, int c_count, int R, double *X,
                 int grid, cudaStream_t s);
// distance gradient from the raw staging: grad_t[n] += sum_c g_c (D s)^T G_n U
int launch_grad_cx(const KParams &p, int A, const float *sa, const float *sb, const float *gq, const float *g,
                   int c_base, int c_count, double *grad_t, int grid, cudaStream_t s);
// A = 4 posteriors (npost / bpost) from the tree-program kernel
int launch_tree4_post(const KParams &p, int grid, int block, size_t smem, cudaStream_t s);
// A = 64 F81 accumulation on the tensor cores (k_acctc.cu); groups of 8 columns
int launch_acc_f81_tc(const KParams &p, const float *sa, const float *sb, const float2 *sc, int c_base,
                      int c_count, int grid, cudaStream_t s);
bool small_supported(int A);
bool warp_supported(int A);
int small_block();
int warp_block();
size_t warp_smem_per_warp(int A);

}  // namespace subby
