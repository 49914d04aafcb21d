// Host side of the subby_gb300 C ABI: tree validation and scheduling, FP64
// model preparation, J(t) prologue kernel, workspace management and kernel
// dispatch.  See include/subby_gb300.h for the contract.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <complex>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include <cuda_bf16.h>

#include "common.cuh"
#include "subby_gb300.h"

using namespace subby;

namespace {

thread_local std::string g_last_error;
// A fixed reason string set by entry points that must not allocate (a
// std::string assignment could); it takes precedence over g_last_error.
thread_local const char *g_static_error = nullptr;
thread_local int g_launches = 0;
// Test hook (subby_debug_set_kernel): 0 automatic, 1 thread-per-column
// kernel (k_small) for A <= 8 / warp-per-column kernel (k_warp) above, 2
// tree program with shared-memory slots / FP32 CUDA-core walk (no tensor
// cores) for large A, 3 tree program with global-memory slots, 4 generic
// tree program with tensor-memory slots (bypassing the A = 4 specialisation).
int g_kernel_sel = 0;
// Test hook (subby_debug_fail_waits): > 0 makes every tensor-core walk give
// up a prologue wait after that many polls.
std::atomic<int> g_dbg_wait_polls{0};

int fail(int code, const std::string &msg) {
  g_static_error = nullptr;
  g_last_error = msg;
  return code;
}

void clear_error() {
  g_static_error = nullptr;
  g_last_error.clear();
}

int cuda_fail(cudaError_t e, const char *where) {
  return fail(SUBBY_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define CU(call)                                   \
  do {                                             \
    cudaError_t e_ = (call);                       \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
  } while (0)

// J(t) prologue.  J_kl(t) = (e^{mu_k t} - e^{mu_l t}) / (mu_k - mu_l), and
// t e^{mu_k t} when |mu_k - mu_l| < 1e-8 (subby/oracle/oracle.py:931-959,
// subby/jax/eigensub.py:7-50).  Pairs whose |dmu| t is below 1e-3 (the
// near-degenerate ones, where the difference of exponentials cancels) are
// evaluated in FP64; the others in FP32 through the cancellation-free form
// e^{mu_l t} expm1(dmu t) / dmu with dmu taken from the FP64 eigenvalues.
__global__ void k_compute_J(const double *__restrict__ mu, const double *__restrict__ t, int R,
                            int A, float *__restrict__ J, float *__restrict__ JT) {
  const int total = R * A * A;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += gridDim.x * blockDim.x) {
    const int n = idx / (A * A);
    const int k = (idx / A) % A;
    const int l = idx % A;
    const double tn = t[n];
    const double dmu = mu[k] - mu[l];
    float v;
    if (fabs(dmu) < 1e-8) {
      v = (float)(tn * exp(mu[k] * tn));
    } else if (fabs(dmu) * tn < 1e-3) {
      v = (float)((exp(mu[k] * tn) - exp(mu[l] * tn)) / dmu);
    } else {
      const float x = (float)(dmu * tn);
      v = expf((float)(mu[l] * tn)) * expm1f(x) / (float)dmu;
    }
    J[idx] = v;
    JT[(size_t)n * A * A + l * A + k] = v;
  }
}

// Substitution matrices M_n(t) = diag(1/sqrt pi) V e^{Lambda t} V^T diag(sqrt pi)
// (subby/oracle/oracle.py:747-777), evaluated in FP64 from the FP64
// eigensystem (the reference's own model-preparation precision) and stored
// as FP32 tables: MT[n][j][b] = M_n[b][j], MT[n][A][b] = sum_j M_n[b][j]
// (likelihood of an unobserved child), MN[n][b][j] = M_n[b][j].  One thread
// per (node, row); preparing a plan on the device keeps tree set-up off the
// host's critical path when many trees arrive.
__global__ void k_compute_M(const double *__restrict__ V, const double *__restrict__ mu,
                            const double *__restrict__ t, const double *__restrict__ pi, int R, int A,
                            float *__restrict__ MT, float *__restrict__ MN) {
  const int total = R * A;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += gridDim.x * blockDim.x) {
    const int n = idx / A, b = idx % A;
    const double tn = t[n];
    const double isb = 1.0 / sqrt(pi[b]);
    double w[64];  // V[b][k] e^{mu_k t}, A <= 64
    for (int k = 0; k < A; ++k) w[k] = V[b * A + k] * exp(mu[k] * tn);
    double rs = 0.0;
    for (int j = 0; j < A; ++j) {
      double s = 0.0;
      for (int k = 0; k < A; ++k) s += w[k] * V[j * A + k];
      const double m = isb * sqrt(pi[j]) * s;
      MT[((size_t)n * (A + 1) + j) * A + b] = (float)m;
      MN[((size_t)n * A + b) * A + j] = (float)m;
      rs += m;
    }
    MT[((size_t)n * (A + 1) + A) * A + b] = (float)rs;
  }
}

// BF16 hi/lo operand tiles (A = 64) for the tensor-core walk, in the
// canonical K-major layout without swizzle (element (r, k) at byte
// (r&7)*16 + (r>>3)*1024 + (k&7)*2 + (k>>3)*128 of a 64 x 64 tile):
// per node n, B = M_n (rows b, K = j) and B = M_n^T (rows a, K = i); then
// Vd^T and Vu^T, each as three BF16 terms v1 = bf16(v), v2 = bf16(v - v1),
// v3 = bf16(v - v1 - v2).
__global__ void k_pack16(const float *__restrict__ MN, const float *__restrict__ Vd, const float *__restrict__ Vu,
                         int R, uint16_t *__restrict__ out) {
  const int ntiles = 2 * R + 2;
  const int total = ntiles * 4096;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += gridDim.x * blockDim.x) {
    const int tile = idx / 4096, e = idx % 4096, r = e / 64, k = e % 64;
    float v;
    if (tile < 2 * R) {
      const int n = tile / 2;
      v = (tile & 1) ? MN[(size_t)n * 4096 + k * 64 + r] : MN[(size_t)n * 4096 + r * 64 + k];
    } else {
      const float *Vt = (tile == 2 * R) ? Vd : Vu;
      v = Vt[k * 64 + r];  // B[r][k] = V[k][r]
    }
    const __nv_bfloat16 t1 = __float2bfloat16_rn(v);
    const float r1 = v - __bfloat162float(t1);
    const __nv_bfloat16 t2 = __float2bfloat16_rn(r1);
    const __nv_bfloat16 t3 = __float2bfloat16_rn(r1 - __bfloat162float(t2));
    const size_t base = (size_t)tile * 12288;  // elements: three terms of 4096
    const int off = ((r & 7) * 16 + (r >> 3) * 1024 + (k & 7) * 2 + (k >> 3) * 128) / 2;
    out[base + off] = __bfloat16_as_ushort(t1);
    out[base + 4096 + off] = __bfloat16_as_ushort(t2);
    out[base + 8192 + off] = __bfloat16_as_ushort(t3);
  }
}

// Leaf-branch weights K_n[code][k][l] = J_n[k][l] U~(code)_l (A <= 8; row
// stride A*A + 4), so
// that a leaf branch's J-weighted outer product needs one multiply per entry.
__global__ void k_compute_K(const float *__restrict__ J, const float *__restrict__ Ut, int R, int A,
                            float *__restrict__ K) {
  const int total = R * (A + 1) * A * A;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += gridDim.x * blockDim.x) {
    const int l = idx % A;
    const int k = (idx / A) % A;
    const int code = (idx / (A * A)) % (A + 1);
    const int n = idx / ((A + 1) * A * A);
    // rows of A*A + 4 floats (padding keeps per-thread rows on distinct banks)
    K[((size_t)n * (A + 1) + code) * (A * A + 4) + k * A + l] = J[(size_t)n * A * A + k * A + l] * Ut[code * A + l];
  }
}

// Device memory of plans comes from one library-owned stream-ordered pool per
// device: allocations and frees are ordered on CUDA streams (no implicit
// device-wide synchronisation, so creating or evicting a plan never stalls
// kernels of other streams), and freed blocks stay cached in the pool for
// the next plan up to SUBBY_POOL_KEEP_MB megabytes (default 2048).
uint64_t pool_keep_bytes() {
  const char *v = std::getenv("SUBBY_POOL_KEEP_MB");
  const long long mb = v ? std::atoll(v) : 2048;
  return (uint64_t)(mb > 0 ? mb : 0) << 20;
}

cudaMemPool_t lib_pool(int dev) {
  static std::mutex m;
  static cudaMemPool_t pools[64] = {};
  if (dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> g(m);
  if (!pools[dev]) {
    cudaMemPoolProps pr{};
    pr.allocType = cudaMemAllocationTypePinned;
    pr.location.type = cudaMemLocationTypeDevice;
    pr.location.id = dev;
    if (cudaMemPoolCreate(&pools[dev], &pr) != cudaSuccess) {
      cudaGetLastError();
      pools[dev] = nullptr;
      return nullptr;
    }
    uint64_t keep = pool_keep_bytes();
    cudaMemPoolSetAttribute(pools[dev], cudaMemPoolAttrReleaseThreshold, &keep);
  }
  return pools[dev];
}

cudaError_t pool_alloc(void **p, size_t bytes, cudaMemPool_t pool, cudaStream_t s) {
  return pool ? cudaMallocFromPoolAsync(p, bytes, pool, s) : cudaMallocAsync(p, bytes, s);
}

struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
  // Grow to `need` bytes in stream order on `s`; the old block is freed on
  // `s` once `after` (the plan's last use, possibly on another stream) has
  // completed.
  int grow(size_t need, cudaStream_t s, cudaMemPool_t pool, cudaEvent_t after) {
    if (need <= bytes) return 0;
    if (p) {
      if (after) cudaStreamWaitEvent(s, after, 0);
      cudaFreeAsync(p, s);
    }
    p = nullptr;
    bytes = 0;
    size_t want = need + need / 4;
    cudaError_t e = pool_alloc(&p, want, pool, s);
    if (e != cudaSuccess) {
      cudaGetLastError();
      e = pool_alloc(&p, need, pool, s);
      if (e != cudaSuccess) {
        cudaGetLastError();
        p = nullptr;
        return fail(SUBBY_ERR_NOMEM, "device allocation of " + std::to_string(need) + " bytes failed");
      }
      want = need;
    }
    bytes = want;
    return 0;
  }
  void release(cudaStream_t s) {
    if (p) cudaFreeAsync(p, s);
    p = nullptr;
    bytes = 0;
  }
};

}  // namespace

struct subby_plan {
  int R = 0, A = 0, nInt = 0, device = 0, nsm = 0;
  int root_is_leaf = 0;
  std::vector<int4> steps, slots;
  int nslots = 0;
  // tree program of k_tree (stored / derived node classification), and the
  // walk's program with every internal node stored
  std::vector<int4> prog, prog_w;
  int prog_steps = 0, prog_slots = 0, prog_w_steps = 0, prog_w_slots = 0;
  int4 *d_prog = nullptr, *d_prog_w = nullptr;
  std::vector<double> V, mu, pi, t;   // FP64 model and branch lengths (host)
  float f81_mu = 0.f;
  int f81_model = 0;   // M(t) has the F81 / JC closed form (checked on the host)
  // irreversible model: M(t) from the complex eigensystem (host FP64), and
  // the complex tables of the counts (J (R x A x A), V, V^-1, rate matrix)
  bool irrev = false;
  float2 *d_cx = nullptr;
  // per-branch models (rows): the tree's branches grouped by distinct model;
  // group g's complex tables at d_cx + (R + 13 g) A^2, its branches at
  // d_grp_br[grp_off[g] .. grp_off[g + 1]); counts use the exact formula
  bool rows = false;
  int ngroups = 1;
  std::vector<int> grp_off;
  int *d_grp_br = nullptr;
  float *d_gq = nullptr;   // complex-system plans: dM_n/dt = Re V diag(mu e^{mu t_n}) V^-1 (R x A x A)
  TableOffsets off{};
  float *d_tab = nullptr;
  double *d_tab64 = nullptr;
  uint16_t *d_tab16 = nullptr;   // A = 64: BF16 hi/lo operand tiles of the tensor-core walk
  int *d_err = nullptr;          // device status word (bounded waits that gave up)
  int4 *d_steps = nullptr, *d_slots = nullptr;
  size_t tab_bytes = 0;
  DevBuf work;     // scratch + gradient partials
  DevBuf io;       // staging of alignment/mask/outputs in host-pointer mode
  // host-pointer mode: copy queues of the column-chunk pipeline and its events
  cudaStream_t s_in = nullptr, s_out = nullptr;
  // stream-ordered lifetime: tables are built on s_prep; last_use marks the
  // end of the latest enqueued kernel, after which buffers may be freed
  cudaStream_t s_prep = nullptr;
  cudaEvent_t last_use = nullptr;
  cudaEvent_t ready = nullptr;   // end of the table preparation on s_prep
  bool used = false;
  cudaMemPool_t pool = nullptr;
  int grow(DevBuf &b, size_t need, cudaStream_t s) {
    return b.grow(need, s, pool, used ? last_use : nullptr);
  }
  std::vector<cudaEvent_t> ev;
  std::mutex lock;
};

namespace {

int validate_tree(const int32_t *parent, int R, std::vector<int> &left, std::vector<int> &right) {
  if (R < 1) return fail(SUBBY_ERR_TREE, "tree must have at least one node");
  if (parent[0] >= 0) return fail(SUBBY_ERR_TREE, "parentIndex[0] must be negative (root)");
  left.assign(R, -1);
  right.assign(R, -1);
  std::vector<int> cnt(R, 0);
  for (int n = 1; n < R; ++n) {
    const int p = parent[n];
    if (p < 0 || p >= n)
      return fail(SUBBY_ERR_TREE, "parentIndex[" + std::to_string(n) + "] = " + std::to_string(p) +
                                       " is not in [0, " + std::to_string(n) + ")");
    cnt[p]++;
    if (left[p] < 0) left[p] = n;           // first seen = smaller index
    else right[p] = n;
  }
  for (int n = 0; n < R; ++n)
    if (cnt[n] != 0 && cnt[n] != 2)
      return fail(SUBBY_ERR_TREE, "Node " + std::to_string(n) + " has " + std::to_string(cnt[n]) +
                                       " children; expected 0 or 2.");
  return 0;
}

}  // namespace

namespace subby {
void set_static_error(const char *why) { g_static_error = why; }
}  // namespace subby

extern "C" {

const char *subby_version(void) { return "subby_gb300 0.1 (sm_103a)"; }

const char *subby_strerror(int s) {
  switch (s) {
    case SUBBY_OK: return "ok";
    case SUBBY_ERR_ARG: return "invalid argument";
    case SUBBY_ERR_TREE: return "invalid tree";
    case SUBBY_ERR_UNSUPPORTED: return "unsupported size";
    case SUBBY_ERR_CUDA: return "CUDA error";
    case SUBBY_ERR_NOMEM: return "out of memory";
    case SUBBY_ERR_TIMEOUT: return "device wait timed out";
    default: return "unknown status";
  }
}

const char *subby_last_error(void) { return g_static_error ? g_static_error : g_last_error.c_str(); }

int subby_debug_set_kernel(int which) {
  if (which < 0 || which > 6) return fail(SUBBY_ERR_ARG, "kernel selector must be 0..6");
  g_kernel_sel = which;
  return SUBBY_OK;
}
int subby_last_launch_count(void) { return g_launches; }

int subby_debug_fail_waits(int polls) {
  if (polls < 0 || polls > 4096) return fail(SUBBY_ERR_ARG, "polls must be 0..4096");
  g_dbg_wait_polls.store(polls);
  return SUBBY_OK;
}

}  // extern "C"

namespace {

// Complex-eigensystem input: eigenvalues, V and V^-1 (interleaved re, im),
// one system for every branch, or (per_row) one per node n at offsets
// n A / n A^2 (complex values).
struct IrrevInput {
  const double *mu, *V, *Vi;
  int per_row;
};

int plan_create(const int32_t *parent, const double *dist, const double *evals, const double *evecs,
                const double *pi, int R, int A, subby_plan **out, const IrrevInput *ir) {
  clear_error();
  if (!out || !parent || !dist || !evals || !evecs || !pi) return fail(SUBBY_ERR_ARG, "null argument");
  *out = nullptr;
  if (!small_supported(A) && !warp_supported(A))
    return fail(SUBBY_ERR_UNSUPPORTED, "alphabet size A=" + std::to_string(A) +
                                            " not supported (2..8, 16, 20, 32, 64)");
  if (R > (1 << 20)) return fail(SUBBY_ERR_UNSUPPORTED, "tree too large");
  std::vector<int> left, right;
  if (int rc = validate_tree(parent, R, left, right)) return rc;
  for (int a = 0; a < A; ++a)
    if (!(pi[a] > 0.0)) return fail(SUBBY_ERR_ARG, "pi must be strictly positive");
  for (int n = 0; n < R; ++n)
    if (!(dist[n] >= 0.0) || !std::isfinite(dist[n]))
      return fail(SUBBY_ERR_ARG, "distances must be finite and non-negative");

  auto *P = new subby_plan();
  P->R = R;
  P->A = A;
  P->irrev = ir != nullptr;
  P->rows = ir && ir->per_row;
  cudaGetDevice(&P->device);
  cudaDeviceGetAttribute(&P->nsm, cudaDevAttrMultiProcessorCount, P->device);
  P->root_is_leaf = (R == 1);
  P->pool = lib_pool(P->device);
  {
    // the preparation stream has the highest priority, so the prologue
    // kernels start as soon as SMs free up when other work fills the device
    int lo = 0, hi = 0;
    cudaDeviceGetStreamPriorityRange(&lo, &hi);
    cudaError_t e0 = cudaStreamCreateWithPriority(&P->s_prep, cudaStreamNonBlocking, hi);
    if (e0 == cudaSuccess) e0 = cudaEventCreateWithFlags(&P->last_use, cudaEventDisableTiming);
    if (e0 == cudaSuccess) e0 = cudaEventCreateWithFlags(&P->ready, cudaEventDisableTiming);
    if (e0 != cudaSuccess) {
      subby_plan_destroy(P);
      return cuda_fail(e0, "plan stream");
    }
  }

  // DFS postorder of the internal nodes (children before parents).
  std::vector<int> order;
  if (R > 1) {
    std::vector<std::pair<int, int>> st;
    st.push_back({0, 0});
    while (!st.empty()) {
      auto &top = st.back();
      const int v = top.first;
      if (left[v] < 0) {  // leaf
        st.pop_back();
        continue;
      }
      if (top.second == 0) {
        top.second = 1;
        st.push_back({left[v], 0});
      } else if (top.second == 1) {
        top.second = 2;
        st.push_back({right[v], 0});
      } else {
        order.push_back(v);
        st.pop_back();
      }
    }
  }
  P->nInt = (int)order.size();
  std::vector<int> slot(R, -1);
  int ns = 0;
  for (int v : order)
    if (v != 0) slot[v] = ns++;
  P->nslots = ns;
  for (int v : order) {
    const int l = left[v], r = right[v];
    int flags = 0;
    if (left[l] < 0) flags |= kLeafL;
    if (left[r] < 0) flags |= kLeafR;
    if (v == 0) flags |= kRoot;
    P->steps.push_back(make_int4(v, l, r, flags));
    P->slots.push_back(make_int4(slot[v], slot[l], slot[r], 0));
  }

  // ---- tree program (k_tree, k_tree4): a node is DERIVED when both
  // children are leaves or stored (its CC is recomputed from them),
  // otherwise STORED.  The walk (k_walk, slots in global memory) takes the
  // program in which every internal node is stored: a derived node costs
  // the walk one more M product (a tensor-core round trip at A = 64) in the
  // outside pass, a slot only 2 A floats per column.
  auto build_prog = [&](bool store_all, std::vector<int4> &prog, int &prog_steps, int &prog_slots) {
    std::vector<int> kind(R, -1);  // -1 leaf, -2 derived, -3 root, >= 0 slot
    int nsl = 0;
    for (int v : order) {          // postorder of internal nodes
      if (v == 0) {
        kind[v] = -3;
        continue;
      }
      const bool ok = !store_all && (kind[left[v]] == -1 || kind[left[v]] >= 0) &&
                      (kind[right[v]] == -1 || kind[right[v]] >= 0);
      kind[v] = ok ? -2 : nsl++;
    }
    for (int v : order) {
      if (!(v == 0 || kind[v] >= 0)) continue;
      int4 c[2];
      int gk[4] = {0, 0, 0, 0};
      for (int side = 0; side < 2; ++side) {
        const int ch = side ? right[v] : left[v];
        const int kl = left[ch], kr = right[ch];
        c[side] = make_int4(ch, kind[ch], std::max(kl, 0), std::max(kr, 0));
        if (kind[ch] == -2) {
          gk[2 * side] = kind[kl];
          gk[2 * side + 1] = kind[kr];
        }
      }
      prog.push_back(make_int4(v, v == 0 ? -1 : kind[v], v == 0 ? 1 : 0, 0));
      prog.push_back(c[0]);
      prog.push_back(c[1]);
      prog.push_back(make_int4(gk[0], gk[1], gk[2], gk[3]));
    }
    prog_steps = (int)prog.size() / 4;
    prog_slots = nsl;
  };
  build_prog(false, P->prog, P->prog_steps, P->prog_slots);
  build_prog(true, P->prog_w, P->prog_w_steps, P->prog_w_slots);

  // ---- FP64 host tables
  P->t.assign(dist, dist + R);
  P->V.assign(evecs, evecs + (size_t)A * A);
  P->mu.assign(evals, evals + A);
  P->pi.assign(pi, pi + A);
  std::vector<double> sp(A), isp(A);
  double pi2 = 0.0;
  for (int a = 0; a < A; ++a) {
    sp[a] = std::sqrt(pi[a]);
    isp[a] = 1.0 / sp[a];
    pi2 += pi[a] * pi[a];
  }
  const double mu81 = 1.0 / (1.0 - pi2);
  P->f81_mu = (float)mu81;
  {
    // Is M(t) = e I + (1 - e) 1 pi^T, e = exp(-mu81 t)?  Checked in FP64 at
    // two branch lengths; then the large-alphabet walk uses the closed form.
    double worst = 0.0;
    std::vector<double> ek(A);
    for (double t : {0.3, 2.0}) {
      const double e = std::exp(-mu81 * t);
      for (int k = 0; k < A; ++k) ek[k] = std::exp(evals[k] * t);
      for (int i = 0; i < A; ++i)
        for (int j = 0; j < A; ++j) {
          double m = 0.0;
          for (int k = 0; k < A; ++k) m += evecs[i * A + k] * ek[k] * evecs[j * A + k];
          m *= std::sqrt(pi[j] / pi[i]);
          const double f = (i == j ? e : 0.0) + (1.0 - e) * pi[j];
          worst = std::max(worst, std::fabs(m - f));
        }
    }
    P->f81_model = !ir && std::isfinite(mu81) && worst < 1e-9;
  }

  TableOffsets &o = P->off;
  int cur = 0;
  auto take = [&](int n) {
    int at = cur;
    cur += (n + 3) & ~3;  // 16-byte aligned tables
    return at;
  };
  o.MT = take(R * (A + 1) * A);
  // small block, contiguous in this order: Vu, Vd, Ut, pi, S, V, root prior
  const int small_n = A * A + A * A + (A + 1) * A + A + A * A + A * A + A;
  o.Vu = take(small_n);
  o.Vd = o.Vu + A * A;
  o.Ut = o.Vd + A * A;
  o.pi = o.Ut + (A + 1) * A;
  o.S = o.pi + A;
  o.V = o.S + A * A;
  o.pi0 = o.V + A * A;
  o.MN = take(R * A * A);
  o.J = take(R * A * A);
  o.JT = take(R * A * A);
  o.F81 = take(R * 4);
  o.ME = take(R * A);
  o.K = (A <= 8) ? take(R * (A + 1) * (A * A + 4)) : 0;
  o.EF = take(R * 2);
  o.total = cur;
  // Host-computed parts only: the small block and the F81 / ME tables (MT,
  // MN, J, JT and K are written on the device by the prologue kernels).
  std::vector<float> hsm((size_t)small_n, 0.f), hfm((size_t)(o.ME + R * A - o.F81), 0.f), hef((size_t)R * 2);
  auto at = [&](int off) -> float & { return off >= o.F81 ? hfm[off - o.F81] : hsm[off - o.Vu]; };
  std::vector<double> E(A);
  // M(t) itself (MT / MN tables) is formed by k_compute_M on the device, in
  // FP64, right after the upload below.
  for (int n = 0; n < R; ++n) {
    const double t = dist[n];
    for (int k = 0; k < A; ++k) E[k] = std::exp(evals[k] * t);
    // F81 branch coefficients (subby/oracle/oracle.py:1226-1233)
    const double e = std::exp(-mu81 * t), pp = 1.0 - e;
    float *f = &at(o.F81 + n * 4);
    f[0] = (float)(t * e);
    f[1] = (float)(pp / mu81 - t * e);
    f[2] = (float)(t * (1.0 + e) - 2.0 * pp / mu81);
    f[3] = (float)t;
    hef[2 * n] = (float)e;
    hef[2 * n + 1] = (float)(-std::expm1(-mu81 * t));
    for (int k = 0; k < A; ++k) at(o.ME + n * A + k) = (float)(evals[k] * E[k]);
  }
  std::vector<double> S64((size_t)A * A);
  for (int i = 0; i < A; ++i)
    for (int j = 0; j < A; ++j) {
      double s = 0.0;
      for (int k = 0; k < A; ++k) s += evecs[i * A + k] * evals[k] * evecs[j * A + k];
      S64[i * A + j] = s;
    }
  for (int b = 0; b < A; ++b)
    for (int l = 0; l < A; ++l) {
      at(o.Vu + b * A + l) = (float)(sp[b] * evecs[b * A + l]);
      at(o.Vd + b * A + l) = (float)(isp[b] * evecs[b * A + l]);
      at(o.Ut + b * A + l) = (float)(sp[b] * evecs[b * A + l]);
      at(o.S + b * A + l) = (float)S64[b * A + l];
      at(o.V + b * A + l) = (float)evecs[b * A + l];
    }
  for (int l = 0; l < A; ++l) {
    double s = 0.0;
    for (int b = 0; b < A; ++b) s += sp[b] * evecs[b * A + l];
    at(o.Ut + A * A + l) = (float)s;
  }
  for (int a = 0; a < A; ++a) at(o.pi + a) = at(o.pi0 + a) = (float)pi[a];

  // ---- device upload
  auto cleanup = [&](int rc) {
    subby_plan_destroy(P);
    return rc;
  };
  P->tab_bytes = (size_t)o.total * sizeof(float);
  cudaStream_t qs = P->s_prep;
  cudaError_t e = pool_alloc((void **)&P->d_tab, P->tab_bytes, P->pool, qs);
  if (e != cudaSuccess) return cleanup(cuda_fail(e, "table allocation"));
  e = cudaMemcpyAsync(P->d_tab + o.Vu, hsm.data(), hsm.size() * sizeof(float), cudaMemcpyHostToDevice, qs);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(P->d_tab + o.F81, hfm.data(), hfm.size() * sizeof(float), cudaMemcpyHostToDevice, qs);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(P->d_tab + o.EF, hef.data(), hef.size() * sizeof(float), cudaMemcpyHostToDevice, qs);
  if (e != cudaSuccess) return cleanup(cuda_fail(e, "table upload"));
  e = pool_alloc((void **)&P->d_tab64, sizeof(double) * (2 * A * A + A + R + A), P->pool, qs);
  if (e != cudaSuccess) return cleanup(cuda_fail(e, "FP64 table allocation"));
  std::vector<double> t64((size_t)2 * A * A + A + R + A);
  std::copy(evecs, evecs + A * A, t64.begin());
  std::copy(S64.begin(), S64.end(), t64.begin() + A * A);
  std::copy(evals, evals + A, t64.begin() + 2 * A * A);
  std::copy(dist, dist + R, t64.begin() + 2 * A * A + A);
  std::copy(pi, pi + A, t64.begin() + 2 * A * A + A + R);
  e = cudaMemcpyAsync(P->d_tab64, t64.data(), sizeof(double) * t64.size(), cudaMemcpyHostToDevice, qs);
  if (e != cudaSuccess) return cleanup(cuda_fail(e, "FP64 table upload"));
  if (P->nInt > 0) {
    e = pool_alloc((void **)&P->d_steps, sizeof(int4) * P->nInt, P->pool, qs);
    if (e == cudaSuccess) e = pool_alloc((void **)&P->d_slots, sizeof(int4) * P->nInt, P->pool, qs);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(P->d_steps, P->steps.data(), sizeof(int4) * P->nInt, cudaMemcpyHostToDevice, qs);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(P->d_slots, P->slots.data(), sizeof(int4) * P->nInt, cudaMemcpyHostToDevice, qs);
    if (e != cudaSuccess) return cleanup(cuda_fail(e, "schedule upload"));
  }
  if (P->prog_steps > 0) {
    e = pool_alloc((void **)&P->d_prog, sizeof(int4) * P->prog.size(), P->pool, qs);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(P->d_prog, P->prog.data(), sizeof(int4) * P->prog.size(), cudaMemcpyHostToDevice, qs);
    if (e == cudaSuccess) e = pool_alloc((void **)&P->d_prog_w, sizeof(int4) * P->prog_w.size(), P->pool, qs);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(P->d_prog_w, P->prog_w.data(), sizeof(int4) * P->prog_w.size(), cudaMemcpyHostToDevice,
                          qs);
    if (e != cudaSuccess) return cleanup(cuda_fail(e, "program upload"));
  }
  std::vector<float> hMT, hMN, hGQ;
  std::vector<float2> hcx;
  std::vector<int> grp_br;
  if (ir) {
    // M_n = Re V diag(e^{mu t_n}) V^-1 and the complex tables, in FP64
    // (subby/oracle/oracle.py:474-534, 642-693); per-row systems for
    // per-branch models
    using cd = std::complex<double>;
    const size_t AA = (size_t)A * A;
    auto mu_of = [&](int n, int k) {
      const size_t q = (ir->per_row ? (size_t)n * A : 0) + k;
      return cd(ir->mu[2 * q], ir->mu[2 * q + 1]);
    };
    auto V_of = [&](int n, size_t e) {
      const size_t q = (ir->per_row ? (size_t)n * AA : 0) + e;
      return cd(ir->V[2 * q], ir->V[2 * q + 1]);
    };
    auto Vi_of = [&](int n, size_t e) {
      const size_t q = (ir->per_row ? (size_t)n * AA : 0) + e;
      return cd(ir->Vi[2 * q], ir->Vi[2 * q + 1]);
    };
    // groups of branches with identical systems (one group for a single model)
    std::vector<int> grp_of(R, 0), rep;  // rep[g]: a node of group g
    if (ir->per_row && R > 1) {
      for (int n = 1; n < R; ++n) {
        int g = -1;
        for (int h = 0; h < (int)rep.size() && g < 0; ++h) {
          const int m = rep[h];
          bool same = std::memcmp(ir->mu + 2 * (size_t)n * A, ir->mu + 2 * (size_t)m * A, 2 * A * sizeof(double)) == 0 &&
                      std::memcmp(ir->V + 2 * (size_t)n * AA, ir->V + 2 * (size_t)m * AA, 2 * AA * sizeof(double)) == 0 &&
                      std::memcmp(ir->Vi + 2 * (size_t)n * AA, ir->Vi + 2 * (size_t)m * AA, 2 * AA * sizeof(double)) == 0;
          if (same) g = h;
        }
        if (g < 0) {
          g = (int)rep.size();
          rep.push_back(n);
        }
        grp_of[n] = g;
      }
    } else {
      rep.push_back(R > 1 ? 1 : 0);
    }
    P->ngroups = (int)rep.size();
    P->grp_off.assign(P->ngroups + 1, 0);
    for (int n = 1; n < R; ++n) P->grp_off[grp_of[n] + 1]++;
    for (int g = 0; g < P->ngroups; ++g) P->grp_off[g + 1] += P->grp_off[g];
    grp_br.assign(std::max(R - 1, 1), 0);
    {
      std::vector<int> fill(P->grp_off.begin(), P->grp_off.end() - 1);
      for (int n = 1; n < R; ++n) grp_br[fill[grp_of[n]]++] = n;
    }
    hMT.assign((size_t)R * (A + 1) * A, 0.f);
    hMN.assign((size_t)R * A * A, 0.f);
    // float2: J (R A^2), then per group 13 A^2: V, Vinv, rate, Vinv^T, V^T;
    // FP64 pairs of V, Vinv, Vinv^T, V^T (two float2 slots per value)
    hcx.assign((size_t)(R + 13 * P->ngroups) * AA, make_float2(0.f, 0.f));
    std::vector<cd> E(A), w(A), wq(A);
    hGQ.assign((size_t)R * AA, 0.f);
    for (int n = 0; n < R; ++n) {
      const double t = dist[n];
      for (int k = 0; k < A; ++k) E[k] = std::exp(mu_of(n, k) * t);
      // dM_n/dt for the distance gradient
      for (int b = 0; b < A; ++b) {
        for (int k = 0; k < A; ++k) wq[k] = V_of(n, (size_t)b * A + k) * mu_of(n, k) * E[k];
        for (int j = 0; j < A; ++j) {
          cd sum = 0.0;
          for (int k = 0; k < A; ++k) sum += wq[k] * Vi_of(n, (size_t)k * A + j);
          hGQ[(size_t)n * AA + (size_t)b * A + j] = (float)sum.real();
        }
      }
      for (int b = 0; b < A; ++b) {
        for (int k = 0; k < A; ++k) w[k] = V_of(n, (size_t)b * A + k) * E[k];
        double rs = 0.0;
        for (int j = 0; j < A; ++j) {
          cd sum = 0.0;
          for (int k = 0; k < A; ++k) sum += w[k] * Vi_of(n, (size_t)k * A + j);
          const double m = sum.real();
          hMT[((size_t)n * (A + 1) + j) * A + b] = (float)m;
          hMN[((size_t)n * A + b) * A + j] = (float)m;
          rs += m;
        }
        hMT[((size_t)n * (A + 1) + A) * A + b] = (float)rs;
      }
      for (int k = 0; k < A; ++k)
        for (int l = 0; l < A; ++l) {
          const cd d = mu_of(n, k) - mu_of(n, l);
          const cd J = std::abs(d) < 1e-8 ? t * E[k] : (E[k] - E[l]) / d;
          hcx[((size_t)n * A + k) * A + l] = make_float2((float)J.real(), (float)J.imag());
        }
    }
    auto f2 = [](cd z) { return make_float2((float)z.real(), (float)z.imag()); };
    for (int g = 0; g < P->ngroups; ++g) {
      const int n = rep[g];
      float2 *cV = hcx.data() + (size_t)(R + 13 * g) * AA, *cVi = cV + AA, *cR = cVi + AA, *cViT = cR + AA,
             *cVT = cViT + AA;
      double *d64 = reinterpret_cast<double *>(cV + 5 * AA);  // 4 blocks of A^2 pairs
      auto put64 = [&](int blk, size_t e, cd z) {
        d64[2 * ((size_t)blk * AA + e)] = z.real();
        d64[2 * ((size_t)blk * AA + e) + 1] = z.imag();
      };
      for (int i = 0; i < A; ++i)
        for (int j = 0; j < A; ++j) {
          cd r = 0.0;
          for (int k = 0; k < A; ++k) r += V_of(n, (size_t)i * A + k) * mu_of(n, k) * Vi_of(n, (size_t)k * A + j);
          const size_t e = (size_t)i * A + j, et = (size_t)j * A + i;
          cV[e] = f2(V_of(n, e));
          cVi[e] = f2(Vi_of(n, e));
          cR[e] = f2(r);
          cViT[e] = f2(Vi_of(n, et));
          cVT[e] = f2(V_of(n, et));
          put64(0, e, V_of(n, e));
          put64(1, e, Vi_of(n, e));
          put64(2, e, Vi_of(n, et));
          put64(3, e, V_of(n, et));
        }
    }
    e = cudaMemcpyAsync(P->d_tab + o.MT, hMT.data(), hMT.size() * sizeof(float), cudaMemcpyHostToDevice, qs);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(P->d_tab + o.MN, hMN.data(), hMN.size() * sizeof(float), cudaMemcpyHostToDevice, qs);
    if (e == cudaSuccess) e = pool_alloc((void **)&P->d_cx, hcx.size() * sizeof(float2), P->pool, qs);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(P->d_cx, hcx.data(), hcx.size() * sizeof(float2), cudaMemcpyHostToDevice, qs);
    if (e == cudaSuccess) e = pool_alloc((void **)&P->d_gq, hGQ.size() * sizeof(float), P->pool, qs);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(P->d_gq, hGQ.data(), hGQ.size() * sizeof(float), cudaMemcpyHostToDevice, qs);
    if (e == cudaSuccess) e = pool_alloc((void **)&P->d_grp_br, grp_br.size() * sizeof(int), P->pool, qs);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(P->d_grp_br, grp_br.data(), grp_br.size() * sizeof(int), cudaMemcpyHostToDevice, qs);
    if (e != cudaSuccess) return cleanup(cuda_fail(e, "irreversible table upload"));
  }
  {
    const int tm = R * A;
    if (!ir)
      k_compute_M<<<std::max(1, std::min((tm + 127) / 128, 4096)), 128, 0, qs>>>(
          P->d_tab64, P->d_tab64 + 2 * A * A, P->d_tab64 + 2 * A * A + A, P->d_tab64 + 2 * A * A + A + R, R, A,
          P->d_tab + o.MT, P->d_tab + o.MN);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cleanup(cuda_fail(e, "M(t) prologue"));
    const int total = R * A * A;
    const int blk = 256, grd = std::max(1, std::min((total + blk - 1) / blk, 4096));
    k_compute_J<<<grd, blk, 0, qs>>>(P->d_tab64 + 2 * A * A, P->d_tab64 + 2 * A * A + A, R, A,
                              P->d_tab + o.J, P->d_tab + o.JT);
    e = cudaGetLastError();
    if (e == cudaSuccess && A <= 8) {
      const int tk = R * (A + 1) * A * A;
      k_compute_K<<<std::max(1, std::min((tk + 255) / 256, 4096)), 256, 0, qs>>>(P->d_tab + o.J, P->d_tab + o.Ut, R, A,
                                                                         P->d_tab + o.K);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess && A == 64) {
      e = pool_alloc((void **)&P->d_tab16, sizeof(uint16_t) * (size_t)(2 * R + 2) * 12288, P->pool, qs);
      if (e == cudaSuccess) {
        const int tt = (2 * R + 2) * 4096;
        k_pack16<<<std::max(1, std::min((tt + 255) / 256, 8192)), 256, 0, qs>>>(P->d_tab + o.MN, P->d_tab + o.Vd,
                                                                         P->d_tab + o.Vu, R, P->d_tab16);
        e = cudaGetLastError();
      }
    }
    if (e == cudaSuccess) e = pool_alloc((void **)&P->d_err, sizeof(int), P->pool, qs);
    if (e == cudaSuccess) e = cudaMemsetAsync(P->d_err, 0, sizeof(int), qs);
    // no host wait: runs order themselves after `ready` on their own streams
    if (e == cudaSuccess) e = cudaEventRecord(P->ready, qs);
    if (e != cudaSuccess) return cleanup(cuda_fail(e, "J(t) prologue"));
  }
  *out = P;
  return SUBBY_OK;
}

}  // namespace

extern "C" {

int subby_plan_create(const int32_t *parent, const double *dist, const double *evals,
                      const double *evecs, const double *pi, int R, int A, subby_plan **out) {
  return plan_create(parent, dist, evals, evecs, pi, R, A, out, nullptr);
}

int subby_plan_create_irrev(const int32_t *parent, const double *dist, const double *eigenvalues,
                            const double *eigenvectors, const double *eigenvectors_inv, const double *pi, int R,
                            int A, subby_plan **out) {
  clear_error();
  if (!eigenvalues || !eigenvectors || !eigenvectors_inv) return fail(SUBBY_ERR_ARG, "null argument");
  if (!(A >= 2 && A <= 64)) return fail(SUBBY_ERR_UNSUPPORTED, "alphabet size out of range");
  for (int i = 0; i < 2 * A; ++i)
    if (!std::isfinite(eigenvalues[i])) return fail(SUBBY_ERR_ARG, "eigenvalues must be finite");
  for (int i = 0; i < 2 * A * A; ++i)
    if (!std::isfinite(eigenvectors[i]) || !std::isfinite(eigenvectors_inv[i]))
      return fail(SUBBY_ERR_ARG, "eigenvectors must be finite");
  // the real eigensystem slots of the plan get an inert stand-in (zero
  // rates, identity vectors); M(t) and the count tables come from the
  // complex eigensystem
  std::vector<double> ev0((size_t)A, 0.0), eye((size_t)A * A, 0.0);
  for (int a = 0; a < A; ++a) eye[(size_t)a * A + a] = 1.0;
  const IrrevInput ir{eigenvalues, eigenvectors, eigenvectors_inv, 0};
  return plan_create(parent, dist, ev0.data(), eye.data(), pi, R, A, out, &ir);
}

int subby_plan_create_rows(const int32_t *parent, const double *dist, const double *eigenvalues,
                           const double *eigenvectors, const double *pi, int R, int A, subby_plan **out) {
  clear_error();
  if (!parent || !dist || !eigenvalues || !eigenvectors || !pi || !out) return fail(SUBBY_ERR_ARG, "null argument");
  if (!(A >= 2 && A <= 64) || R < 1) return fail(SUBBY_ERR_UNSUPPORTED, "alphabet size out of range");
  // node n's reversible system as V = diag(pi)^-1/2 W, V^-1 = W^T diag(pi)^1/2
  const size_t AA = (size_t)A * A;
  std::vector<double> mu((size_t)2 * R * A, 0.0), V(2 * R * AA, 0.0), Vi(2 * R * AA, 0.0);
  for (int n = 0; n < R; ++n) {
    const double *W = eigenvectors + (size_t)n * AA, *p = pi + (size_t)n * A;
    for (int a = 0; a < A; ++a) {
      if (!(p[a] > 0.0)) return fail(SUBBY_ERR_ARG, "pi must be strictly positive");
      mu[2 * ((size_t)n * A + a)] = eigenvalues[(size_t)n * A + a];
    }
    for (int i = 0; i < A; ++i)
      for (int k = 0; k < A; ++k) {
        V[2 * ((size_t)n * AA + (size_t)i * A + k)] = W[(size_t)i * A + k] / std::sqrt(p[i]);
        Vi[2 * ((size_t)n * AA + (size_t)k * A + i)] = W[(size_t)i * A + k] * std::sqrt(p[i]);
      }
  }
  std::vector<double> ev0((size_t)A, 0.0), eye(AA, 0.0);
  for (int a = 0; a < A; ++a) eye[(size_t)a * A + a] = 1.0;
  const IrrevInput ir{mu.data(), V.data(), Vi.data(), 1};
  // the root prior is node 0's pi
  return plan_create(parent, dist, ev0.data(), eye.data(), pi, R, A, out, &ir);
}

int subby_plan_destroy(subby_plan *P) {
  if (!P) return SUBBY_OK;
  int cur = 0;
  cudaGetDevice(&cur);
  if (cur != P->device) cudaSetDevice(P->device);
  // frees are ordered after the plan's last enqueued kernel; nothing here
  // waits for the device
  cudaStream_t s = P->s_prep;
  if (s && P->used) cudaStreamWaitEvent(s, P->last_use, 0);
  if (P->s_in) cudaStreamSynchronize(P->s_in);
  if (P->s_out) cudaStreamSynchronize(P->s_out);
  void *bufs[] = {P->d_tab, P->d_tab64, P->d_steps, P->d_slots, P->d_prog, P->d_prog_w, P->d_tab16, P->d_err,
                  P->d_cx, P->d_grp_br, P->d_gq};
  for (void *b : bufs)
    if (b) cudaFreeAsync(b, s);
  P->work.release(s);
  P->io.release(s);
  for (cudaEvent_t e : P->ev) cudaEventDestroy(e);
  if (P->last_use) cudaEventDestroy(P->last_use);
  if (P->ready) cudaEventDestroy(P->ready);
  if (P->s_in) cudaStreamDestroy(P->s_in);
  if (P->s_out) cudaStreamDestroy(P->s_out);
  if (s) cudaStreamDestroy(s);
  if (cur != P->device) cudaSetDevice(cur);
  delete P;
  return SUBBY_OK;
}

int subby_plan_status(subby_plan *P) {
  if (!P) return fail(SUBBY_ERR_ARG, "null plan");
  std::lock_guard<std::mutex> g(P->lock);
  if (!P->d_err) return SUBBY_OK;
  int cur = 0;
  cudaGetDevice(&cur);
  if (cur != P->device) cudaSetDevice(P->device);
  int dev_err = 0;
  cudaError_t e = cudaSuccess;
  if (P->used) e = cudaStreamWaitEvent(P->s_prep, P->last_use, 0);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&dev_err, P->d_err, sizeof(int), cudaMemcpyDeviceToHost, P->s_prep);
  if (e == cudaSuccess) e = cudaStreamSynchronize(P->s_prep);
  if (e == cudaSuccess && dev_err) {
    cudaMemsetAsync(P->d_err, 0, sizeof(int), P->s_prep);
    e = cudaStreamSynchronize(P->s_prep);
  }
  if (cur != P->device) cudaSetDevice(cur);
  if (e != cudaSuccess) return cuda_fail(e, "plan status");
  if (dev_err) return fail(SUBBY_ERR_TIMEOUT, "a bounded device wait gave up in " + std::to_string(dev_err) +
                                                 " CTA(s) since the last status check");
  return SUBBY_OK;
}

int subby_plan_set_root_prior(subby_plan *P, const double *root_prior) {
  clear_error();
  if (!P || !root_prior) return fail(SUBBY_ERR_ARG, "null argument");
  const int A = P->A;
  std::vector<float> h(A);
  for (int a = 0; a < A; ++a) {
    if (!(root_prior[a] > 0.0) || !std::isfinite(root_prior[a]))
      return fail(SUBBY_ERR_ARG, "root prior entries must be positive and finite");
    h[a] = (float)root_prior[a];
  }
  std::lock_guard<std::mutex> g(P->lock);
  int cur = 0;
  cudaGetDevice(&cur);
  if (cur != P->device) cudaSetDevice(P->device);
  // after every enqueued use of the tables; later runs wait for `ready`
  cudaError_t e = P->used ? cudaStreamWaitEvent(P->s_prep, P->last_use, 0) : cudaSuccess;
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(P->d_tab + P->off.pi0, h.data(), sizeof(float) * A, cudaMemcpyHostToDevice, P->s_prep);
  if (e == cudaSuccess) e = cudaEventRecord(P->ready, P->s_prep);
  if (e == cudaSuccess) e = cudaStreamSynchronize(P->s_prep);
  if (cur != P->device) cudaSetDevice(cur);
  if (e != cudaSuccess) return cuda_fail(e, "root prior upload");
  return SUBBY_OK;
}

int subby_plan_trim(subby_plan *P) {
  if (!P) return fail(SUBBY_ERR_ARG, "null plan");
  std::lock_guard<std::mutex> g(P->lock);
  int cur = 0;
  cudaGetDevice(&cur);
  if (cur != P->device) cudaSetDevice(P->device);
  if (P->used) cudaStreamWaitEvent(P->s_prep, P->last_use, 0);
  P->work.release(P->s_prep);
  P->io.release(P->s_prep);
  if (cur != P->device) cudaSetDevice(cur);
  return SUBBY_OK;
}

}  // extern "C"

namespace subby {
// Serving support (server.cu): enqueue on `s` a copy of the plan's device
// status word into the pinned host word *h (valid once `s` passes this
// point) followed by clearing the device word, so a completed job's status
// is known without a blocking copy.
int plan_status_async(subby_plan *P, int *h, cudaStream_t s) {
  if (!P || !h) return SUBBY_ERR_ARG;
  if (!P->d_err) {
    *h = 0;
    return SUBBY_OK;
  }
  cudaError_t e = cudaMemcpyAsync(h, P->d_err, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(P->d_err, 0, sizeof(int), s);
  return e == cudaSuccess ? SUBBY_OK : SUBBY_ERR_CUDA;
}
}  // namespace subby

extern "C" {

size_t subby_plan_device_bytes(const subby_plan *P) {
  if (!P) return 0;
  return P->tab_bytes + P->work.bytes + P->io.bytes + sizeof(int4) * 2 * P->nInt;
}

}  // extern "C"

namespace {

struct Launch {
  KParams kp{};
  int kernel = 0;        // 0 small (thread/column), 1 warp/column, 2 tree program
  bool global_slots = false;
  int store = 0;         // k_tree slot storage: 0 shared, 1 global, 2 tensor memory
  bool small = true;
  int grid = 1, block = 128;
  size_t smem = 0;
  int nworkers = 0;
};

// Shared-memory tables and grid size of the small (thread-per-column) kernel.
int plan_small(subby_plan *P, int mode, int C, Launch &L) {
  const int A = P->A, R = P->R;
  KParams &k = L.kp;
  int ntab = 0, sofs = 0;
  auto add = [&](int gofs, int n) {
    k.stab[ntab++] = SmemTable{gofs, sofs, n};
    sofs += (n + 3) & ~3;
  };
  const TableOffsets &o = P->off;
  add(o.MT, R * (A + 1) * A);
  add(o.Vu, A * A * 4 + (A + 1) * A + A);
  if (mode & (kModeCounts | kModeGrad)) {
    add(o.MN, R * A * A);
    if (mode & kModeF81) add(o.F81, R * 4);
    else add(o.J, R * A * A);
    if (mode & kModeGrad) add(o.ME, R * A);
  }
  k.ntab = ntab;
  k.smem_steps = sofs;
  sofs += 4 * P->nInt;
  k.smem_slots = sofs;
  sofs += 4 * P->nInt;
  L.smem = (size_t)sofs * sizeof(float);
  int maxsm = 0;
  cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, P->device);
  if (L.smem > (size_t)maxsm)
    return fail(SUBBY_ERR_UNSUPPORTED, "tree too large for the shared-memory tables (R=" +
                                           std::to_string(R) + ", A=" + std::to_string(A) + ")");
  L.small = true;
  L.block = small_block();
  // occupancy-limited persistent grid
  int per_sm = std::max(1, (int)(((size_t)maxsm + 1024) / (L.smem + 1024)));
  per_sm = std::min(per_sm, 2048 / L.block);
  int want = (C + L.block - 1) / L.block;
  L.grid = std::max(1, std::min(want, P->nsm * per_sm));
  L.nworkers = L.grid * L.block;
  return 0;
}

int plan_warp(subby_plan *P, int mode, int C, Launch &L) {
  (void)mode;
  L.small = false;
  L.block = warp_block();
  const int wpb = L.block / 32;
  L.smem = warp_smem_per_warp(P->A) * wpb;
  L.kp.ntab = 0;
  L.kp.smem_steps = -1;
  int maxsm = 0;
  cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, P->device);
  int per_sm = std::max(1, (int)((size_t)maxsm / (L.smem + 1024)));
  per_sm = std::min(per_sm, 8);
  int want = (C + wpb - 1) / wpb;
  L.grid = std::max(1, std::min(want, P->nsm * per_sm));
  L.nworkers = L.grid * wpb;
  return 0;
}

// Tree-program kernel: one CTA per SM, as many threads as the per-column slot
// state allows in shared memory (global-memory slots when even 64 do not fit).
int plan_tree(subby_plan *P, int mode, int C, Launch &L) {
  const int A = P->A, R = P->R;
  KParams &k = L.kp;
  int ntab = 0, sofs = 0;
  auto add = [&](int gofs, int n) {
    k.stab[ntab++] = SmemTable{gofs, sofs, n};
    sofs += (n + 3) & ~3;
  };
  const TableOffsets &o = P->off;
  add(o.MT, R * (A + 1) * A);
  add(o.Vu, A * A * 4 + (A + 1) * A + A);
  if (mode & kModeCounts) {
    if (mode & kModeF81) add(o.F81, R * 4);
    else add(o.J, R * A * A);
  }
  k.ntab = ntab;
  k.smem_steps = sofs;
  sofs += 16 * P->prog_steps;
  int maxsm = 0;
  cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, P->device);
  const size_t fixed = (size_t)sofs * sizeof(float);
  const size_t per_thread = (size_t)P->prog_slots * (A + 1) * sizeof(float);
  if (fixed + 1024 > (size_t)maxsm)
    return fail(SUBBY_ERR_UNSUPPORTED, "tree too large for the shared-memory tables (R=" +
                                           std::to_string(R) + ", A=" + std::to_string(A) + ")");
  const int kMaxThreads = 256;
  int threads = kMaxThreads;
  if (per_thread > 0) threads = (int)(((size_t)maxsm - fixed) / per_thread);
  threads = std::min(kMaxThreads, threads / 32 * 32);
  L.kernel = 2;
  L.small = false;
  // Tensor memory holds the slot vectors when A = 4 and they fit (512
  // columns per SM shared by 128 or 256 threads); the slot words stay in
  // shared memory.  Otherwise shared-memory slots, else global-memory slots.
  int tm_threads = 0;
  if (A == 4 && P->prog_slots > 0 && g_kernel_sel != 2 && g_kernel_sel != 3) {
    for (int t : {256, 128}) {
      if (P->prog_slots * 4 <= 512 / (t / 128) &&
          fixed + (size_t)P->prog_slots * t * sizeof(int) + 1024 <= (size_t)maxsm) {
        tm_threads = t;
        break;
      }
    }
  }
  if (tm_threads) {
    L.store = 2;
    L.block = tm_threads;
    k.smem_slots = -1;
    k.smem_words = sofs;
    sofs += P->prog_slots * tm_threads;
    // at least half of the SM's shared memory, so that exactly one CTA (the
    // owner of all 512 TMEM columns) is resident per SM
    sofs = std::max(sofs, (maxsm / 2 + 4096) / 4);
  } else if (threads >= 64 && g_kernel_sel != 3) {
    L.store = 0;
    L.block = threads;
    k.smem_slots = sofs;
    sofs += P->prog_slots * threads * A;
    k.smem_words = sofs;
    sofs += P->prog_slots * threads;
  } else {
    L.store = 1;
    L.block = 256;
    k.smem_slots = -1;
    k.smem_words = -1;
  }
  L.global_slots = (L.store == 1);
  L.smem = (size_t)sofs * sizeof(float);
  const int want = (C + L.block - 1) / L.block;
  L.grid = std::max(1, std::min(want, P->nsm));
  L.nworkers = L.grid * L.block;
  k.prog = P->d_prog;
  k.nsteps = P->prog_steps;
  k.nslots = P->prog_slots;
  return 0;
}

// A = 4 tree kernel: all tables in shared memory, slot vectors in tensor
// memory, one CTA of 256 (or 128) threads per SM.  Returns 1 when the plan
// does not fit (the caller then uses the generic tree kernel).
int plan_tree4(subby_plan *P, int mode, int C, Launch &L) {
  const int R = P->R;
  if (P->A != 4 || g_kernel_sel != 0) return 1;
  KParams &k = L.kp;
  int ntab = 0, sofs = 0;
  auto add = [&](int gofs, int n) {
    k.stab[ntab++] = SmemTable{gofs, sofs, n};
    sofs += (n + 3) & ~3;
  };
  const TableOffsets &o = P->off;
  const bool f81 = (mode & kModeF81) != 0;
  add(o.MT, R * 20);
  add(o.Vu, 16 * 4 + 20 + 4 + 4);
  if (f81) add(o.F81, R * 4);
  else add(o.J, R * 16);
  if (!f81) add(o.K, R * 100);
  // observation rows (filled in the kernel): 5 x 4 + 5, rounded up
  k.stab[ntab++] = SmemTable{0, sofs, 0};
  sofs += 28;
  k.ntab = ntab;
  k.smem_steps = sofs;
  sofs += 16 * P->prog_steps;
  int maxsm = 0;
  cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, P->device);
  int threads = 0;
  for (int t : {256, 128}) {
    if (P->prog_slots * 4 <= 512 / (t / 128) &&
        (size_t)(sofs + P->prog_slots * t) * sizeof(float) + 1024 <= (size_t)maxsm) {
      threads = t;
      break;
    }
  }
  if (!threads) return 1;
  k.smem_slots = -1;
  k.smem_words = sofs;
  sofs += P->prog_slots * threads;
  sofs = std::max(sofs, (maxsm / 2 + 4096) / 4);  // one CTA (TMEM owner) per SM
  L.kernel = 3;
  L.small = false;
  L.store = 2;
  L.block = threads;
  L.smem = (size_t)sofs * sizeof(float);
  const int want = (C + L.block - 1) / L.block;
  L.grid = std::max(1, std::min(want, P->nsm));
  L.nworkers = L.grid * L.block;
  k.prog = P->d_prog;
  k.nsteps = P->prog_steps;
  k.nslots = P->prog_slots;
  return 0;
}

// Large alphabets (A = 16, 20, 32, 64): k_walk (tree walk, 128 columns per
// CTA, stored-node slots in global memory) then, for Counts, k_acc over the
// staged per-branch vectors.  Columns are processed in chunks so that the
// staging (2 (R-1) A floats per column) stays within kStageBudget bytes.
constexpr size_t kStageBudget = size_t(4) << 30;

// Marks the end of the work just enqueued on `stream` as the plan's last use.
int mark_use(subby_plan *P, cudaStream_t stream) {
  CU(cudaEventRecord(P->last_use, stream));
  P->used = true;
  return 0;
}

// Parameters of the walk (k_walk) and the kernels that consume its staging.
// A walk with an outside pass and costly M products (A >= 16, not the F81
// closed form) runs the program in which every internal node is stored (its
// M product is not repeated in the outside pass); other walks run the
// derived-node program (no slot round trips through global memory for nodes
// whose parent can recompute them cheaply).
KParams walk_params(const subby_plan *P, const int32_t *d_aln, int C, int mode, int mask_mode,
                    const uint8_t *d_mask, float *d_logL, float *d_counts, float *d_root,
                    bool outside = true) {
  KParams k{};
  k.aln = d_aln;
  k.C = C;
  k.R = P->R;
  k.A = P->A;
  k.nInt = P->nInt;
  k.mode = mode;
  k.mask_mode = mask_mode;
  k.mask = d_mask;
  k.tab = P->d_tab;
  k.tab64 = P->d_tab64;
  k.off = P->off;
  k.root_is_leaf = P->root_is_leaf;
  k.f81_mu = P->f81_mu;
  k.f81_model = P->f81_model;
  k.logL = d_logL;
  k.counts = d_counts;
  k.rootp = d_root;
  const bool all = outside && P->A >= 16 && !P->f81_model;
  k.prog = all ? P->d_prog_w : P->d_prog;
  k.noderiv = all ? 1 : 0;
  k.nsteps = all ? P->prog_w_steps : P->prog_steps;
  k.nslots = std::max(all ? P->prog_w_slots : P->prog_slots, 1);
  k.tab16 = P->d_tab16;
  k.err = P->d_err;
  k.dbg_wait_polls = g_dbg_wait_polls.load();
  return k;
}

int run_big(subby_plan *P, const int32_t *d_aln, int C, float *d_logL, float *d_counts, float *d_root,
            int mode, int mask_mode, const uint8_t *d_mask, cudaStream_t stream) {
  const int A = P->A, R = P->R;
  KParams k = walk_params(P, d_aln, C, mode, mask_mode, d_mask, d_logL, d_counts, d_root,
                          (mode & kModeCounts) != 0 && R > 1);
  // 5: tensor-core walk with the CUDA-core back-transform; 6: CUDA-core walk
  // with the tensor-core back-transform (test hooks)
  const bool tc = (A == 64) && P->d_tab16 && (g_kernel_sel == 0 || g_kernel_sel == 5);
  const bool tcb = (A == 64) && P->d_tab16 && (g_kernel_sel == 0 || g_kernel_sel == 6);
  const int tile = big_tile();
  const int H = (A + 31) / 32;
  const bool counts = (mode & kModeCounts) != 0 && R > 1;
  // chunk of columns (multiple of the tile) bounded by the staging budget
  int chunk = C;
  if (counts) {
    const size_t per_col = (size_t)2 * (R - 1) * A * sizeof(float);
    size_t cmax = std::max<size_t>(tile, kStageBudget / per_col);
    cmax = cmax / tile * tile;
    // equal chunks (whole tiles), so the last one is not a sliver
    const size_t nch = ((size_t)C + cmax - 1) / cmax;
    const size_t even = ((size_t)C + nch - 1) / nch;
    chunk = (int)std::min<size_t>((size_t)C, (even + tile - 1) / tile * tile);
  }
  const int walk_grid = std::max(1, std::min((chunk + tile - 1) / tile, P->nsm * (H == 2 ? 1 : 2)));
  const size_t slot_floats = (size_t)walk_grid * k.nslots * tile * A;
  const size_t slot_ints = (size_t)walk_grid * k.nslots * tile * 2;  // a word per column half
  const size_t stage_floats = counts ? (size_t)(R - 1) * chunk * A : 0;
  // A = 64 F81 counts on the tensor cores: per-branch scalars staged too
  const bool f81tc = counts && (mode & kModeF81) && tc && !(mode & kModeBranch);
  const size_t stage_c_floats = f81tc ? (size_t)(R - 1) * chunk * 2 : 0;
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  int rc;
  if ((rc = P->grow(P->work,
                    al(slot_floats * 4) + al(slot_ints * 4) + 2 * al(stage_floats * 4) + al(stage_c_floats * 4) + 256,
                    stream)))
    return rc;
  char *base = (char *)P->work.p;
  k.scrV = (float *)base;
  base += al(slot_floats * 4);
  k.scrW = (int *)base;
  base += al(slot_ints * 4);
  float *sa = (float *)base;
  base += al(stage_floats * 4);
  float *sb = (float *)base;
  base += al(stage_floats * 4);
  k.stage_c = f81tc ? (float2 *)base : nullptr;
  const int wmode = counts ? ((mode & kModeF81) ? 2 : 1) : 0;
  if (!counts && (mode & kModeCounts)) {
    // a single-node tree has no branch: counts are zero
    cudaError_t e = cudaMemsetAsync(d_counts, 0, (size_t)A * A * C * sizeof(float), stream);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync");
  }
  for (int c0 = 0; c0 < C; c0 += chunk) {
    const int cc = std::min(chunk, C - c0);
    int lr = launch_walk(k, A, wmode, tc, sa, sb, c0, cc, walk_grid, stream);
    if (lr != 0) return fail(SUBBY_ERR_CUDA, std::string("walk launch failed: ") + cudaGetErrorString((cudaError_t)lr));
    g_launches += 1;
    if (counts) {
      const int G = big_acc_group(A);
      const long long items = (long long)(cc + G - 1) / G * ((mode & kModeBranch) ? (R - 1) : 1);
      const int agrid = (int)std::max<long long>(1, std::min<long long>(items, P->nsm));
      lr = f81tc ? launch_acc_f81_tc(k, sa, sb, k.stage_c, c0, cc, agrid, stream)
                 : launch_acc(k, A, (mode & kModeF81) != 0, tcb, sa, sb, c0, cc, agrid, stream);
      if (lr != 0) return fail(SUBBY_ERR_CUDA, std::string("accumulate launch failed: ") + cudaGetErrorString((cudaError_t)lr));
      g_launches += 1;
    }
  }
  return mark_use(P, stream);
}

// Node / branch posteriors.  The walk (mode 3) writes the node posteriors of
// every non-root node from the D_n, U_n it holds and, for the branch
// posteriors, stages D_n s_n and U_n (raw basis) for k_post; the root's row
// is the walk's RootProb (mode 0 alone for node 0 or a one-node tree).
// node < 0: every node (branch 0 of the branch posteriors zero); node > 0:
// that node only, in row 0.  Columns in chunks bounded by the staging budget.
int run_post(subby_plan *P, const int32_t *d_aln, int C, int node, float *d_node, float *d_br,
             cudaStream_t stream) {
  const int A = P->A, R = P->R;
  const bool all = node < 0;
  if (all && d_br) CU(cudaMemsetAsync(d_br, 0, (size_t)A * A * C * sizeof(float), stream));
  const bool outside = R > 1 && node != 0;
  if (!outside && !d_node) return mark_use(P, stream);
  Launch L4;
  if (A == 4 && R > 1 && plan_tree4(P, 0, C, L4) == 0) {
    // the A = 4 tree-program kernel writes both posteriors directly
    KParams &k = L4.kp;
    k.aln = d_aln;
    k.C = C;
    k.R = R;
    k.A = A;
    k.nInt = P->nInt;
    k.mode = (node <= 0 && d_node) ? kModeRootProb : 0;
    k.mask_mode = kMaskNone;
    k.tab = P->d_tab;
    k.tab64 = P->d_tab64;
    k.off = P->off;
    k.steps = P->d_steps;
    k.slots = P->d_slots;
    k.root_is_leaf = P->root_is_leaf;
    k.f81_mu = P->f81_mu;
    k.nworkers = L4.nworkers;
    k.rootp = node <= 0 ? d_node : nullptr;
    k.npost = d_node;
    k.npost_node = node;
    k.bpost = d_br;
    const int lr = launch_tree4_post(k, L4.grid, L4.block, L4.smem, stream);
    if (lr != 0) return fail(SUBBY_ERR_CUDA, std::string("kernel launch failed: ") + cudaGetErrorString((cudaError_t)lr));
    g_launches += 1;
    return mark_use(P, stream);
  }
  const bool stage = outside && d_br;
  const int mode = (node <= 0 && d_node) ? kModeRootProb : 0;
  KParams k = walk_params(P, d_aln, C, mode, SUBBY_MASK_NONE, nullptr, nullptr, nullptr, node <= 0 ? d_node : nullptr,
                          outside);
  k.npost = d_node;
  k.npost_node = node;
  const bool tc = (A == 64) && P->d_tab16 && (g_kernel_sel == 0 || g_kernel_sel == 5);
  const int tile = big_tile();
  const int H = (A + 31) / 32;
  int chunk = C;
  if (stage) {
    const size_t per_col = (size_t)2 * (R - 1) * A * sizeof(float);
    size_t cmax = std::max<size_t>(tile, kStageBudget / per_col);
    cmax = cmax / tile * tile;
    const size_t nch = ((size_t)C + cmax - 1) / cmax;
    const size_t even = ((size_t)C + nch - 1) / nch;
    chunk = (int)std::min<size_t>((size_t)C, (even + tile - 1) / tile * tile);
  }
  const int per_sm = A <= 8 ? 8 : (H == 2 ? 1 : 2);
  const int walk_grid = std::max(1, std::min((chunk + tile - 1) / tile, P->nsm * per_sm));
  const size_t slot_floats = (size_t)walk_grid * k.nslots * tile * A;
  const size_t slot_ints = (size_t)walk_grid * k.nslots * tile * 2;  // a word per column half
  const size_t stage_floats = stage ? (size_t)(R - 1) * chunk * A : 0;
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  int rc;
  if ((rc = P->grow(P->work, al(slot_floats * 4) + al(slot_ints * 4) + 2 * al(stage_floats * 4) + 256, stream)))
    return rc;
  char *base = (char *)P->work.p;
  k.scrV = (float *)base;
  base += al(slot_floats * 4);
  k.scrW = (int *)base;
  base += al(slot_ints * 4);
  float *sa = stage ? (float *)base : nullptr;
  base += al(stage_floats * 4);
  float *sb = stage ? (float *)base : nullptr;
  const int n_lo = all ? 1 : node, n_hi = all ? R : node + 1;
  const int row_off = all ? 0 : node;
  for (int c0 = 0; c0 < C; c0 += chunk) {
    const int cc = std::min(chunk, C - c0);
    int lr = launch_walk_post(k, A, outside ? 3 : 0, tc, sa, sb, c0, cc, walk_grid, stream);
    if (lr != 0) return fail(SUBBY_ERR_CUDA, std::string("walk launch failed: ") + cudaGetErrorString((cudaError_t)lr));
    g_launches += 1;
    if (!stage) continue;
    const long long items = (long long)(cc + post_tile() - 1) / post_tile() * (n_hi - n_lo);
    const int pgrid = (int)std::max<long long>(1, std::min<long long>(items, (long long)P->nsm * 8));
    lr = launch_post(k, A, sa, sb, c0, cc, n_lo, n_hi, row_off, d_br, pgrid, stream);
    if (lr != 0) return fail(SUBBY_ERR_CUDA, std::string("posterior launch failed: ") + cudaGetErrorString((cudaError_t)lr));
    g_launches += 1;
  }
  return mark_use(P, stream);
}

// Irreversible models, Counts / BranchCounts: the walk (mode 3) stages
// D_n s_n and U_n in the raw basis (LogLike / RootProb from its inside
// pass), k_acc_cx does the complex accumulation and back-transform.
int run_cx(subby_plan *P, const int32_t *d_aln, int C, float *d_logL, float *d_counts, float *d_root, int mode,
           int mask_mode, const uint8_t *d_mask, cudaStream_t stream) {
  // A = 64: C buffered per chunk (per branch for per-branch counts) and
  // back-transformed in FP64 by k_bt_cx
  const int A = P->A, R = P->R;
  if (!cx_supported(A) || !post_supported(A))
    return fail(SUBBY_ERR_UNSUPPORTED, "irreversible counts are implemented for A = 4, 8, 16, 20, 32, 64");
  if (mode & kModeF81) return fail(SUBBY_ERR_ARG, "the F81 fast path is reversible-only");
  const bool pb = (mode & kModeBranch) != 0;
  const bool counts = R > 1;
  if (!counts && !pb) CU(cudaMemsetAsync(d_counts, 0, (size_t)A * A * C * sizeof(float), stream));
  KParams k = walk_params(P, d_aln, C, mode & (kModeLogLike | kModeRootProb), mask_mode, d_mask, d_logL, d_counts,
                          d_root);
  k.cx = P->d_cx;
  k.cx_exact = P->rows || (mode & kModeIrrevExact) != 0;
  k.npost = nullptr;
  k.npost_node = -1;
  const bool bt64 = cx_bt64(A) && !P->rows;   // per-branch reversible systems are well conditioned
  const bool tc = (A == 64) && P->d_tab16 && (g_kernel_sel == 0 || g_kernel_sel == 5);
  const int tile = big_tile();
  const int H = (A + 31) / 32;
  int chunk = C;
  if (counts) {
    const size_t per_col = (size_t)2 * (R - 1) * A * sizeof(float);
    size_t cmax = std::max<size_t>(tile, kStageBudget / per_col);
    cmax = cmax / tile * tile;
    const size_t nch = ((size_t)C + cmax - 1) / cmax;
    const size_t even = ((size_t)C + nch - 1) / nch;
    chunk = (int)std::min<size_t>((size_t)C, (even + tile - 1) / tile * tile);
  }
  const int per_sm = A <= 8 ? 8 : (H == 2 ? 1 : 2);
  const int walk_grid = std::max(1, std::min((chunk + tile - 1) / tile, P->nsm * per_sm));
  const size_t slot_floats = (size_t)walk_grid * k.nslots * tile * A;
  const size_t slot_ints = (size_t)walk_grid * k.nslots * tile * 2;  // a word per column half
  const size_t stage_floats = counts ? (size_t)(R - 1) * chunk * A : 0;
  const size_t cbuf_bytes = (counts && bt64) ? (size_t)chunk * A * A * sizeof(float2) : 0;
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  int rc;
  if ((rc = P->grow(P->work, al(slot_floats * 4) + al(slot_ints * 4) + 2 * al(stage_floats * 4) + al(cbuf_bytes) + 256,
                    stream)))
    return rc;
  char *base = (char *)P->work.p;
  k.scrV = (float *)base;
  base += al(slot_floats * 4);
  k.scrW = (int *)base;
  base += al(slot_ints * 4);
  float *sa = counts ? (float *)base : nullptr;
  base += al(stage_floats * 4);
  float *sb = counts ? (float *)base : nullptr;
  base += al(stage_floats * 4);
  float2 *cbuf = cbuf_bytes ? (float2 *)base : nullptr;
  const int G = cx_columns_per_cta(A);
  for (int c0 = 0; c0 < C; c0 += chunk) {
    const int cc = std::min(chunk, C - c0);
    int lr = launch_walk_post(k, A, counts ? 3 : 0, tc, sa, sb, c0, cc, walk_grid, stream);
    if (lr != 0) return fail(SUBBY_ERR_CUDA, std::string("walk launch failed: ") + cudaGetErrorString((cudaError_t)lr));
    g_launches += 1;
    if (!counts) continue;
    const long long groups = (cc + G - 1) / G;
    const int grid = (int)std::max<long long>(1, std::min<long long>(groups, (long long)P->nsm * 2));
    if (!bt64) {
      // one launch per group of branches sharing a system; the summed
      // counts of later groups add to the earlier ones
      for (int g = 0; g < P->ngroups; ++g) {
        KParams kg = k;
        kg.cx_tab = P->d_cx + (size_t)(R + 13 * g) * A * A;
        kg.cx_br = P->d_grp_br + P->grp_off[g];
        kg.cx_accum = g > 0;
        const int nb = P->grp_off[g + 1] - P->grp_off[g];
        lr = launch_acc_cx(kg, A, pb, sa, sb, c0, cc, 0, nb, nullptr, grid, stream);
        if (lr != 0)
          return fail(SUBBY_ERR_CUDA, std::string("accumulate launch failed: ") + cudaGetErrorString((cudaError_t)lr));
        g_launches += 1;
      }
      continue;
    }
    k.cx_tab = P->d_cx + (size_t)R * A * A;
    k.cx_br = P->d_grp_br;
    k.cx_accum = 0;
    // FP64 back-transform: all branches at once, or branch by branch
    const int bgrid = std::max(1, std::min(cc, P->nsm));
    for (int n = pb ? 1 : 0; n < (pb ? R : 1); ++n) {
      // branch list d_grp_br holds 1 .. R-1 in order for a single system
      lr = launch_acc_cx(k, A, false, sa, sb, c0, cc, pb ? n - 1 : 0, pb ? n : R - 1, cbuf, grid, stream);
      if (lr == 0) lr = launch_bt_cx(k, A, cbuf, c0, cc, pb ? n : 0, bgrid, stream);
      if (lr != 0)
        return fail(SUBBY_ERR_CUDA, std::string("accumulate launch failed: ") + cudaGetErrorString((cudaError_t)lr));
      g_launches += 2;
    }
  }
  return mark_use(P, stream);
}

// Gradient of reversible large-alphabet plans: the walk's eigen staging
// (mode 1, unmasked; LogLike from its inside pass) and k_xgram's per-branch
// X_n = sum_c g_c D~_nc (x) U~_nc accumulated into d_X (R x A x A, FP64).
int run_big_grad(subby_plan *P, const int32_t *d_aln, int C, float *d_logL, const float *d_g, double *d_X,
                 cudaStream_t stream) {
  const int A = P->A, R = P->R;
  KParams k = walk_params(P, d_aln, C, kModeCounts | (d_logL ? kModeLogLike : 0), SUBBY_MASK_NONE, nullptr,
                          d_logL, nullptr, nullptr);
  const bool tc = (A == 64) && P->d_tab16 && (g_kernel_sel == 0 || g_kernel_sel == 5);
  const int tile = big_tile();
  const int H = (A + 31) / 32;
  int chunk = C;
  if (R > 1) {
    const size_t per_col = (size_t)2 * (R - 1) * A * sizeof(float);
    size_t cmax = std::max<size_t>(tile, kStageBudget / per_col);
    cmax = cmax / tile * tile;
    const size_t nch = ((size_t)C + cmax - 1) / cmax;
    const size_t even = ((size_t)C + nch - 1) / nch;
    chunk = (int)std::min<size_t>((size_t)C, (even + tile - 1) / tile * tile);
  }
  const int walk_grid = std::max(1, std::min((chunk + tile - 1) / tile, P->nsm * (H == 2 ? 1 : 2)));
  const size_t slot_floats = (size_t)walk_grid * k.nslots * tile * A;
  const size_t slot_ints = (size_t)walk_grid * k.nslots * tile * 2;  // a word per column half
  const size_t stage_floats = R > 1 ? (size_t)(R - 1) * chunk * A : 0;
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  int rc;
  if ((rc = P->grow(P->work, al(slot_floats * 4) + al(slot_ints * 4) + 2 * al(stage_floats * 4) + 256, stream)))
    return rc;
  char *base = (char *)P->work.p;
  k.scrV = (float *)base;
  base += al(slot_floats * 4);
  k.scrW = (int *)base;
  base += al(slot_ints * 4);
  float *sa = (float *)base;
  base += al(stage_floats * 4);
  float *sb = (float *)base;
  for (int c0 = 0; c0 < C; c0 += chunk) {
    const int cc = std::min(chunk, C - c0);
    int lr = launch_walk(k, A, R > 1 ? 1 : 0, tc, sa, sb, c0, cc, walk_grid, stream);
    if (lr != 0) return fail(SUBBY_ERR_CUDA, std::string("walk launch failed: ") + cudaGetErrorString((cudaError_t)lr));
    g_launches += 1;
    if (R == 1) continue;
    const int grid = std::max(1, std::min(xgram_items(R, cc), P->nsm * 4));
    lr = launch_xgram(A, sa, sb, d_g, c0, cc, R, d_X, grid, stream);
    if (lr != 0) return fail(SUBBY_ERR_CUDA, std::string("gradient launch failed: ") + cudaGetErrorString((cudaError_t)lr));
    g_launches += 1;
  }
  return mark_use(P, stream);
}

// Distance gradient of complex-system plans (irreversible or per-branch
// models; subby/jax/vjp.py:62-133): the walk stages D_n s_n and U_n (no
// mask), k_grad_cx adds sum_c g_c (D_n s_n)^T (dM_n/dt) U_n into grad_t[n].
int run_cx_grad(subby_plan *P, const int32_t *d_aln, int C, float *d_logL, const float *d_g, double *d_gt,
                cudaStream_t stream) {
  const int A = P->A, R = P->R;
  if (!post_supported(A))
    return fail(SUBBY_ERR_UNSUPPORTED, "gradients of these models are implemented for A = 4, 8, 16, 20, 32, 64");
  KParams k = walk_params(P, d_aln, C, d_logL ? kModeLogLike : 0, SUBBY_MASK_NONE, nullptr, d_logL, nullptr,
                          nullptr);
  k.npost = nullptr;
  k.npost_node = -1;
  const bool tc = (A == 64) && P->d_tab16 && (g_kernel_sel == 0 || g_kernel_sel == 5);
  const int tile = big_tile();
  const int H = (A + 31) / 32;
  int chunk = C;
  if (R > 1) {
    const size_t per_col = (size_t)2 * (R - 1) * A * sizeof(float);
    size_t cmax = std::max<size_t>(tile, kStageBudget / per_col);
    cmax = cmax / tile * tile;
    const size_t nch = ((size_t)C + cmax - 1) / cmax;
    const size_t even = ((size_t)C + nch - 1) / nch;
    chunk = (int)std::min<size_t>((size_t)C, (even + tile - 1) / tile * tile);
  }
  const int per_sm = A <= 8 ? 8 : (H == 2 ? 1 : 2);
  const int walk_grid = std::max(1, std::min((chunk + tile - 1) / tile, P->nsm * per_sm));
  const size_t slot_floats = (size_t)walk_grid * k.nslots * tile * A;
  const size_t slot_ints = (size_t)walk_grid * k.nslots * tile * 2;  // a word per column half
  const size_t stage_floats = R > 1 ? (size_t)(R - 1) * chunk * A : 0;
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  int rc;
  if ((rc = P->grow(P->work, al(slot_floats * 4) + al(slot_ints * 4) + 2 * al(stage_floats * 4) + 256, stream)))
    return rc;
  char *base = (char *)P->work.p;
  k.scrV = (float *)base;
  base += al(slot_floats * 4);
  k.scrW = (int *)base;
  base += al(slot_ints * 4);
  float *sa = R > 1 ? (float *)base : nullptr;
  base += al(stage_floats * 4);
  float *sb = R > 1 ? (float *)base : nullptr;
  for (int c0 = 0; c0 < C; c0 += chunk) {
    const int cc = std::min(chunk, C - c0);
    int lr = launch_walk_post(k, A, R > 1 ? 3 : 0, tc, sa, sb, c0, cc, walk_grid, stream);
    if (lr != 0) return fail(SUBBY_ERR_CUDA, std::string("walk launch failed: ") + cudaGetErrorString((cudaError_t)lr));
    g_launches += 1;
    if (R == 1) continue;
    const long long items = (long long)(cc + post_tile() - 1) / post_tile() * (R - 1);
    const int grid = (int)std::max<long long>(1, std::min<long long>(items, (long long)P->nsm * 8));
    lr = launch_grad_cx(k, A, sa, sb, P->d_gq, d_g, c0, cc, d_gt, grid, stream);
    if (lr != 0) return fail(SUBBY_ERR_CUDA, std::string("gradient launch failed: ") + cudaGetErrorString((cudaError_t)lr));
    g_launches += 1;
  }
  return mark_use(P, stream);
}

// Columns per chunk of the host-pointer pipeline: whole waves of the
// one-CTA-per-SM kernels (nsm x 256 columns), about eight chunks for large C,
// a single chunk below two waves (nothing to overlap).
int host_chunk_columns(const subby_plan *P, int C) {
  const long long wave = (long long)std::max(P->nsm, 1) * 256;
  if (C < 2 * wave) return std::max(C, 1);
  const long long waves = (C + wave - 1) / wave;
  const long long per = std::max(1LL, (waves + 7) / 8);
  return (int)std::min<long long>(C, per * wave);
}

int ensure_pipeline(subby_plan *P, int nev) {
  if (!P->s_in) CU(cudaStreamCreateWithFlags(&P->s_in, cudaStreamNonBlocking));
  if (!P->s_out) CU(cudaStreamCreateWithFlags(&P->s_out, cudaStreamNonBlocking));
  while ((int)P->ev.size() < nev) {
    cudaEvent_t e;
    CU(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    P->ev.push_back(e);
  }
  return 0;
}

int run_common(subby_plan *P, const int32_t *d_aln, int C, float *d_logL, float *d_counts,
               float *d_root, int mode, int mask_mode, const uint8_t *d_mask, const float *d_g,
               double *d_gt, double *d_gC, int *grid_out, cudaStream_t stream) {
  if (P->irrev) {
    if (mode & kModeGrad) return fail(SUBBY_ERR_UNSUPPORTED, "gradients of irreversible models are not implemented");
    if (mode & kModeCounts)
      return run_cx(P, d_aln, C, d_logL, d_counts, d_root, mode, mask_mode, d_mask, stream);
  }
  if (mode & kModeBranch) {
    // per-branch counts: the A = 4 tree-program kernel, or the large-alphabet
    // walk with the per-branch accumulation
    Launch L4;
    const bool ok4 = P->A == 4 && plan_tree4(P, mode, C, L4) == 0;
    if (!ok4 && !(big_supported(P->A) && g_kernel_sel != 1))
      return fail(SUBBY_ERR_UNSUPPORTED, "per-branch counts are implemented for A = 4 (tree program within "
                                         "the on-chip budget) and A = 16, 20, 32, 64");
  }
  if (big_supported(P->A) && !(mode & kModeGrad) && g_kernel_sel != 1)
    return run_big(P, d_aln, C, d_logL, d_counts, d_root, mode, mask_mode, d_mask, stream);
  Launch L;
  const bool tree = tree_supported(P->A) && !(mode & kModeGrad) && g_kernel_sel != 1;
  const bool small = small_supported(P->A);
  int rc;
  bool tree4 = false;
  if (tree && (rc = plan_tree4(P, mode, C, L)) == 0) {
    tree4 = true;
  } else {
    L = Launch();
    rc = tree ? plan_tree(P, mode, C, L) : small ? plan_small(P, mode, C, L) : plan_warp(P, mode, C, L);
    if (rc) return rc;
  }
  KParams &k = L.kp;
  k.aln = d_aln;
  k.C = C;
  k.R = P->R;
  k.A = P->A;
  k.nInt = P->nInt;
  k.mode = mode;
  k.mask_mode = mask_mode;
  k.mask = d_mask;
  k.tab = P->d_tab;
  k.tab64 = P->d_tab64;
  k.off = P->off;
  k.steps = P->d_steps;
  k.slots = P->d_slots;
  k.root_is_leaf = P->root_is_leaf;
  k.f81_mu = P->f81_mu;
  k.nworkers = L.nworkers;
  k.logL = d_logL;
  k.counts = d_counts;
  k.rootp = d_root;
  k.g = d_g;
  k.grad_t = d_gt;
  k.grad_C = d_gC;
  // scratch
  const size_t nsl = (size_t)std::max(tree ? P->prog_slots : P->nslots, 1);
  const size_t vbytes = (tree && !L.global_slots) ? 0 : nsl * L.nworkers * P->A * sizeof(float);
  const size_t wbytes = (tree && !L.global_slots) ? 0 : nsl * L.nworkers * 2 * sizeof(int);
  const size_t vb_al = (vbytes + 255) & ~(size_t)255;
  if ((rc = P->grow(P->work, vb_al + wbytes + 256, stream))) return rc;
  k.scrV = (float *)P->work.p;
  k.scrW = (int *)((char *)P->work.p + vb_al);
  if (grid_out) *grid_out = L.grid;
  int lr = tree4 ? launch_tree4(k, (mode & kModeF81) != 0, mask_mode, L.grid, L.block, L.smem, stream)
           : tree ? launch_tree(k, P->A, L.store, L.grid, L.block, L.smem, stream)
           : small ? launch_small(k, P->A, L.grid, L.block, L.smem, stream)
                   : launch_warp(k, P->A, L.grid, L.block, L.smem, stream);
  if (lr != 0) return fail(SUBBY_ERR_CUDA, std::string("kernel launch failed: ") +
                                               cudaGetErrorString((cudaError_t)lr));
  g_launches += 1;
  return mark_use(P, stream);
}

}  // namespace

namespace subby {
// Packed serving (server.cu): the A = 4 tree kernel's parameters of a
// device-pointer run of plan P over d_aln (R, C), without launching.  On
// success `stream` waits for the plan's tables and *smem / *block are the
// launch's dynamic shared memory and CTA size; the caller launches the
// packed kernel on `stream` and then calls plan_mark_used.  Returns nonzero
// (nothing enqueued) when the plan does not take the A = 4 tree kernel with
// 256 threads per CTA, or the kernel selector is not automatic.
int plan_tree4_params(subby_plan *P, const int32_t *d_aln, int C, float *d_logL, float *d_counts,
                      float *d_root, int counts_kind, int mask_mode, KParams *out, size_t *smem, int *block,
                      cudaStream_t stream) {
  if (!P || P->irrev || P->rows || P->A != 4 || P->R < 2 || C < 1 || !out) return SUBBY_ERR_UNSUPPORTED;
  if (mask_mode != SUBBY_MASK_NONE && mask_mode != SUBBY_MASK_AUTO) return SUBBY_ERR_UNSUPPORTED;
  int mode = kModeBT64;
  if (d_logL) mode |= kModeLogLike;
  if (d_root) mode |= kModeRootProb;
  if (d_counts) mode |= kModeCounts;
  if (d_counts && counts_kind == SUBBY_COUNTS_F81) mode |= kModeF81;
  if (!d_counts) mask_mode = SUBBY_MASK_NONE;
  std::lock_guard<std::mutex> g(P->lock);
  Launch L;
  if (plan_tree4(P, mode, C, L) != 0 || L.block != 256) return SUBBY_ERR_UNSUPPORTED;
  KParams &k = L.kp;
  k.aln = d_aln;
  k.C = C;
  k.R = P->R;
  k.A = P->A;
  k.nInt = P->nInt;
  k.mode = mode;
  k.mask_mode = mask_mode;
  k.mask = nullptr;
  k.tab = P->d_tab;
  k.tab64 = P->d_tab64;
  k.off = P->off;
  k.steps = P->d_steps;
  k.slots = P->d_slots;
  k.root_is_leaf = P->root_is_leaf;
  k.f81_mu = P->f81_mu;
  k.nworkers = L.nworkers;
  k.logL = d_logL;
  k.counts = d_counts;
  k.rootp = d_root;
  if (cudaStreamWaitEvent(stream, P->ready, 0) != cudaSuccess) return SUBBY_ERR_CUDA;
  *out = k;
  *smem = L.smem;
  *block = L.block;
  return SUBBY_OK;
}

// The plan's tables were read by work enqueued on `stream` up to here.
int plan_mark_used(subby_plan *P, cudaStream_t stream) {
  std::lock_guard<std::mutex> g(P->lock);
  return mark_use(P, stream);
}
}  // namespace subby

extern "C" {

int subby_plan_run(subby_plan *P, const int32_t *aln, int C, float *logL, float *counts,
                   float *rootProb, int counts_kind, int mask_mode, const uint8_t *mask, int flags,
                   void *stream_) {
  clear_error();
  g_launches = 0;
  if (!P) return fail(SUBBY_ERR_ARG, "null plan");
  if (C < 0) return fail(SUBBY_ERR_ARG, "negative column count");
  if (mask_mode < 0 || mask_mode > 2) return fail(SUBBY_ERR_ARG, "bad mask_mode");
  if (counts_kind != SUBBY_COUNTS_EIGEN && counts_kind != SUBBY_COUNTS_F81)
    return fail(SUBBY_ERR_ARG, "bad counts_kind");
  // zero columns: nothing to compute (an empty device buffer may be null)
  if (C == 0) return SUBBY_OK;
  if (!aln) return fail(SUBBY_ERR_ARG, "null alignment");
  if (mask_mode == SUBBY_MASK_GIVEN && !mask) return fail(SUBBY_ERR_ARG, "mask required");
  std::lock_guard<std::mutex> g(P->lock);
  cudaStream_t stream = (cudaStream_t)stream_;
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev != P->device) CU(cudaSetDevice(P->device));
  const int A = P->A, R = P->R;
  CU(cudaStreamWaitEvent(stream, P->ready, 0));
  int mode = 0;
  if (logL) mode |= kModeLogLike;
  if (rootProb) mode |= kModeRootProb;
  if (counts) mode |= kModeCounts;
  if (counts && counts_kind == SUBBY_COUNTS_F81) mode |= kModeF81;
  if (flags & SUBBY_IRREV_EXACT) mode |= kModeIrrevExact;
  const bool bt64 = (flags & SUBBY_BT_FP64) || (!(flags & SUBBY_BT_FP32) && A <= 8);
  if (bt64) mode |= kModeBT64;
  if (!mode) return SUBBY_OK;
  int rc = 0;
  if (flags & SUBBY_DEVICE_PTRS) {
    rc = run_common(P, aln, C, logL, counts, rootProb, mode, mask_mode, mask, nullptr, nullptr,
                    nullptr, nullptr, stream);
    if (rc == 0 && dev != P->device) cudaSetDevice(dev);
    return rc;
  }
  // host pointers: column chunks flow through three queues — host-to-device
  // copies on P->s_in, kernels on `stream`, device-to-host copies on
  // P->s_out — so the copies of one chunk overlap the kernels of its
  // neighbours.  Chunk c0..c0+cc is staged compactly ((R, cc) tokens at
  // R*c0, (A*A, cc) counts at A*A*c0, ...), so no device region is reused
  // within a call and the only ordering needed is copy-in -> kernel ->
  // copy-out per chunk.
  const size_t b_aln = (size_t)R * C * sizeof(int32_t);
  const size_t b_mask = (mask_mode == SUBBY_MASK_GIVEN) ? (size_t)R * C : 0;
  const size_t b_ll = logL ? (size_t)C * 4 : 0;
  const size_t b_ct = counts ? (size_t)A * A * C * 4 : 0;
  const size_t b_rp = rootProb ? (size_t)A * C * 4 : 0;
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t total = al(b_aln) + al(b_mask) + al(b_ll) + al(b_ct) + al(b_rp);
  if ((rc = P->grow(P->io, total, stream))) return rc;
  char *base = (char *)P->io.p;
  int32_t *d_aln = (int32_t *)base;
  base += al(b_aln);
  uint8_t *d_mask = b_mask ? (uint8_t *)base : nullptr;
  base += al(b_mask);
  float *d_ll = b_ll ? (float *)base : nullptr;
  base += al(b_ll);
  float *d_ct = b_ct ? (float *)base : nullptr;
  base += al(b_ct);
  float *d_rp = b_rp ? (float *)base : nullptr;
  const int chunk = host_chunk_columns(P, C);
  const int nch = (C + chunk - 1) / chunk;
  if ((rc = ensure_pipeline(P, 2 * nch + 2))) return rc;
  cudaEvent_t *ev = P->ev.data();
  // drains both copy queues before any return, so P->io is idle afterwards
  auto finish = [&](int code) {
    cudaStreamSynchronize(P->s_in);
    cudaStreamSynchronize(P->s_out);
    cudaStreamSynchronize(stream);
    return code;
  };
  CU(cudaEventRecord(ev[0], stream));
  CU(cudaStreamWaitEvent(P->s_in, ev[0], 0));
  for (int i = 0; i < nch; ++i) {
    const int c0 = i * chunk, cc = std::min(chunk, C - c0);
    cudaError_t e = cudaMemcpy2DAsync(d_aln + (size_t)R * c0, (size_t)cc * 4, aln + c0, (size_t)C * 4,
                                      (size_t)cc * 4, R, cudaMemcpyHostToDevice, P->s_in);
    if (e == cudaSuccess && b_mask)
      e = cudaMemcpy2DAsync(d_mask + (size_t)R * c0, (size_t)cc, mask + c0, (size_t)C, (size_t)cc, R,
                            cudaMemcpyHostToDevice, P->s_in);
    if (e == cudaSuccess) e = cudaEventRecord(ev[2 + 2 * i], P->s_in);
    if (e != cudaSuccess) return finish(cuda_fail(e, "chunk copy-in"));
  }
  for (int i = 0; i < nch; ++i) {
    const int c0 = i * chunk, cc = std::min(chunk, C - c0);
    cudaError_t e = cudaStreamWaitEvent(stream, ev[2 + 2 * i], 0);
    if (e != cudaSuccess) return finish(cuda_fail(e, "cudaStreamWaitEvent"));
    rc = run_common(P, d_aln + (size_t)R * c0, cc, d_ll ? d_ll + c0 : nullptr,
                    d_ct ? d_ct + (size_t)A * A * c0 : nullptr, d_rp ? d_rp + (size_t)A * c0 : nullptr,
                    mode, mask_mode, d_mask ? d_mask + (size_t)R * c0 : nullptr, nullptr, nullptr, nullptr,
                    nullptr, stream);
    if (rc) return finish(rc);
    e = cudaEventRecord(ev[3 + 2 * i], stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(P->s_out, ev[3 + 2 * i], 0);
    if (e == cudaSuccess && b_ll)
      e = cudaMemcpyAsync(logL + c0, d_ll + c0, (size_t)cc * 4, cudaMemcpyDeviceToHost, P->s_out);
    if (e == cudaSuccess && b_ct)
      e = cudaMemcpy2DAsync(counts + c0, (size_t)C * 4, d_ct + (size_t)A * A * c0, (size_t)cc * 4,
                            (size_t)cc * 4, (size_t)A * A, cudaMemcpyDeviceToHost, P->s_out);
    if (e == cudaSuccess && b_rp)
      e = cudaMemcpy2DAsync(rootProb + c0, (size_t)C * 4, d_rp + (size_t)A * c0, (size_t)cc * 4,
                            (size_t)cc * 4, (size_t)A, cudaMemcpyDeviceToHost, P->s_out);
    if (e != cudaSuccess) return finish(cuda_fail(e, "chunk copy-out"));
  }
  {
    cudaError_t e = cudaEventRecord(ev[1], P->s_out);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(stream, ev[1], 0);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return finish(cuda_fail(e, "chunk pipeline"));
  }
  if (P->d_err) {
    int dev_err = 0;
    CU(cudaMemcpyAsync(&dev_err, P->d_err, sizeof(int), cudaMemcpyDeviceToHost, stream));
    CU(cudaStreamSynchronize(stream));
    if (dev_err) {
      cudaMemsetAsync(P->d_err, 0, sizeof(int), stream);
      cudaStreamSynchronize(stream);
      if (dev != P->device) cudaSetDevice(dev);
      return fail(SUBBY_ERR_TIMEOUT, "a bounded device wait gave up (tensor-core walk)");
    }
  }
  if (dev != P->device) cudaSetDevice(dev);
  return SUBBY_OK;
}

int subby_plan_branch_counts(subby_plan *P, const int32_t *aln, int C, float *branchCounts, int counts_kind,
                             int mask_mode, const uint8_t *mask, int flags, void *stream_) {
  clear_error();
  g_launches = 0;
  if (!P) return fail(SUBBY_ERR_ARG, "null plan");
  if (C < 0) return fail(SUBBY_ERR_ARG, "negative column count");
  if (mask_mode < 0 || mask_mode > 2) return fail(SUBBY_ERR_ARG, "bad mask_mode");
  if (counts_kind != SUBBY_COUNTS_EIGEN && counts_kind != SUBBY_COUNTS_F81)
    return fail(SUBBY_ERR_ARG, "bad counts_kind");
  if (C == 0) return SUBBY_OK;
  if (!aln || !branchCounts) return fail(SUBBY_ERR_ARG, "null argument");
  if (mask_mode == SUBBY_MASK_GIVEN && !mask) return fail(SUBBY_ERR_ARG, "mask required");
  std::lock_guard<std::mutex> g(P->lock);
  cudaStream_t stream = (cudaStream_t)stream_;
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev != P->device) CU(cudaSetDevice(P->device));
  const int A = P->A, R = P->R;
  CU(cudaStreamWaitEvent(stream, P->ready, 0));
  const int mode = kModeCounts | kModeBranch | (counts_kind == SUBBY_COUNTS_F81 ? kModeF81 : 0) |
                   ((flags & SUBBY_IRREV_EXACT) ? kModeIrrevExact : 0);
  const size_t b_out = (size_t)R * A * A * C * sizeof(float);
  int rc;
  if (flags & SUBBY_DEVICE_PTRS) {
    // branch 0 (the root) has no branch: zeros
    CU(cudaMemsetAsync(branchCounts, 0, (size_t)A * A * C * sizeof(float), stream));
    if (R > 1)
      rc = run_common(P, aln, C, nullptr, branchCounts, nullptr, mode, mask_mode, mask, nullptr, nullptr, nullptr,
                      nullptr, stream);
    else
      rc = 0;
    if (dev != P->device) cudaSetDevice(dev);
    return rc;
  }
  const size_t b_aln = (size_t)R * C * sizeof(int32_t);
  const size_t b_mask = (mask_mode == SUBBY_MASK_GIVEN) ? (size_t)R * C : 0;
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  if ((rc = P->grow(P->io, al(b_aln) + al(b_mask) + al(b_out), stream))) return rc;
  char *base = (char *)P->io.p;
  int32_t *d_aln = (int32_t *)base;
  uint8_t *d_mask = b_mask ? (uint8_t *)(base + al(b_aln)) : nullptr;
  float *d_out = (float *)(base + al(b_aln) + al(b_mask));
  CU(cudaMemcpyAsync(d_aln, aln, b_aln, cudaMemcpyHostToDevice, stream));
  if (b_mask) CU(cudaMemcpyAsync(d_mask, mask, b_mask, cudaMemcpyHostToDevice, stream));
  CU(cudaMemsetAsync(d_out, 0, (size_t)A * A * C * sizeof(float), stream));
  if (R > 1 && (rc = run_common(P, d_aln, C, nullptr, d_out, nullptr, mode, mask_mode, d_mask, nullptr, nullptr,
                                nullptr, nullptr, stream))) {
    cudaStreamSynchronize(stream);
    return rc;
  }
  CU(cudaMemcpyAsync(branchCounts, d_out, b_out, cudaMemcpyDeviceToHost, stream));
  CU(cudaStreamSynchronize(stream));
  if (dev != P->device) cudaSetDevice(dev);
  return SUBBY_OK;
}

int subby_plan_posteriors(subby_plan *P, const int32_t *aln, int C, int node, float *nodePost, float *branchPost,
                          int flags, void *stream_) {
  clear_error();
  g_launches = 0;
  if (!P) return fail(SUBBY_ERR_ARG, "null plan");
  if (C < 0) return fail(SUBBY_ERR_ARG, "negative column count");
  if (node < -1 || node >= P->R) return fail(SUBBY_ERR_ARG, "node index out of range");
  if (!post_supported(P->A))
    return fail(SUBBY_ERR_UNSUPPORTED, "posteriors are implemented for A = 4, 8, 16, 20, 32, 64");
  if (C == 0) return SUBBY_OK;
  if (!aln) return fail(SUBBY_ERR_ARG, "null alignment");
  if (!nodePost && !branchPost) return fail(SUBBY_ERR_ARG, "no output requested");
  if (node == 0 && branchPost) return fail(SUBBY_ERR_ARG, "node 0 (the root) has no branch");
  std::lock_guard<std::mutex> g(P->lock);
  cudaStream_t stream = (cudaStream_t)stream_;
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev != P->device) CU(cudaSetDevice(P->device));
  const int A = P->A, R = P->R;
  CU(cudaStreamWaitEvent(stream, P->ready, 0));
  const size_t rows = node < 0 ? (size_t)R : 1;
  int rc;
  if (flags & SUBBY_DEVICE_PTRS) {
    rc = run_post(P, aln, C, node, nodePost, branchPost, stream);
    if (dev != P->device) cudaSetDevice(dev);
    return rc;
  }
  const size_t b_aln = (size_t)R * C * sizeof(int32_t);
  const size_t b_node = nodePost ? rows * A * C * sizeof(float) : 0;
  const size_t b_br = branchPost ? rows * A * A * C * sizeof(float) : 0;
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  if ((rc = P->grow(P->io, al(b_aln) + al(b_node) + al(b_br), stream))) return rc;
  char *base = (char *)P->io.p;
  int32_t *d_aln = (int32_t *)base;
  float *d_node = b_node ? (float *)(base + al(b_aln)) : nullptr;
  float *d_br = b_br ? (float *)(base + al(b_aln) + al(b_node)) : nullptr;
  CU(cudaMemcpyAsync(d_aln, aln, b_aln, cudaMemcpyHostToDevice, stream));
  if ((rc = run_post(P, d_aln, C, node, d_node, d_br, stream))) {
    cudaStreamSynchronize(stream);
    return rc;
  }
  if (b_node) CU(cudaMemcpyAsync(nodePost, d_node, b_node, cudaMemcpyDeviceToHost, stream));
  if (b_br) CU(cudaMemcpyAsync(branchPost, d_br, b_br, cudaMemcpyDeviceToHost, stream));
  CU(cudaStreamSynchronize(stream));
  if (dev != P->device) cudaSetDevice(dev);
  return SUBBY_OK;
}

int subby_plan_grad(subby_plan *P, const int32_t *aln, int C, const float *g, float *logL,
                    double *dldt, double *dldS, int flags, void *stream_) {
  clear_error();
  g_launches = 0;
  if (!P || !dldt || !dldS) return fail(SUBBY_ERR_ARG, "null argument");
  if (C < 0) return fail(SUBBY_ERR_ARG, "negative column count");
  if (C == 0) {  // the empty sum: zero gradients
    std::fill(dldt, dldt + P->R, 0.0);
    std::fill(dldS, dldS + (size_t)P->A * P->A, 0.0);
    return SUBBY_OK;
  }
  if (!aln) return fail(SUBBY_ERR_ARG, "null alignment");
  std::lock_guard<std::mutex> lk(P->lock);
  cudaStream_t stream = (cudaStream_t)stream_;
  const int A = P->A, R = P->R;
  CU(cudaStreamWaitEvent(stream, P->ready, 0));
  const bool dev = (flags & SUBBY_DEVICE_PTRS) != 0;
  // staging for host pointers
  const int32_t *d_aln = aln;
  const float *d_g = g;
  float *d_ll = logL;
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  int rc = 0;
  if (!dev) {
    const size_t b_aln = (size_t)R * C * 4, b_g = g ? (size_t)C * 4 : 0, b_ll = logL ? (size_t)C * 4 : 0;
    if ((rc = P->grow(P->io, al(b_aln) + al(b_g) + al(b_ll), stream))) return rc;
    char *base = (char *)P->io.p;
    int32_t *a = (int32_t *)base;
    base += al(b_aln);
    float *gg = b_g ? (float *)base : nullptr;
    base += al(b_g);
    float *ll = b_ll ? (float *)base : nullptr;
    CU(cudaMemcpyAsync(a, aln, b_aln, cudaMemcpyHostToDevice, stream));
    if (b_g) CU(cudaMemcpyAsync(gg, g, b_g, cudaMemcpyHostToDevice, stream));
    d_aln = a;
    d_g = gg;
    d_ll = ll;
  }
  if (P->irrev) {
    // complex-system plans: distance gradient only (dldS: the gradient with
    // respect to exchangeabilities does not apply; zeros)
    double *d_gt = nullptr;
    CU(pool_alloc((void **)&d_gt, sizeof(double) * R, P->pool, stream));
    CU(cudaMemsetAsync(d_gt, 0, sizeof(double) * R, stream));
    rc = run_cx_grad(P, d_aln, C, logL ? d_ll : nullptr, d_g, d_gt, stream);
    cudaError_t e = cudaSuccess;
    if (rc == 0) e = cudaMemcpyAsync(dldt, d_gt, sizeof(double) * R, cudaMemcpyDeviceToHost, stream);
    if (rc == 0 && e == cudaSuccess && logL && !dev)
      e = cudaMemcpyAsync(logL, d_ll, (size_t)C * 4, cudaMemcpyDeviceToHost, stream);
    cudaFreeAsync(d_gt, stream);
    cudaError_t e2 = cudaStreamSynchronize(stream);
    if (rc) return rc;
    if (e != cudaSuccess || e2 != cudaSuccess) return cuda_fail(e != cudaSuccess ? e : e2, "gradient readback");
    dldt[0] = 0.0;
    for (int i = 0; i < A * A; ++i) dldS[i] = 0.0;
    return SUBBY_OK;
  }
  if (big_supported(A) && g_kernel_sel == 0) {
    // walk + per-branch X_n (k_grad.cu); the gradients follow on the host in FP64
    double *d_X = nullptr;
    const size_t xb = sizeof(double) * (size_t)R * A * A;
    CU(pool_alloc((void **)&d_X, xb, P->pool, stream));
    CU(cudaMemsetAsync(d_X, 0, xb, stream));
    rc = run_big_grad(P, d_aln, C, logL ? d_ll : nullptr, d_g, d_X, stream);
    std::vector<double> X((size_t)R * A * A);
    cudaError_t e = cudaSuccess;
    if (rc == 0) e = cudaMemcpyAsync(X.data(), d_X, xb, cudaMemcpyDeviceToHost, stream);
    if (rc == 0 && e == cudaSuccess && logL && !dev)
      e = cudaMemcpyAsync(logL, d_ll, (size_t)C * 4, cudaMemcpyDeviceToHost, stream);
    cudaFreeAsync(d_X, stream);
    cudaError_t e2 = cudaStreamSynchronize(stream);
    if (rc) return rc;
    if (e != cudaSuccess || e2 != cudaSuccess) return cuda_fail(e != cudaSuccess ? e : e2, "gradient readback");
    // d/dt_n = sum_k mu_k e^{mu_k t_n} X_n[k][k];  Cg = sum_n J_n o X_n
    // (J with the 1e-8 degeneracy rule, subby/oracle/oracle.py:931-959)
    std::vector<double> Cg((size_t)A * A, 0.0), E(A);
    dldt[0] = 0.0;
    for (int n = 1; n < R; ++n) {
      const double tn = P->t[n];
      const double *Xn = X.data() + (size_t)n * A * A;
      for (int k2 = 0; k2 < A; ++k2) E[k2] = std::exp(P->mu[k2] * tn);
      double gd = 0.0;
      for (int k2 = 0; k2 < A; ++k2) gd += P->mu[k2] * E[k2] * Xn[k2 * A + k2];
      dldt[n] = gd;
      for (int k2 = 0; k2 < A; ++k2)
        for (int l = 0; l < A; ++l) {
          const double d = P->mu[k2] - P->mu[l];
          const double J = std::fabs(d) < 1e-8 ? tn * E[k2] : (E[k2] - E[l]) / d;
          Cg[k2 * A + l] += J * Xn[k2 * A + l];
        }
    }
    const std::vector<double> &V = P->V;
    std::vector<double> T((size_t)A * A, 0.0);
    for (int k2 = 0; k2 < A; ++k2)
      for (int j = 0; j < A; ++j) {
        double sm = 0.0;
        for (int l = 0; l < A; ++l) sm += Cg[k2 * A + l] * V[j * A + l];
        T[k2 * A + j] = sm;
      }
    for (int i = 0; i < A; ++i)
      for (int j = 0; j < A; ++j) {
        double sm = 0.0;
        for (int k2 = 0; k2 < A; ++k2) sm += V[i * A + k2] * T[k2 * A + j];
        dldS[i * A + j] = sm;
      }
    return SUBBY_OK;
  }
  // gradient partials live in a separate small allocation per call
  Launch L;
  const int mode = kModeGrad | (logL ? kModeLogLike : 0);
  rc = small_supported(A) ? plan_small(P, mode, C, L) : plan_warp(P, mode, C, L);
  if (rc) return rc;
  const size_t nb = (size_t)L.grid;
  double *d_part = nullptr;
  const size_t pbytes = nb * ((size_t)R + (size_t)A * A) * sizeof(double);
  CU(pool_alloc((void **)&d_part, pbytes, P->pool, stream));
  CU(cudaMemsetAsync(d_part, 0, pbytes, stream));
  int grid = 0;
  rc = run_common(P, d_aln, C, d_ll, nullptr, nullptr, mode, SUBBY_MASK_NONE, nullptr, d_g, d_part,
                  d_part + nb * R, &grid, stream);
  if (rc) {
    cudaFreeAsync(d_part, stream);
    cudaStreamSynchronize(stream);
    return rc;
  }
  std::vector<double> part(nb * ((size_t)R + (size_t)A * A));
  cudaError_t e = cudaMemcpyAsync(part.data(), d_part, pbytes, cudaMemcpyDeviceToHost, stream);
  if (e == cudaSuccess && logL && !dev)
    e = cudaMemcpyAsync(logL, d_ll, (size_t)C * 4, cudaMemcpyDeviceToHost, stream);
  if (e == cudaSuccess) e = cudaFreeAsync(d_part, stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) return cuda_fail(e, "gradient readback");
  if ((size_t)grid != nb) return fail(SUBBY_ERR_CUDA, "grid mismatch");
  for (int n = 0; n < R; ++n) {
    double s = 0.0;
    for (size_t b = 0; b < nb; ++b) s += part[b * R + n];
    dldt[n] = (n == 0) ? 0.0 : s;
  }
  std::vector<double> Cg((size_t)A * A, 0.0);
  const double *pc = part.data() + nb * R;
  for (size_t b = 0; b < nb; ++b)
    for (int i = 0; i < A * A; ++i) Cg[i] += pc[b * A * A + i];
  // dL/dS~ = V Cg V^T (FP64)
  const std::vector<double> &V = P->V;
  std::vector<double> T((size_t)A * A, 0.0);
  for (int k = 0; k < A; ++k)
    for (int j = 0; j < A; ++j) {
      double s = 0.0;
      for (int l = 0; l < A; ++l) s += Cg[k * A + l] * V[j * A + l];
      T[k * A + j] = s;
    }
  for (int i = 0; i < A; ++i)
    for (int j = 0; j < A; ++j) {
      double s = 0.0;
      for (int k = 0; k < A; ++k) s += V[i * A + k] * T[k * A + j];
      dldS[i * A + j] = s;
    }
  return SUBBY_OK;
}

static int one_shot(const int32_t *aln, const int32_t *parent, const double *dist, const double *ev,
                    const double *evec, const double *pi, int R, int C, int A, float *ll, float *ct,
                    float *rp, int kind, int mask_mode, const uint8_t *mask, int flags, void *stream) {
  subby_plan *P = nullptr;
  int rc = subby_plan_create(parent, dist, ev, evec, pi, R, A, &P);
  if (rc) return rc;
  rc = subby_plan_run(P, aln, C, ll, ct, rp, kind, mask_mode, mask, flags, stream);
  if (rc == 0 && (flags & SUBBY_DEVICE_PTRS)) {
    cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) rc = cuda_fail(e, "stream sync");
  }
  std::string keep = g_last_error;
  subby_plan_destroy(P);
  g_last_error = keep;
  g_static_error = nullptr;
  return rc;
}

int subby_loglike(const int32_t *aln, const int32_t *parent, const double *dist, const double *ev,
                  const double *evec, const double *pi, int R, int C, int A, float *logL, int flags,
                  void *stream) {
  if (!logL) return fail(SUBBY_ERR_ARG, "null output");
  return one_shot(aln, parent, dist, ev, evec, pi, R, C, A, logL, nullptr, nullptr, 0,
                  SUBBY_MASK_NONE, nullptr, flags, stream);
}

int subby_counts(const int32_t *aln, const int32_t *parent, const double *dist, const double *ev,
                 const double *evec, const double *pi, int R, int C, int A, int kind, int mask_mode,
                 const uint8_t *mask, float *counts, int flags, void *stream) {
  if (!counts) return fail(SUBBY_ERR_ARG, "null output");
  return one_shot(aln, parent, dist, ev, evec, pi, R, C, A, nullptr, counts, nullptr, kind,
                  mask_mode, mask, flags, stream);
}

int subby_rootprob(const int32_t *aln, const int32_t *parent, const double *dist, const double *ev,
                   const double *evec, const double *pi, int R, int C, int A, float *rootProb,
                   int flags, void *stream) {
  if (!rootProb) return fail(SUBBY_ERR_ARG, "null output");
  return one_shot(aln, parent, dist, ev, evec, pi, R, C, A, nullptr, nullptr, rootProb, 0,
                  SUBBY_MASK_NONE, nullptr, flags, stream);
}

}  // extern "C"
