// subby_counts_noalloc: the A = 4 Counts / LogLike path without any memory
// allocation, for callers that cannot allocate device memory.
//
// Who needs it: code that runs where cudaMalloc is unavailable or forbidden —
// an allocator-owning host framework (a caching allocator that owns the whole
// device heap), a driver or plugin callback that must not allocate, or a
// long-running service that fixes its device footprint at start-up.  The
// regular path (subby_plan_create / subby_plan_run) allocates per-plan tables
// and a workspace with cudaMalloc; this entry point instead keeps every table
// the kernel reads in one file-scope device array of fixed size, which every
// GPU that loads the library holds until the process exits.
//
// Limits and behaviour:
//  * A = 4 only, R <= kNoAllocMaxNodes (1023) nodes, and the tree program
//    must fit the tensor-memory / shared-memory budget of the A = 4 kernel;
//    anything larger returns SUBBY_ERR_UNSUPPORTED with a message.
//  * Alignment, mask and outputs are device pointers supplied by the caller.
//  * The first call on a device resolves the device address of the array
//    (cudaGetSymbolAddress, with that device current) and loads the kernel
//    variants (cudaFuncGetAttributes), so that no later call needs lazy
//    module loading; make that first call before any stream capture.  A
//    call with C = 0 does only this set-up (after validating its arguments)
//    and is the warm-up step.
//  * The tables are uploaded from one host staging buffer that the next call
//    rewrites, so a call on a stream that is being captured returns
//    SUBBY_ERR_UNSUPPORTED instead of recording a copy of that buffer.
//  * Every call rewrites the whole table region it uses, so nothing carries
//    over between calls and nothing needs clearing; calls that overlap on
//    the GPU (for example on two streams) share the array and race.
//  * No cudaMalloc, cudaFree or other allocating routine is called, on the
//    device or on the host: host-side staging uses a fixed static buffer.
//  * A rejection's reason is a fixed string that subby_last_error returns
//    (no message is formatted, which could allocate).
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>

#include "common.cuh"
#include "subby_gb300.h"

namespace {

constexpr int kNoAllocMaxNodes = 1023;
constexpr int kNoAllocFloats = 1 << 18;  // 1 MiB of tables per device
constexpr int kMaxDevices = 64;

static __device__ __align__(256) float g_noalloc_tables[kNoAllocFloats];

float g_stage[kNoAllocFloats];            // host staging of the tables
float *g_dev_tables[kMaxDevices] = {nullptr};
std::mutex g_noalloc_lock;

// Failure with a fixed reason string for subby_last_error (no formatting,
// no allocation).
int nfail(int code, const char *why) {
  subby::set_static_error(why);
  return code;
}

// Once per device, with it current: the device address of the table array
// and the kernel variants loaded.  Called with g_noalloc_lock held.
int noalloc_setup(int dev, float **dtab) {
  if (!g_dev_tables[dev]) {
    float *ptr = nullptr;
    const cudaError_t ce = cudaGetSymbolAddress((void **)&ptr, g_noalloc_tables);
    if (ce != cudaSuccess || !ptr) return nfail(SUBBY_ERR_CUDA, "cudaGetSymbolAddress failed");
    if (subby::preload_tree4() != 0) return nfail(SUBBY_ERR_CUDA, "loading the A=4 kernels failed");
    g_dev_tables[dev] = ptr;
  }
  *dtab = g_dev_tables[dev];
  return SUBBY_OK;
}

int align4(int n) { return (n + 3) & ~3; }

}  // namespace

extern "C" int subby_counts_noalloc(const int32_t *d_aln, const int32_t *parent, const double *dist,
                                    const double *evals, const double *evecs, const double *pi, int R,
                                    int C, int counts_kind, int mask_mode, const uint8_t *d_mask,
                                    float *d_counts, float *d_logL, void *stream_) {
  using namespace subby;
  const int A = 4;
  set_static_error("");
  if (!parent || !dist || !evals || !evecs || !pi) return nfail(SUBBY_ERR_ARG, "null argument");
  if (C < 0) return nfail(SUBBY_ERR_ARG, "negative column count");
  if (counts_kind != SUBBY_COUNTS_EIGEN && counts_kind != SUBBY_COUNTS_F81)
    return nfail(SUBBY_ERR_ARG, "bad counts_kind");
  if (mask_mode < 0 || mask_mode > 2) return nfail(SUBBY_ERR_ARG, "bad mask_mode");
  if (R < 1 || R > kNoAllocMaxNodes)
    return nfail(SUBBY_ERR_UNSUPPORTED, "tree larger than the no-allocation limit of 1023 nodes");
  cudaStream_t stream = (cudaStream_t)stream_;
  int dev = 0;
  cudaError_t ce = cudaGetDevice(&dev);
  if (ce != cudaSuccess || dev < 0 || dev >= kMaxDevices) return nfail(SUBBY_ERR_CUDA, "cudaGetDevice failed");
  // zero columns: only the per-device set-up (empty device buffers may be null)
  if (C == 0) {
    std::lock_guard<std::mutex> guard(g_noalloc_lock);
    float *dtab = nullptr;
    return noalloc_setup(dev, &dtab);
  }
  {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    ce = cudaStreamIsCapturing(stream, &cs);
    if (ce != cudaSuccess) return nfail(SUBBY_ERR_CUDA, "cudaStreamIsCapturing failed");
    if (cs != cudaStreamCaptureStatusNone)
      return nfail(SUBBY_ERR_UNSUPPORTED, "the stream is capturing: the table upload reads a host buffer that "
                                          "later calls rewrite");
  }
  if (!d_aln || !d_counts) return nfail(SUBBY_ERR_ARG, "null alignment or counts");
  if (mask_mode == SUBBY_MASK_GIVEN && !d_mask) return nfail(SUBBY_ERR_ARG, "missing mask");

  // ---- tree validation and children (fixed-size arrays, no heap)
  int left[kNoAllocMaxNodes], right[kNoAllocMaxNodes], cnt[kNoAllocMaxNodes];
  if (parent[0] >= 0) return nfail(SUBBY_ERR_TREE, "parentIndex[0] must be negative (root)");
  for (int n = 0; n < R; ++n) left[n] = right[n] = -1, cnt[n] = 0;
  for (int n = 1; n < R; ++n) {
    const int p = parent[n];
    if (p < 0 || p >= n) return nfail(SUBBY_ERR_TREE, "parentIndex[n] must lie in [0, n)");
    cnt[p]++;
    if (left[p] < 0) left[p] = n;
    else right[p] = n;
  }
  for (int n = 0; n < R; ++n)
    if (cnt[n] != 0 && cnt[n] != 2) return nfail(SUBBY_ERR_TREE, "every node needs 0 or 2 children");
  for (int a = 0; a < A; ++a)
    if (!(pi[a] > 0.0)) return nfail(SUBBY_ERR_ARG, "pi must be strictly positive");
  for (int n = 0; n < R; ++n)
    if (!(dist[n] >= 0.0) || !std::isfinite(dist[n]))
      return nfail(SUBBY_ERR_ARG, "distances must be finite and non-negative");

  // ---- DFS postorder of the internal nodes, stored / derived classification
  int order[kNoAllocMaxNodes], norder = 0;
  {
    int stv[kNoAllocMaxNodes], sts[kNoAllocMaxNodes], top = 0;
    if (R > 1) {
      stv[0] = 0;
      sts[0] = 0;
      top = 1;
    }
    while (top > 0) {
      const int v = stv[top - 1];
      if (left[v] < 0) {
        --top;
        continue;
      }
      if (sts[top - 1] == 0) {
        sts[top - 1] = 1;
        stv[top] = left[v], sts[top] = 0, ++top;
      } else if (sts[top - 1] == 1) {
        sts[top - 1] = 2;
        stv[top] = right[v], sts[top] = 0, ++top;
      } else {
        order[norder++] = v;
        --top;
      }
    }
  }
  int kind[kNoAllocMaxNodes];
  int nslots = 0;
  for (int n = 0; n < R; ++n) kind[n] = -1;
  for (int i = 0; i < norder; ++i) {
    const int v = order[i];
    if (v == 0) {
      kind[v] = -3;
      continue;
    }
    const bool ok = (kind[left[v]] == -1 || kind[left[v]] >= 0) && (kind[right[v]] == -1 || kind[right[v]] >= 0);
    kind[v] = ok ? -2 : nslots++;
  }
  int nsteps = 0;
  for (int i = 0; i < norder; ++i)
    if (order[i] == 0 || kind[order[i]] >= 0) ++nsteps;

  std::lock_guard<std::mutex> guard(g_noalloc_lock);
  float *dtab = nullptr;
  {
    const int rc = noalloc_setup(dev, &dtab);
    if (rc != SUBBY_OK) return rc;
  }

  // ---- table layout inside the array (floats)
  TableOffsets o{};
  int cur = 0;
  auto take = [&](int n) {
    const int at = cur;
    cur += align4(n);
    return at;
  };
  o.MT = take(R * 20);
  o.Vu = take(4 * 16 + 20 + 4 + 4);
  o.Vd = o.Vu + 16;
  o.Ut = o.Vd + 16;
  o.pi = o.Ut + 20;
  o.S = o.pi + 4;
  o.V = o.S + 16;
  o.pi0 = o.V + 16;
  o.J = take(R * 16);
  o.F81 = take(R * 4);
  o.K = take(R * 100);
  const int prog_at = take(16 * nsteps);
  const int t64_at = take(2 * (2 * 16 + 4 + R));  // FP64 V, S (8-byte aligned: offset multiple of 4)
  o.total = cur;
  if (cur > kNoAllocFloats) return nfail(SUBBY_ERR_UNSUPPORTED, "tables exceed the no-allocation array");

  // ---- FP64 model preparation on the host (same formulas as subby_plan_create)
  float *T = g_stage;
  double sp[4], isp[4], pi2 = 0.0;
  for (int a = 0; a < 4; ++a) sp[a] = std::sqrt(pi[a]), isp[a] = 1.0 / sp[a], pi2 += pi[a] * pi[a];
  const double mu81 = 1.0 / (1.0 - pi2);
  double S64[16], Ut64[20];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      double s = 0.0;
      for (int k = 0; k < 4; ++k) s += evecs[i * 4 + k] * evals[k] * evecs[j * 4 + k];
      S64[i * 4 + j] = s;
    }
  for (int b = 0; b < 4; ++b)
    for (int l = 0; l < 4; ++l) {
      T[o.Vu + b * 4 + l] = (float)(sp[b] * evecs[b * 4 + l]);
      T[o.Vd + b * 4 + l] = (float)(isp[b] * evecs[b * 4 + l]);
      Ut64[b * 4 + l] = sp[b] * evecs[b * 4 + l];
      T[o.S + b * 4 + l] = (float)S64[b * 4 + l];
      T[o.V + b * 4 + l] = (float)evecs[b * 4 + l];
    }
  for (int l = 0; l < 4; ++l) {
    double s = 0.0;
    for (int b = 0; b < 4; ++b) s += sp[b] * evecs[b * 4 + l];
    Ut64[16 + l] = s;
  }
  for (int i = 0; i < 20; ++i) T[o.Ut + i] = (float)Ut64[i];
  for (int a = 0; a < 4; ++a) T[o.pi + a] = T[o.pi0 + a] = (float)pi[a];
  for (int n = 0; n < R; ++n) {
    const double t = dist[n];
    double E[4], M[16], J[16];
    for (int k = 0; k < 4; ++k) E[k] = std::exp(evals[k] * t);
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j) {
        double s = 0.0;
        for (int k = 0; k < 4; ++k) s += evecs[i * 4 + k] * E[k] * evecs[j * 4 + k];
        M[i * 4 + j] = isp[i] * sp[j] * s;
      }
    for (int b = 0; b < 4; ++b) {
      double rs = 0.0;
      for (int j = 0; j < 4; ++j) {
        T[o.MT + n * 20 + j * 4 + b] = (float)M[b * 4 + j];
        rs += M[b * 4 + j];
      }
      T[o.MT + n * 20 + 16 + b] = (float)rs;
    }
    // J(t) in FP64 with the 1e-8 degeneracy rule; expm1 form near degeneracy
    for (int k = 0; k < 4; ++k)
      for (int l = 0; l < 4; ++l) {
        const double d = evals[k] - evals[l];
        double v;
        if (std::fabs(d) < 1e-8) v = t * E[k];
        else v = E[l] * std::expm1(d * t) / d;
        J[k * 4 + l] = v;
        T[o.J + n * 16 + k * 4 + l] = (float)v;
      }
    for (int code = 0; code < 5; ++code)
      for (int k = 0; k < 4; ++k) {
        for (int l = 0; l < 4; ++l)
          T[o.K + (n * 5 + code) * 20 + k * 4 + l] = (float)(J[k * 4 + l] * Ut64[code * 4 + l]);
      }
    const double e = std::exp(-mu81 * t), pp = 1.0 - e;
    T[o.F81 + n * 4 + 0] = (float)(t * e);
    T[o.F81 + n * 4 + 1] = (float)(pp / mu81 - t * e);
    T[o.F81 + n * 4 + 2] = (float)(t * (1.0 + e) - 2.0 * pp / mu81);
    T[o.F81 + n * 4 + 3] = (float)t;
  }
  {
    int4 *pg = reinterpret_cast<int4 *>(T + prog_at);
    int q = 0;
    for (int i = 0; i < norder; ++i) {
      const int v = order[i];
      if (!(v == 0 || kind[v] >= 0)) continue;
      int4 c[2];
      int gk[4] = {0, 0, 0, 0};
      for (int side = 0; side < 2; ++side) {
        const int ch = side ? right[v] : left[v];
        const int kl = left[ch], kr = right[ch];
        c[side] = make_int4(ch, kind[ch], kl > 0 ? kl : 0, kr > 0 ? kr : 0);
        if (kind[ch] == -2) gk[2 * side] = kind[kl], gk[2 * side + 1] = kind[kr];
      }
      pg[q++] = make_int4(v, v == 0 ? -1 : kind[v], v == 0 ? 1 : 0, 0);
      pg[q++] = c[0];
      pg[q++] = c[1];
      pg[q++] = make_int4(gk[0], gk[1], gk[2], gk[3]);
    }
    double *t64 = reinterpret_cast<double *>(T + t64_at);
    for (int i = 0; i < 16; ++i) t64[i] = evecs[i], t64[16 + i] = S64[i];
  }

  // ---- launch geometry of the A = 4 tree kernel (tables in shared memory,
  // slot vectors in tensor memory)
  const bool f81 = counts_kind == SUBBY_COUNTS_F81;
  KParams k{};
  int sofs = 0, ntab = 0;
  auto add = [&](int gofs, int n) {
    k.stab[ntab++] = SmemTable{gofs, sofs, n};
    sofs += align4(n);
  };
  add(o.MT, R * 20);
  add(o.Vu, 16 * 4 + 20 + 4 + 4);
  if (f81) add(o.F81, R * 4);
  else add(o.J, R * 16);
  if (!f81) add(o.K, R * 100);
  k.stab[ntab++] = SmemTable{0, sofs, 0};
  sofs += 28;
  k.ntab = ntab;
  k.smem_steps = sofs;
  sofs += 16 * nsteps;
  int maxsm = 0, nsm = 0;
  cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  int threads = 0;
  for (int t : {256, 128})
    if (nslots * 4 <= 512 / (t / 128) && (size_t)(sofs + nslots * t) * 4 + 1024 <= (size_t)maxsm) {
      threads = t;
      break;
    }
  if (!threads) return nfail(SUBBY_ERR_UNSUPPORTED, "tree program exceeds the on-chip budget of the A=4 kernel");
  k.smem_slots = -1;
  k.smem_words = sofs;
  sofs += nslots * threads;
  if (sofs < (maxsm / 2 + 4096) / 4) sofs = (maxsm / 2 + 4096) / 4;

  ce = cudaMemcpyAsync(dtab, T, (size_t)cur * sizeof(float), cudaMemcpyHostToDevice, stream);
  if (ce != cudaSuccess) return nfail(SUBBY_ERR_CUDA, "table upload failed");

  k.aln = d_aln;
  k.C = C;
  k.R = R;
  k.A = 4;
  k.nInt = norder;
  k.mode = kModeCounts | kModeBT64 | (f81 ? kModeF81 : 0) | (d_logL ? kModeLogLike : 0);
  k.mask_mode = mask_mode;
  k.mask = d_mask;
  k.tab = dtab;
  k.tab64 = reinterpret_cast<const double *>(dtab + t64_at);
  k.off = o;
  k.root_is_leaf = (R == 1);
  k.f81_mu = (float)mu81;
  k.logL = d_logL;
  k.counts = d_counts;
  k.prog = reinterpret_cast<const int4 *>(dtab + prog_at);
  k.nsteps = nsteps;
  k.nslots = nslots;
  const int grid = std::max(1, std::min((C + threads - 1) / threads, nsm));
  const int lr = launch_tree4(k, f81, mask_mode, grid, threads, (size_t)sofs * sizeof(float), stream);
  if (lr != 0) return nfail(SUBBY_ERR_CUDA, "kernel launch failed");
  return SUBBY_OK;
}
