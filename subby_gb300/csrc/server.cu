// Native serving engine: continuous batching of (alignment, tree, model)
// jobs of uneven R, C and A on one GPU, behind the subby_server_* C ABI.
//
// The reference has no server (its only batching is jax.vmap over
// same-shaped trees, scripts/batch_eigensub_maf.py:527-532); this engine
// takes jobs as they arrive and keeps the device busy with their work:
//
//  * one engine thread owns the device work.  Callers submit job
//    descriptors (the engine copies the tree and model) and collect
//    completions; nothing on their side touches CUDA;
//  * prepared plans (tree program, M(t), J(t) and operand tables) stay
//    resident in an LRU cache keyed by a hash of tree and model;
//  * short A = 4 jobs waiting together run as one launch of the persistent
//    packed kernel over their flattened (job, 256-column tile) queue
//    (k_tree4_packed);
//  * every other job is admitted when one of `max_inflight` slots is free
//    and its device footprint fits the budget; among waiting jobs the one
//    with the smallest estimated device time goes first, less a credit that
//    grows with its wait, so long jobs are delayed but not starved, and two
//    slots are kept for short jobs;
//  * each slot owns two streams (short jobs take the high-priority one, so
//    the block scheduler starts their kernels ahead of queued work of long
//    jobs) and a device arena that grows to the largest run it served;
//  * a job's alignment rows are gathered straight from host memory by the
//    SMs (subby_gather_rows), its kernels run on the slot stream, and its
//    outputs are copied into pinned host blocks of a size-class pool; long
//    jobs run as column slices of whole kernel waves, each slice's results
//    copied out as soon as it is done, so short jobs wait for one slice of a
//    long job, not all of it;
//  * completion is one event per slot; the device status word (bounded waits
//    that gave up) is copied to pinned memory on the run's stream, so a
//    completed run's status needs no blocking call.
//
// Results of a job do not depend on what else is in flight: every column is
// computed by the same kernels on the same inputs as a single call.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <list>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "common.cuh"
#include "subby_gb300.h"

namespace subby {
int plan_status_async(subby_plan *P, int *h, cudaStream_t s);
int plan_tree4_params(subby_plan *P, const int32_t *d_aln, int C, float *d_logL, float *d_counts,
                      float *d_root, int counts_kind, int mask_mode, KParams *out, size_t *smem, int *block,
                      cudaStream_t stream);
int plan_mark_used(subby_plan *P, cudaStream_t stream);
}  // namespace subby

using subby::KParams;
using subby::T4Queue;

namespace {

using Clock = std::chrono::steady_clock;

// Kernel time per (column x tree node), ns, of Counts by path on GB300
// (measured: A = 4 R = 255, A = 20 R = 399, A = 64 R = 127 workloads), plus
// the host-link time of the job's tokens and results; used only to order
// and slice work, never to skip any.
double ns_per_col_node(int A, bool f81) {
  if (A <= 8) return f81 ? 0.011 : 0.012;
  if (A <= 20) return f81 ? 0.10 : 0.30;
  return f81 ? 0.70 : 1.2;
}
double job_cost_ms(const subby_job &d) {
  const bool f81 = d.counts_kind == SUBBY_COUNTS_F81 && (d.want & SUBBY_WANT_COUNTS);
  const double kern = ns_per_col_node(d.A, f81) * d.R * (double)d.C * 1e-6;
  const double out_b = 4.0 * d.C * (((d.want & SUBBY_WANT_LOGLIKE) ? 1 : 0) +
                                    ((d.want & SUBBY_WANT_COUNTS) ? d.A * d.A : 0) +
                                    ((d.want & SUBBY_WANT_ROOTPROB) ? d.A : 0));
  const double in_b = 4.0 * d.R * (double)d.C;
  return kern + out_b / 1.7e8 + in_b / 2.0e8;  // ~170 GB/s out, ~200 GB/s in
}

uint64_t fnv(uint64_t h, const void *p, size_t n) {
  const unsigned char *b = static_cast<const unsigned char *>(p);
  for (size_t i = 0; i < n; ++i) h = (h ^ b[i]) * 1099511628211ull;
  return h;
}

// Pinned host blocks in power-of-two size classes (page pinning costs
// milliseconds per large block, so blocks are reused).
struct PinnedPool {
  std::map<size_t, std::vector<void *>> free_;
  std::unordered_map<void *, size_t> sizes_;
  std::vector<void *> all_;
  static size_t cls(size_t n) {
    size_t c = 1 << 16;
    while (c < n) c <<= 1;
    return c;
  }
  void *fresh(size_t c) {
    void *p = nullptr;
    if (cudaHostAlloc(&p, c, cudaHostAllocPortable) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    all_.push_back(p);
    sizes_[p] = c;
    return p;
  }
  void *get(size_t n) {
    const size_t c = cls(n);
    auto &v = free_[c];
    if (!v.empty()) {
      void *p = v.back();
      v.pop_back();
      return p;
    }
    return fresh(c);
  }
  void put(void *p) {
    if (p) free_[sizes_[p]].push_back(p);
  }
  void prewarm(size_t max_bytes, int per_class) {
    for (size_t c = 1 << 16; c <= max_bytes; c <<= 1)
      for (int i = 0; i < per_class; ++i) {
        void *p = fresh(c);
        if (!p) return;
        free_[c].push_back(p);
      }
  }
  ~PinnedPool() {
    for (void *p : all_) cudaFreeHost(p);
  }
};

struct SJob {
  subby_job d{};
  std::vector<int32_t> parent, rowmap;
  std::vector<double> dist, ev, V, pi;
  uint64_t key = 0;
  double arrival = 0, t_start = -1, t_finish = -1;
  double cost_ms = 0;
  size_t bytes = 0;
  int slot = -1;
  int status = 0;
  void *out[3] = {nullptr, nullptr, nullptr};  // pinned logLike, counts, rootProb
  int64_t handle = 0;
  bool nopack = false;   // its plan does not take the packed A = 4 kernel
};

// Work in flight on one slot: one job, or a batch of short A = 4 jobs run
// by one launch of the packed kernel.
struct Run {
  std::vector<SJob *> jobs;
  int slot = -1;
  size_t bytes = 0;
};

struct PlanEntry {
  subby_plan *p = nullptr;
  bool busy = false;
  std::list<uint64_t>::iterator lru;
};

struct Slot {
  cudaStream_t s_norm = nullptr, s_hi = nullptr;
  cudaEvent_t done = nullptr;    // end of the slot's current run
  void *arena = nullptr;
  size_t arena_bytes = 0;
  int *h_err = nullptr;          // pinned status word of the run in the slot
  int32_t *h_rowmap = nullptr;   // pinned row map of the job in the slot
  void *h_stage = nullptr;       // pinned staging of a packed batch (queue, row maps)
  size_t h_stage_bytes = 0;
  Run *run = nullptr;
};

}  // namespace

struct subby_server {
  int device = 0, nsm = 0;
  int max_inflight = 8, short_slots = 2;
  size_t budget = 0, used = 0;
  double short_ms = 5.0, slice_ms = 8.0, aging = 0.2;
  int plan_cache = 64;
  int wave_cols = 0;   // slice granularity in columns (0: one wave of the kernels' grids)
  bool pack = true;    // short A = 4 jobs waiting together share one packed launch
  int pack_max_jobs = 64;
  // tiles of 256 columns per packed work item, by tree size (R <= 64, <= 256,
  // larger): the item shape the serving autotuner picks
  int pack_tiles_r[3] = {1, 1, 1};
  long long pack_max_cols = 152LL * 256 * 16;
  Clock::time_point t0;
  cudaMemPool_t pool = nullptr;

  std::vector<Slot> slots;
  std::vector<int> free_slots;
  std::unordered_map<uint64_t, PlanEntry> plans;
  std::list<uint64_t> lru;
  PinnedPool pinned;

  std::mutex mu;                      // submissions, completions, release
  std::condition_variable cv_work, cv_done;
  std::deque<SJob *> submitted;
  std::deque<SJob *> completed;
  std::unordered_map<int64_t, SJob *> held;   // completed, results not yet released
  std::vector<void *> to_release;             // pinned blocks handed back by callers
  std::atomic<bool> stop{false};
  std::thread th;
  int64_t next_handle = 1;

  std::vector<SJob *> waiting;
  std::vector<Run *> inflight;
  double busy_s = 0;                          // engine-thread time spent on work
  long long packed_jobs = 0, packed_launches = 0;
  // published by the engine thread for subby_server_stats
  std::atomic<double> pub_busy_s{0.0};
  std::atomic<int> pub_plans{0}, pub_inflight{0}, pub_waiting{0};
  std::atomic<long long> pub_packed_jobs{0}, pub_packed_launches{0};

  double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

namespace {

uint64_t job_key(const SJob &j) {
  uint64_t h = 1469598103934665603ull;
  h = fnv(h, j.parent.data(), j.parent.size() * 4);
  h = fnv(h, j.dist.data(), j.dist.size() * 8);
  h = fnv(h, j.ev.data(), j.ev.size() * 8);
  h = fnv(h, j.V.data(), j.V.size() * 8);
  h = fnv(h, j.pi.data(), j.pi.size() * 8);
  return h;
}

// Device footprint estimate of one in-flight job: plan tables, tokens,
// outputs and the plan's scratch (staging of the large-alphabet path,
// capped per plan).
size_t job_bytes(int R, int C, int A) {
  const size_t tables = (size_t)4 * R * (A + 1) * A * 6 + (A <= 8 ? (size_t)4 * R * (A + 1) * (A * A + 4) : 0);
  const size_t tokens = (size_t)4 * R * C;
  const size_t outputs = (size_t)4 * C * (A * A + A + 1);
  const size_t scratch = A >= 16 ? std::min<size_t>((size_t)4 << 30, (size_t)8 * (R - 1) * A * C) +
                                       (size_t)4 * R * (A + 1) * std::min(C, 152 * 128)
                                 : (size_t)4 * R * (A + 2) * std::min(C, 152 * 256);
  return tables + tokens + outputs + scratch;
}

size_t align256(size_t n) { return (n + 255) & ~(size_t)255; }

int plan_for(subby_server *S, SJob *j, subby_plan **out) {
  auto it = S->plans.find(j->key);
  if (it != S->plans.end()) {
    S->lru.erase(it->second.lru);
    S->lru.push_front(j->key);
    it->second.lru = S->lru.begin();
    *out = it->second.p;
    return SUBBY_OK;
  }
  subby_plan *p = nullptr;
  const int rc = subby_plan_create(j->parent.data(), j->dist.data(), j->ev.data(), j->V.data(), j->pi.data(),
                                   j->d.R, j->d.A, &p);
  if (rc != 0) return rc;
  S->lru.push_front(j->key);
  S->plans[j->key] = PlanEntry{p, false, S->lru.begin()};
  // evict least recently used plans that no job is running
  while ((int)S->plans.size() > S->plan_cache) {
    bool evicted = false;
    for (auto r = S->lru.rbegin(); r != S->lru.rend(); ++r) {
      auto e = S->plans.find(*r);
      if (e != S->plans.end() && !e->second.busy && e->first != j->key) {
        subby_plan_destroy(e->second.p);
        S->lru.erase(std::next(r).base());
        S->plans.erase(e);
        evicted = true;
        break;
      }
    }
    if (!evicted) break;
  }
  *out = p;
  return SUBBY_OK;
}

bool plan_busy(subby_server *S, uint64_t key) {
  auto it = S->plans.find(key);
  return it != S->plans.end() && it->second.busy;
}

bool fits(subby_server *S, SJob *j) {
  if (S->free_slots.empty()) return false;
  if (j->cost_ms > S->short_ms) {
    int longs = 0;
    for (Run *r : S->inflight)
      for (SJob *k : r->jobs) longs += k->cost_ms > S->short_ms;
    if (longs >= S->max_inflight - S->short_slots) return false;
  }
  if (plan_busy(S, j->key)) return false;
  return S->used + j->bytes <= S->budget || S->inflight.empty();
}

int grow_arena(subby_server *S, Slot &sl, size_t need, cudaStream_t s) {
  if (need <= sl.arena_bytes) return 0;
  if (sl.arena) cudaFreeAsync(sl.arena, s);
  sl.arena = nullptr;
  sl.arena_bytes = 0;
  size_t want = 1 << 20;
  while (want < need) want <<= 1;
  cudaError_t e = S->pool ? cudaMallocFromPoolAsync(&sl.arena, want, S->pool, s) : cudaMallocAsync(&sl.arena, want, s);
  if (e != cudaSuccess) {
    cudaGetLastError();
    sl.arena = nullptr;
    return SUBBY_ERR_NOMEM;
  }
  sl.arena_bytes = want;
  return 0;
}

void start_run(subby_server *S, int slot_i, const std::vector<SJob *> &jobs) {
  Slot &sl = S->slots[slot_i];
  S->free_slots.erase(std::find(S->free_slots.begin(), S->free_slots.end(), slot_i));
  Run *run = new Run();
  run->slot = slot_i;
  for (SJob *j : jobs) {
    S->plans[j->key].busy = true;
    j->slot = slot_i;
    run->jobs.push_back(j);
    run->bytes += j->bytes;
  }
  sl.run = run;
  S->used += run->bytes;
  S->inflight.push_back(run);
}

// Enqueue one job on a free slot; returns a status code (the job completes
// with it at once when it is not 0; nothing of it is then in flight).
int launch(subby_server *S, SJob *j) {
  const int slot_i = S->free_slots.back();
  Slot &sl = S->slots[slot_i];
  const subby_job &d = j->d;
  const int R = d.R, C = d.C, A = d.A;
  cudaStream_t st = j->cost_ms <= S->short_ms ? sl.s_hi : sl.s_norm;
  subby_plan *plan = nullptr;
  {
    const int rc = plan_for(S, j, &plan);
    if (rc) return rc;
  }
  // a failure after work was enqueued waits for that work before the
  // caller hands the job's buffers back
  auto bail = [&](int rc) {
    cudaStreamSynchronize(st);
    cudaGetLastError();
    return rc;
  };
  const bool wl = d.want & SUBBY_WANT_LOGLIKE, wc = d.want & SUBBY_WANT_COUNTS, wr = d.want & SUBBY_WANT_ROOTPROB;
  // column slices: whole waves of the kernels' persistent grids
  const long long wave = S->wave_cols > 0 ? S->wave_cols : (long long)S->nsm * (A == 64 ? 128 : 256);
  long long nsl = std::max(1LL, (long long)std::ceil(j->cost_ms / S->slice_ms));
  nsl = std::min(nsl, (C + wave - 1) / wave);
  const long long cmax = (nsl == 1) ? C : ((C + nsl - 1) / nsl + wave - 1) / wave * wave;
  // arena: tokens of one slice | outputs of one slice
  const size_t b_aln = align256((size_t)4 * R * cmax), b_ll = wl ? align256((size_t)4 * cmax) : 0,
               b_ct = wc ? align256((size_t)4 * A * A * cmax) : 0, b_rp = wr ? align256((size_t)4 * A * cmax) : 0;
  if (grow_arena(S, sl, b_aln + b_ll + b_ct + b_rp, st)) return bail(SUBBY_ERR_NOMEM);
  char *base = static_cast<char *>(sl.arena);
  int32_t *s_aln = reinterpret_cast<int32_t *>(base);
  float *s_ll = wl ? reinterpret_cast<float *>(base + b_aln) : nullptr;
  float *s_ct = wc ? reinterpret_cast<float *>(base + b_aln + b_ll) : nullptr;
  float *s_rp = wr ? reinterpret_cast<float *>(base + b_aln + b_ll + b_ct) : nullptr;
  // pinned host outputs
  const size_t n_out[3] = {(size_t)4 * C, (size_t)4 * A * A * C, (size_t)4 * A * C};
  const bool want_k[3] = {wl, wc, wr};
  for (int k = 0; k < 3; ++k)
    if (want_k[k] && !(j->out[k] = S->pinned.get(n_out[k]))) return bail(SUBBY_ERR_NOMEM);
  const int32_t *rowmap = nullptr;
  if (!j->rowmap.empty()) {
    std::memcpy(sl.h_rowmap, j->rowmap.data(), 4 * (size_t)R);
    rowmap = sl.h_rowmap;
  }
  for (long long c0 = 0; c0 < C; c0 += cmax) {
    const int cc = (int)std::min<long long>(cmax, C - c0);
    int rc = subby_gather_rows(d.alignment + c0, d.pitch, rowmap, R, cc, s_aln, st);
    if (rc) return bail(rc);
    rc = subby_plan_run(plan, s_aln, cc, s_ll, s_ct, s_rp, d.counts_kind, d.mask_mode, nullptr,
                        SUBBY_DEVICE_PTRS, st);
    if (rc) return bail(rc);
    // this slice's outputs into columns [c0, c0 + cc) of the host outputs,
    // copied by the SMs so that other jobs' copies interleave with them
    int e = 0;
    if (wl) e = subby::launch_copy_rows(static_cast<float *>(j->out[0]) + c0, 0, s_ll, 0, (size_t)4 * cc, 1, st);
    if (!e && wc)
      e = subby::launch_copy_rows(static_cast<float *>(j->out[1]) + c0, (size_t)4 * C, s_ct, (size_t)4 * cc,
                                  (size_t)4 * cc, A * A, st);
    if (!e && wr)
      e = subby::launch_copy_rows(static_cast<float *>(j->out[2]) + c0, (size_t)4 * C, s_rp, (size_t)4 * cc,
                                  (size_t)4 * cc, A, st);
    if (e) return bail(SUBBY_ERR_CUDA);
  }
  if (subby::plan_status_async(plan, sl.h_err, st)) return bail(SUBBY_ERR_CUDA);
  if (cudaEventRecord(sl.done, st) != cudaSuccess) return bail(SUBBY_ERR_CUDA);
  start_run(S, slot_i, {j});
  return SUBBY_OK;
}

int pack_tiles(const subby_server *S, int R) { return S->pack_tiles_r[R <= 64 ? 0 : R <= 256 ? 1 : 2]; }

bool packable(const subby_server *S, const SJob *j) {
  return S->pack && !j->nopack && j->d.A == 4 && j->d.R >= 2 && j->cost_ms <= S->short_ms;
}

bool same_group(const SJob *a, const SJob *b) {
  auto key = [](const SJob *j) {
    const bool c = j->d.want & SUBBY_WANT_COUNTS;
    return (c ? (j->d.counts_kind == SUBBY_COUNTS_F81 ? 2 : 1) : 0) * 4 + (c ? j->d.mask_mode : 0);
  };
  return key(a) == key(b);
}

// A batch of short A = 4 jobs waiting together: their tokens gathered into
// the slot arena, one launch of the packed persistent kernel over the
// flattened (job, 256-column tile) queue, each job's outputs copied out.
// Jobs whose plan does not take the kernel are marked and left out (they
// stay waiting for the one-job path).  Returns the number of jobs launched
// (0: nothing enqueued), or a negative status after which every job of the
// batch completes with that status (nothing of it is then in flight).
int launch_batch(subby_server *S, std::vector<SJob *> &batch) {
  const int slot_i = S->free_slots.back();
  Slot &sl = S->slots[slot_i];
  cudaStream_t st = sl.s_hi;
  auto bail = [&](int rc) {
    cudaStreamSynchronize(st);
    cudaGetLastError();
    return rc;
  };
  const bool counts = batch[0]->d.want & SUBBY_WANT_COUNTS;
  const bool f81 = counts && batch[0]->d.counts_kind == SUBBY_COUNTS_F81;
  const int mask = counts ? batch[0]->d.mask_mode : SUBBY_MASK_NONE;
  const int n = (int)batch.size();
  std::vector<subby_plan *> plans(n, nullptr);
  for (int i = 0; i < n; ++i) {
    const int rc = plan_for(S, batch[i], &plans[i]);
    if (rc) return rc;
  }
  // device layout: per job tokens and outputs, then the queue
  std::vector<size_t> o_tok(n), o_out(n);
  size_t off = 0;
  long long ntiles = 0;
  for (int i = 0; i < n; ++i) {
    const subby_job &d = batch[i]->d;
    o_tok[i] = off;
    off += align256((size_t)4 * d.R * d.C);
    o_out[i] = off;
    off += align256((size_t)4 * d.C) + align256((size_t)64 * d.C) + align256((size_t)16 * d.C);
    ntiles += (d.C + 255) / 256;
  }
  const size_t o_kp = off;
  off += align256(sizeof(KParams) * n);
  const size_t o_items = off;
  off += align256(sizeof(int4) * ntiles);
  const size_t o_ints = off;
  off += 256;
  if (grow_arena(S, sl, off, st)) return bail(SUBBY_ERR_NOMEM);
  char *base = static_cast<char *>(sl.arena);
  // host staging: parameters, items, queue words, then the row maps
  size_t rm_bytes = 0;
  for (SJob *j : batch) rm_bytes += align256((size_t)4 * j->rowmap.size());
  const size_t stage = (o_ints + 256 - o_kp) + rm_bytes;
  if (stage > sl.h_stage_bytes) {
    if (sl.h_stage) cudaFreeHost(sl.h_stage);
    sl.h_stage = nullptr;
    sl.h_stage_bytes = 0;
    if (cudaHostAlloc(&sl.h_stage, stage * 2, cudaHostAllocPortable) != cudaSuccess) return bail(SUBBY_ERR_NOMEM);
    sl.h_stage_bytes = stage * 2;
  }
  char *hs = static_cast<char *>(sl.h_stage);
  KParams *hkp = reinterpret_cast<KParams *>(hs);
  int4 *hit = reinterpret_cast<int4 *>(hs + (o_items - o_kp));
  int *hq = reinterpret_cast<int *>(hs + (o_ints - o_kp));
  char *hrm = hs + (o_ints + 256 - o_kp);
  size_t smem = 0;
  int njobs = 0;
  long long nit = 0;
  std::vector<SJob *> taken;
  std::vector<subby_plan *> taken_plans;
  for (int i = 0; i < n; ++i) {
    SJob *j = batch[i];
    const subby_job &d = j->d;
    int32_t *d_tok = reinterpret_cast<int32_t *>(base + o_tok[i]);
    float *d_ll = (d.want & SUBBY_WANT_LOGLIKE) ? reinterpret_cast<float *>(base + o_out[i]) : nullptr;
    float *d_ct = (d.want & SUBBY_WANT_COUNTS)
                      ? reinterpret_cast<float *>(base + o_out[i] + align256((size_t)4 * d.C)) : nullptr;
    float *d_rp = (d.want & SUBBY_WANT_ROOTPROB)
                      ? reinterpret_cast<float *>(base + o_out[i] + align256((size_t)4 * d.C) +
                                                  align256((size_t)64 * d.C)) : nullptr;
    size_t sm_i = 0;
    int block = 0;
    if (subby::plan_tree4_params(plans[i], d_tok, d.C, d_ll, d_ct, d_rp, d.counts_kind, mask, &hkp[njobs], &sm_i,
                                 &block, st) != 0) {
      j->nopack = true;   // runs on the one-job path instead
      continue;
    }
    smem = std::max(smem, sm_i);
    const int32_t *rowmap = nullptr;
    if (!j->rowmap.empty()) {
      std::memcpy(hrm, j->rowmap.data(), 4 * j->rowmap.size());
      rowmap = reinterpret_cast<const int32_t *>(hrm);
      hrm += align256(4 * j->rowmap.size());
    }
    const int rc = subby_gather_rows(d.alignment, d.pitch, rowmap, d.R, d.C, d_tok, st);
    if (rc) return bail(rc);
    const int span = 256 * pack_tiles(S, d.R);
    for (int c0 = 0; c0 < d.C; c0 += span) hit[nit++] = make_int4(njobs, c0, std::min(d.C, c0 + span), 0);
    const bool want_k[3] = {d_ll != nullptr, d_ct != nullptr, d_rp != nullptr};
    const size_t n_out[3] = {(size_t)4 * d.C, (size_t)64 * d.C, (size_t)16 * d.C};
    for (int k = 0; k < 3; ++k)
      if (want_k[k] && !(j->out[k] = S->pinned.get(n_out[k]))) return bail(SUBBY_ERR_NOMEM);
    taken.push_back(j);
    taken_plans.push_back(plans[i]);
    ++njobs;
  }
  if (njobs == 0) return 0;
  hq[0] = 0;          // head
  hq[1] = (int)nit;   // published: every item
  hq[2] = 1;          // closed
  hq[3] = 0;          // err
  cudaError_t e = cudaMemcpyAsync(base + o_kp, hs, o_ints + 256 - o_kp, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return bail(SUBBY_ERR_CUDA);
  int *d_q = reinterpret_cast<int *>(base + o_ints);
  const T4Queue q{reinterpret_cast<const KParams *>(base + o_kp), reinterpret_cast<const int4 *>(base + o_items),
                  d_q, d_q + 1, d_q + 2, 1, d_q + 3};
  const int grid = (int)std::min<long long>(nit, S->nsm);
  if (subby::launch_tree4_packed(q, f81, mask, grid, 256, smem, st) != 0) return bail(SUBBY_ERR_CUDA);
  for (int i = 0; i < njobs; ++i) {
    SJob *j = taken[i];
    const KParams &k = hkp[i];
    const subby_job &d = j->d;
    int ce = 0;
    if (k.logL) ce = subby::launch_copy_rows(j->out[0], 0, k.logL, 0, (size_t)4 * d.C, 1, st);
    if (!ce && k.counts) ce = subby::launch_copy_rows(j->out[1], 0, k.counts, 0, (size_t)64 * d.C, 1, st);
    if (!ce && k.rootp) ce = subby::launch_copy_rows(j->out[2], 0, k.rootp, 0, (size_t)16 * d.C, 1, st);
    if (!ce && subby::plan_mark_used(taken_plans[i], st) != 0) ce = 1;
    if (ce) return bail(SUBBY_ERR_CUDA);
  }
  if (cudaMemcpyAsync(sl.h_err, d_q + 3, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaEventRecord(sl.done, st) != cudaSuccess)
    return bail(SUBBY_ERR_CUDA);
  start_run(S, slot_i, taken);
  S->packed_jobs += njobs;
  S->packed_launches += 1;
  return njobs;
}

void finish(subby_server *S, SJob *j, int status) {
  j->status = status;
  j->t_finish = S->now();
  {
    std::lock_guard<std::mutex> g(S->mu);
    S->completed.push_back(j);
  }
  S->cv_done.notify_all();
}

void release_outputs(subby_server *S, SJob *j) {
  for (int k = 0; k < 3; ++k)
    if (j->out[k]) S->pinned.put(j->out[k]), j->out[k] = nullptr;
}

void engine(subby_server *S) {
  cudaSetDevice(S->device);
  while (true) {
    bool did = false;
    const auto t_it = Clock::now();
    std::vector<void *> rel;
    {
      std::lock_guard<std::mutex> g(S->mu);
      while (!S->submitted.empty()) {
        S->waiting.push_back(S->submitted.front());
        S->submitted.pop_front();
        did = true;
      }
      rel.swap(S->to_release);
    }
    for (void *p : rel) S->pinned.put(p);
    // short A = 4 jobs waiting together: one packed launch per batch.  (The
    // settings are read only while jobs wait: subby_server_set changes them
    // only before the first submission, under the lock the engine took to
    // move that job here.)
    while (!S->waiting.empty() && S->pack && !S->free_slots.empty()) {
      std::vector<SJob *> cand;
      long long cols = 0;
      size_t bytes = 0;
      for (SJob *w : S->waiting) {
        if (!packable(S, w) || plan_busy(S, w->key) || (!cand.empty() && !same_group(cand[0], w))) continue;
        if (S->used + bytes + w->bytes > S->budget && !(S->inflight.empty() && cand.empty())) continue;
        cand.push_back(w);
        cols += w->d.C;
        bytes += w->bytes;
        if ((int)cand.size() >= S->pack_max_jobs || cols >= S->pack_max_cols) break;
      }
      if (cand.empty()) break;
      did = true;
      const double ts = S->now();
      for (SJob *j : cand) {
        S->waiting.erase(std::find(S->waiting.begin(), S->waiting.end(), j));
        j->t_start = ts;
      }
      const int rc = launch_batch(S, cand);
      if (rc < 0) {
        for (SJob *j : cand) {
          release_outputs(S, j);
          finish(S, j, rc);
        }
        continue;
      }
      // jobs the batch left out (their plan does not take the packed kernel)
      for (SJob *j : cand)
        if (j->slot < 0) {
          j->t_start = -1;
          S->waiting.push_back(j);
        }
    }
    // one-job runs: shortest estimated job first, aged by its wait
    while (!S->waiting.empty() && !S->free_slots.empty()) {
      const double tn = S->now();
      SJob *best = nullptr;
      double best_score = 0;
      for (SJob *w : S->waiting) {
        if (packable(S, w) || !fits(S, w)) continue;
        const double sc = w->cost_ms - S->aging * 1e3 * (tn - w->arrival);
        if (!best || sc < best_score) best = w, best_score = sc;
      }
      if (!best) break;
      S->waiting.erase(std::find(S->waiting.begin(), S->waiting.end(), best));
      best->t_start = S->now();
      const int rc = launch(S, best);
      did = true;
      if (rc) {
        release_outputs(S, best);
        finish(S, best, rc);
      }
    }
    // completions
    for (size_t i = 0; i < S->inflight.size();) {
      Run *r = S->inflight[i];
      Slot &sl = S->slots[r->slot];
      const cudaError_t q = cudaEventQuery(sl.done);
      if (q == cudaErrorNotReady) {
        ++i;
        continue;
      }
      did = true;
      int status = SUBBY_OK;
      if (q != cudaSuccess) {
        cudaGetLastError();
        status = SUBBY_ERR_CUDA;
      } else if (*sl.h_err) {
        status = SUBBY_ERR_TIMEOUT;
      }
      for (SJob *j : r->jobs) {
        auto it = S->plans.find(j->key);
        if (it != S->plans.end()) {
          it->second.busy = false;
          if (r->jobs.size() == 1) subby_plan_trim(it->second.p);  // workspace back to the pool, in stream order
        }
        finish(S, j, status);
      }
      sl.run = nullptr;
      S->free_slots.push_back(r->slot);
      S->used -= r->bytes;
      S->inflight.erase(S->inflight.begin() + i);
      delete r;
    }
    if (did) S->busy_s += std::chrono::duration<double>(Clock::now() - t_it).count();
    S->pub_busy_s.store(S->busy_s);
    S->pub_plans.store((int)S->plans.size());
    S->pub_inflight.store((int)S->inflight.size());
    S->pub_waiting.store((int)S->waiting.size());
    S->pub_packed_jobs.store(S->packed_jobs);
    S->pub_packed_launches.store(S->packed_launches);
    if (S->stop.load() && S->inflight.empty() && S->waiting.empty()) {
      std::lock_guard<std::mutex> g(S->mu);
      if (S->submitted.empty()) break;
    }
    if (!did) {
      std::unique_lock<std::mutex> g(S->mu);
      S->cv_work.wait_for(g, std::chrono::microseconds(S->inflight.empty() ? 2000 : 50));
    }
  }
}

}  // namespace

extern "C" {

int subby_server_create(int max_inflight, size_t device_budget, size_t pinned_prewarm_bytes, subby_server **out) {
  if (!out || max_inflight < 2 || max_inflight > 64) return SUBBY_ERR_ARG;
  *out = nullptr;
  auto *S = new subby_server();
  cudaGetDevice(&S->device);
  cudaDeviceGetAttribute(&S->nsm, cudaDevAttrMultiProcessorCount, S->device);
  S->max_inflight = max_inflight;
  S->short_slots = std::min(2, max_inflight - 1);
  S->budget = device_budget;
  S->t0 = Clock::now();
  {
    cudaMemPoolProps pr{};
    pr.allocType = cudaMemAllocationTypePinned;
    pr.location.type = cudaMemLocationTypeDevice;
    pr.location.id = S->device;
    if (cudaMemPoolCreate(&S->pool, &pr) != cudaSuccess) {
      cudaGetLastError();
      S->pool = nullptr;
    } else {
      uint64_t keep = ~0ull;  // arenas are long-lived: keep freed blocks
      cudaMemPoolSetAttribute(S->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
  }
  int lo = 0, hi = 0;
  cudaDeviceGetStreamPriorityRange(&lo, &hi);
  S->slots.resize(max_inflight);
  for (int i = 0; i < max_inflight; ++i) {
    Slot &sl = S->slots[i];
    cudaError_t e = cudaStreamCreateWithPriority(&sl.s_norm, cudaStreamNonBlocking, lo);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&sl.s_hi, cudaStreamNonBlocking, hi);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaHostAlloc((void **)&sl.h_err, sizeof(int), cudaHostAllocPortable);
    if (e == cudaSuccess) e = cudaHostAlloc((void **)&sl.h_rowmap, sizeof(int32_t) * 65536, cudaHostAllocPortable);
    if (e != cudaSuccess) {
      subby_server_destroy(S);
      return SUBBY_ERR_CUDA;
    }
    *sl.h_err = 0;
    S->free_slots.push_back(i);
  }
  if (pinned_prewarm_bytes) S->pinned.prewarm(pinned_prewarm_bytes, 2);
  S->th = std::thread(engine, S);
  *out = S;
  return SUBBY_OK;
}

int subby_server_submit(subby_server *S, const subby_job *d) {
  if (!S || !d) return SUBBY_ERR_ARG;
  if (!d->parent_index || !d->distances || !d->eigenvalues || !d->eigenvectors || !d->pi || !d->alignment)
    return SUBBY_ERR_ARG;
  if (d->R < 1 || d->R > 65535 || d->C < 1 || d->pitch < d->C || d->A < 2 || d->A > 64) return SUBBY_ERR_ARG;
  if (!(d->want & (SUBBY_WANT_LOGLIKE | SUBBY_WANT_COUNTS | SUBBY_WANT_ROOTPROB))) return SUBBY_ERR_ARG;
  if (d->mask_mode != SUBBY_MASK_NONE && d->mask_mode != SUBBY_MASK_AUTO) return SUBBY_ERR_UNSUPPORTED;
  if (d->counts_kind != SUBBY_COUNTS_EIGEN && d->counts_kind != SUBBY_COUNTS_F81) return SUBBY_ERR_ARG;
  auto *j = new SJob();
  j->d = *d;
  const int R = d->R, A = d->A;
  j->parent.assign(d->parent_index, d->parent_index + R);
  j->dist.assign(d->distances, d->distances + R);
  j->ev.assign(d->eigenvalues, d->eigenvalues + A);
  j->V.assign(d->eigenvectors, d->eigenvectors + (size_t)A * A);
  j->pi.assign(d->pi, d->pi + A);
  if (d->row_map) j->rowmap.assign(d->row_map, d->row_map + R);
  j->d.parent_index = nullptr;
  j->d.distances = j->d.eigenvalues = j->d.eigenvectors = j->d.pi = nullptr;
  j->d.row_map = nullptr;
  j->key = job_key(*j);
  j->cost_ms = job_cost_ms(*d);
  j->bytes = job_bytes(R, d->C, A);
  {
    std::lock_guard<std::mutex> g(S->mu);
    j->arrival = d->arrival >= 0 ? d->arrival : S->now();
    j->handle = S->next_handle++;
    S->submitted.push_back(j);
  }
  S->cv_work.notify_one();
  return SUBBY_OK;
}

int subby_server_wait(subby_server *S, subby_job_result *out, int max, int timeout_ms, int *n) {
  if (!S || !n || (max > 0 && !out)) return SUBBY_ERR_ARG;
  *n = 0;
  std::unique_lock<std::mutex> g(S->mu);
  if (S->completed.empty() && timeout_ms > 0)
    S->cv_done.wait_for(g, std::chrono::milliseconds(timeout_ms), [&] { return !S->completed.empty(); });
  while (*n < max && !S->completed.empty()) {
    SJob *j = S->completed.front();
    S->completed.pop_front();
    subby_job_result &r = out[(*n)++];
    r.tag = j->d.tag;
    r.handle = j->handle;
    r.status = j->status;
    r.logLike = static_cast<const float *>(j->out[0]);
    r.counts = static_cast<const float *>(j->out[1]);
    r.rootProb = static_cast<const float *>(j->out[2]);
    r.t_arrival = j->arrival;
    r.t_start = j->t_start;
    r.t_finish = j->t_finish;
    S->held[j->handle] = j;
  }
  return SUBBY_OK;
}

int subby_server_release(subby_server *S, int64_t handle) {
  if (!S) return SUBBY_ERR_ARG;
  SJob *j = nullptr;
  {
    std::lock_guard<std::mutex> g(S->mu);
    auto it = S->held.find(handle);
    if (it == S->held.end()) return SUBBY_ERR_ARG;
    j = it->second;
    S->held.erase(it);
    for (void *p : j->out)
      if (p) S->to_release.push_back(p);
  }
  delete j;
  return SUBBY_OK;
}

int subby_server_set(subby_server *S, const char *key, double value) {
  if (!S || !key) return SUBBY_ERR_ARG;
  std::lock_guard<std::mutex> g(S->mu);
  if (!S->submitted.empty() || S->next_handle > 1) return SUBBY_ERR_ARG;  // before the first submission
  const std::string k(key);
  if (k == "short_ms" && value >= 0) S->short_ms = value;
  else if (k == "slice_ms" && value > 0) S->slice_ms = value;
  else if (k == "aging" && value >= 0) S->aging = value;
  else if (k == "wave_cols" && value >= 0 && value <= (1 << 30)) S->wave_cols = (int)value;
  else if (k == "short_slots" && value >= 0 && value < S->max_inflight) S->short_slots = (int)value;
  else if (k == "plan_cache" && value >= 1) S->plan_cache = (int)value;
  else if (k == "pack") S->pack = value != 0;
  else if (k == "pack_max_jobs" && value >= 1 && value <= 4096) S->pack_max_jobs = (int)value;
  else if (k == "pack_tiles_r64" && value >= 1 && value <= 64) S->pack_tiles_r[0] = (int)value;
  else if (k == "pack_tiles_r256" && value >= 1 && value <= 64) S->pack_tiles_r[1] = (int)value;
  else if (k == "pack_tiles_big" && value >= 1 && value <= 64) S->pack_tiles_r[2] = (int)value;
  else return SUBBY_ERR_ARG;
  return SUBBY_OK;
}

double subby_server_clock(subby_server *S) { return S ? S->now() : 0.0; }

int subby_server_stats(subby_server *S, double *engine_busy_s, int *plans_cached, int *inflight, int *waiting,
                       long long *packed_jobs, long long *packed_launches) {
  if (!S) return SUBBY_ERR_ARG;
  if (engine_busy_s) *engine_busy_s = S->pub_busy_s.load();
  if (plans_cached) *plans_cached = S->pub_plans.load();
  if (inflight) *inflight = S->pub_inflight.load();
  if (waiting) *waiting = S->pub_waiting.load();
  if (packed_jobs) *packed_jobs = S->pub_packed_jobs.load();
  if (packed_launches) *packed_launches = S->pub_packed_launches.load();
  return SUBBY_OK;
}

int subby_debug_packed_queue_wait(int polls, int grid, int *gave_up) {
  if (polls < 1 || polls > 100000 || grid < 1 || !gave_up) return SUBBY_ERR_ARG;
  int dev = 0, nsm = 0, maxsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  grid = std::min(grid, nsm);
  int *d = nullptr;
  if (cudaMalloc(&d, 4 * sizeof(int)) != cudaSuccess) return SUBBY_ERR_NOMEM;
  // an open queue with nothing published: every CTA's claim waits and gives up
  cudaError_t e = cudaMemset(d, 0, 4 * sizeof(int));
  const T4Queue q{nullptr, nullptr, d, d + 1, d + 2, polls, d + 3};
  if (e == cudaSuccess) {
    // at least half the SM's shared memory: one CTA (owner of the tensor memory) per SM
    const int lr = subby::launch_tree4_packed(q, false, SUBBY_MASK_AUTO, grid, 256, (size_t)(maxsm / 2 + 4096), 0);
    e = lr ? (cudaError_t)lr : cudaDeviceSynchronize();
  }
  int h[4] = {0, 0, 0, 0};
  if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return SUBBY_ERR_CUDA;
  *gave_up = h[3];
  return h[3] ? SUBBY_ERR_TIMEOUT : SUBBY_OK;
}

int subby_server_destroy(subby_server *S) {
  if (!S) return SUBBY_ERR_ARG;
  if (S->th.joinable()) {
    S->stop.store(true);
    S->cv_work.notify_all();
    S->th.join();
  }
  cudaSetDevice(S->device);
  cudaDeviceSynchronize();
  for (auto &kv : S->plans) subby_plan_destroy(kv.second.p);
  for (auto &kv : S->held) delete kv.second;
  for (SJob *j : S->completed) delete j;
  for (Slot &sl : S->slots) {
    if (sl.arena) cudaFree(sl.arena);
    if (sl.s_norm) cudaStreamDestroy(sl.s_norm);
    if (sl.s_hi) cudaStreamDestroy(sl.s_hi);
    if (sl.h_err) cudaFreeHost(sl.h_err);
    if (sl.h_rowmap) cudaFreeHost(sl.h_rowmap);
    if (sl.h_stage) cudaFreeHost(sl.h_stage);
    if (sl.done) cudaEventDestroy(sl.done);
  }
  if (S->pool) cudaMemPoolDestroy(S->pool);
  delete S;
  return SUBBY_OK;
}

}  // extern "C"
