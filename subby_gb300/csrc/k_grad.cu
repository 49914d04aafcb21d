// Gradient of sum_c g_c logL_c for reversible models from the walk's eigen
// staging (k_walk mode 1: D~ = s Vd^T D, U~ = Vu^T U per branch and column,
// unmasked).  Both gradients of subby/jax/vjp.py:62-133 and the
// exchangeability gradient are functions of one A x A matrix per branch,
//   X_n = sum_c g_c D~_nc (x) U~_nc :
//   d/dt_n      = sum_k mu_k e^{mu_k t_n} X_n[k][k]
//   d/dS~ = V (sum_n J_n o X_n) V^T        (formed on the host in FP64).
// k_xgram forms X_n: per (branch, block of 4096 columns) each thread owns a
// 4 x 4 block of (k, l) for a subset of the columns (two 16-byte loads and
// 16 FMAs per column), the column subsets are reduced in shared memory and
// the block's sum is added to X_n in FP64 (one atomic per entry per block).
#include "common.cuh"

namespace subby {
namespace {

constexpr int kXThreads = 256;
constexpr int kXCols = 4096;

template <int A>
__global__ void __launch_bounds__(kXThreads) k_xgram(const float *__restrict__ sa, const float *__restrict__ sb,
                                                     const float *__restrict__ g, int c_base, int c_count, int R,
                                                     double *__restrict__ X) {
  constexpr int KB = A / 4, NB = KB * KB;
  constexpr int GROUPS = (kXThreads / NB) > 0 ? kXThreads / NB : 1;
  constexpr int THREADS = NB * GROUPS;
  static_assert(NB <= kXThreads, "A too large");
  __shared__ float s_part[THREADS * 16];
  const int t = threadIdx.x;
  const bool busy = t < THREADS;
  const int grp = busy ? t / NB : 0, b = busy ? t % NB : 0;
  const int kb = b / KB, lb = b % KB;
  const int nblk = (c_count + kXCols - 1) / kXCols;
  const long long items = (long long)(R - 1) * nblk;
  for (long long it = blockIdx.x; it < items; it += gridDim.x) {
    const int n = 1 + (int)(it / nblk);
    const int c0 = (int)(it % nblk) * kXCols, c1 = min(c_count, c0 + kXCols);
    float acc[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) acc[q] = 0.f;
    auto add = [&](float4 d, const float4 u, float w) {
      d.x *= w, d.y *= w, d.z *= w, d.w *= w;
      const float dv[4] = {d.x, d.y, d.z, d.w}, uv[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[4 * i + j] = fmaf(dv[i], uv[j], acc[4 * i + j]);
    };
    auto ld = [&](const float *base, int c, int blk) {
      return __ldg(reinterpret_cast<const float4 *>(base + ((size_t)(n - 1) * c_count + c) * A) + blk);
    };
    if (busy) {
      int c = c0 + grp;
      // four columns' loads in flight before their FMAs (the pass is load-latency-bound)
      for (; c + 3 * GROUPS < c1; c += 4 * GROUPS) {
        float4 d[4], u[4];
        float w[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          d[q] = ld(sa, c + q * GROUPS, kb);
          u[q] = ld(sb, c + q * GROUPS, lb);
          w[q] = g ? __ldg(g + c_base + c + q * GROUPS) : 1.f;
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) add(d[q], u[q], w[q]);
      }
      for (; c < c1; c += GROUPS) add(ld(sa, c, kb), ld(sb, c, lb), g ? __ldg(g + c_base + c) : 1.f);
    }
    __syncthreads();  // the previous item's reads of s_part are done
    if (busy)
#pragma unroll
      for (int q = 0; q < 16; ++q) s_part[(grp * NB + b) * 16 + q] = acc[q];
    __syncthreads();
    for (int e = t; e < NB * 16; e += blockDim.x) {
      double s = 0.0;
      for (int gi = 0; gi < GROUPS; ++gi) s += (double)s_part[gi * NB * 16 + e];
      const int bb = e / 16, q = e % 16;
      const int k = 4 * (bb / KB) + q / 4, l = 4 * (bb % KB) + q % 4;
      atomicAdd(X + ((size_t)n * A + k) * A + l, s);
    }
  }
}

template <int A>
int xgram_launch(const float *sa, const float *sb, const float *g, int c_base, int c_count, int R, double *X,
                 int grid, cudaStream_t s) {
  k_xgram<A><<<grid, kXThreads, 0, s>>>(sa, sb, g, c_base, c_count, R, X);
  return (int)cudaGetLastError();
}

}  // namespace

int xgram_items(int R, int c_count) { return (R - 1) * ((c_count + kXCols - 1) / kXCols); }

int launch_xgram(int A, const float *sa, const float *sb, const float *g, int c_base, int c_count, int R, double *X,
                 int grid, cudaStream_t s) {
  switch (A) {
    case 16: return xgram_launch<16>(sa, sb, g, c_base, c_count, R, X, grid, s);
    case 20: return xgram_launch<20>(sa, sb, g, c_base, c_count, R, X, grid, s);
    case 32: return xgram_launch<32>(sa, sb, g, c_base, c_count, R, X, grid, s);
    case 64: return xgram_launch<64>(sa, sb, g, c_base, c_count, R, X, grid, s);
    default: return -1;
  }
}

}  // namespace subby
