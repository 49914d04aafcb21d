// Counts of irreversible models: the complex eigenbasis accumulation and
// back-transform (subby/oracle/oracle.py:537-740; subby/jax/eigensub.py:
// 234-434) over the raw per-branch staging of the walk (k_walk mode 3):
//   stage_a[n-1][c][a] = D_n(c, a) s_n(c),  stage_b[n-1][c][b] = U_n(c, b),
// s_n = 2^(e_D + e_U - e_root) / P(column), zero for masked branches.
//
//   D~_k = sum_a Ds_a Vinv[k][a],  U~_l = sum_b U_b V[b][l]        (complex)
//   C_kl += D~_k J_n[k][l] U~_l                                    (complex)
//   counts_ij = Re (V C Vinv)_ij on the diagonal, Re R_ij (V C Vinv)_ij off
//   it, R = V diag(mu) Vinv.
//
// Layout: a CTA of 256 threads holds G columns; the A^2 complex entries of a
// column's C are split over TPC = A^2 / 16 threads (16 entries each, in
// registers).  Per branch the CTA projects its columns' D and U into shared
// memory (double-buffered, one barrier per branch) and each thread updates
// its 16 entries with J_n read through L1.  The epilogue forms T = C Vinv and
// V T through shared memory.  Complex tables (P.cx): J (R x A x A), V, Vinv,
// R (A x A each), FP32 pairs.
#include "common.cuh"

namespace subby {

namespace {

constexpr int kCxThreads = 256;
constexpr int kCxE = 16;  // complex entries of C per thread

template <int A>
struct CxGeo {
  static constexpr int TPC = A * A / kCxE;     // threads per column
  static constexpr int G = kCxThreads / TPC;   // columns per CTA
  static constexpr int THREADS = G * TPC;      // busy threads (250 at A = 20)
  static_assert(A * A % kCxE == 0, "A^2 must be a multiple of 16");
};

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 cfma(float2 a, float2 b, float2 c) {  // a b + c
  return make_float2(fmaf(a.x, b.x, fmaf(-a.y, b.y, c.x)), fmaf(a.x, b.y, fmaf(a.y, b.x, c.y)));
}

template <int A>
constexpr size_t cx_smem() {
  using Gm = CxGeo<A>;
  return (size_t)(2 * A * A + 2 * Gm::G * 2 * A + Gm::G * A * A) * sizeof(float2);
}

// PB: per-branch counts (R, A, A, C) instead of the sum over branches
template <int A, bool PB>
__global__ void __launch_bounds__(kCxThreads) k_acc_cx(const KParams P, const float *__restrict__ sa,
                                                       const float *__restrict__ sb, int c_base, int c_count) {
  using Gm = CxGeo<A>;
  constexpr int TPC = Gm::TPC, G = Gm::G;
  extern __shared__ __align__(16) float2 s_cx[];
  float2 *sV = s_cx;                  // A x A: V[i][k]
  float2 *sVi = sV + A * A;           // A x A: Vinv[k][j]
  float2 *sP = sVi + A * A;           // [2][G][2A]: D~ (k < A), U~ (A + l)
  float2 *sC = sP + 2 * G * 2 * A;    // [G][A][A]: C, then T = C Vinv
  const float2 *J = P.cx;
  const float2 *Vg = P.cx + (size_t)P.R * A * A;
  const float2 *Vig = Vg + A * A;
  const float2 *Rg = Vig + A * A;
  const int t = threadIdx.x;
  for (int e = t; e < A * A; e += blockDim.x) {
    sV[e] = Vg[e];
    sVi[e] = Vig[e];
  }
  __syncthreads();  // V, Vinv visible to every thread before the first projection
  const bool busy = t < Gm::THREADS;
  const int g = busy ? t / TPC : 0, p = busy ? t % TPC : 0;
  const int ngroups = (c_count + G - 1) / G;
  const int C = P.C;
  float2 *myC = sC + (size_t)g * A * A;

  // back-transform of the thread's 16 entries and the stores (row: branch
  // n for PB, else 0); every thread calls it (barriers inside)
  auto epilogue = [&](const float2 (&acc)[kCxE], int row, bool valid, size_t col) {
    __syncthreads();  // earlier readers of sC are done
    if (busy)
#pragma unroll
      for (int i = 0; i < kCxE; ++i) myC[p * kCxE + i] = acc[i];
    __syncthreads();
    float2 T[kCxE];
    if (busy)
#pragma unroll
      for (int i = 0; i < kCxE; ++i) {
        const int e = p * kCxE + i, k = e / A, j = e % A;
        float2 s = make_float2(0.f, 0.f);
#pragma unroll 4
        for (int l = 0; l < A; ++l) s = cfma(myC[k * A + l], sVi[l * A + j], s);
        T[i] = s;
      }
    __syncthreads();
    if (busy)
#pragma unroll
      for (int i = 0; i < kCxE; ++i) myC[p * kCxE + i] = T[i];
    __syncthreads();
    if (busy && valid) {
      float *out = P.counts + (size_t)row * A * A * C + col;
#pragma unroll
      for (int i = 0; i < kCxE; ++i) {
        const int e = p * kCxE + i, ii = e / A, j = e % A;
        float2 s = make_float2(0.f, 0.f);
#pragma unroll 4
        for (int k = 0; k < A; ++k) s = cfma(sV[ii * A + k], myC[k * A + j], s);
        out[(size_t)e * C] = (ii == j) ? s.x : cmul(__ldg(Rg + e), s).x;
      }
    }
  };

  for (int grp = blockIdx.x; grp < ngroups; grp += gridDim.x) {
    const int cc = grp * G + g;
    const bool valid = busy && cc < c_count;
    const int ccl = min(cc, c_count - 1);
    const size_t col = (size_t)c_base + ccl;
    float2 acc[kCxE];
#pragma unroll
    for (int i = 0; i < kCxE; ++i) acc[i] = make_float2(0.f, 0.f);
    for (int n = 1; n < P.R; ++n) {
      float2 *buf = sP + ((size_t)(n & 1) * G + g) * 2 * A;
      if (busy) {
        const size_t srow = ((size_t)(n - 1) * c_count + ccl) * A;
        for (int o = p; o < 2 * A; o += TPC) {
          float2 s = make_float2(0.f, 0.f);
          if (o < A) {
            const float *d = sa + srow;
#pragma unroll 4
            for (int a = 0; a < A; ++a) {
              const float x = __ldg(d + a);
              const float2 v = sVi[o * A + a];
              s.x = fmaf(x, v.x, s.x);
              s.y = fmaf(x, v.y, s.y);
            }
          } else {
            const float *u = sb + srow;
            const int l = o - A;
#pragma unroll 4
            for (int b = 0; b < A; ++b) {
              const float x = __ldg(u + b);
              const float2 v = sV[b * A + l];
              s.x = fmaf(x, v.x, s.x);
              s.y = fmaf(x, v.y, s.y);
            }
          }
          buf[o] = s;
        }
      }
      __syncthreads();
      if (busy) {
        const float2 *Jn = J + (size_t)n * A * A + p * kCxE;
#pragma unroll
        for (int i = 0; i < kCxE; ++i) {
          const int e = p * kCxE + i, k = e / A, l = e % A;
          const float2 x = cmul(buf[k], __ldg(Jn + i));
          acc[i] = PB ? cmul(x, buf[A + l]) : cfma(x, buf[A + l], acc[i]);
        }
      }
      if constexpr (PB) {
        epilogue(acc, n, valid, col);
      }
    }
    if constexpr (!PB) epilogue(acc, 0, valid, col);
  }
}

template <int A, bool PB>
int cx_launch(const KParams &p, const float *sa, const float *sb, int c_base, int c_count, int grid,
              cudaStream_t s) {
  const size_t smem = cx_smem<A>();
  cudaError_t e = cudaFuncSetAttribute(k_acc_cx<A, PB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return (int)e;
  k_acc_cx<A, PB><<<grid, kCxThreads, smem, s>>>(p, sa, sb, c_base, c_count);
  return (int)cudaGetLastError();
}

template <int A>
int cx_launch_pb(const KParams &p, bool pb, const float *sa, const float *sb, int c_base, int c_count, int grid,
                 cudaStream_t s) {
  return pb ? cx_launch<A, true>(p, sa, sb, c_base, c_count, grid, s)
            : cx_launch<A, false>(p, sa, sb, c_base, c_count, grid, s);
}

}  // namespace

bool cx_supported(int A) { return A == 4 || A == 8 || A == 16 || A == 20 || A == 32 || A == 64; }

int cx_columns_per_cta(int A) {
  switch (A) {
    case 4: return CxGeo<4>::G;
    case 8: return CxGeo<8>::G;
    case 16: return CxGeo<16>::G;
    case 20: return CxGeo<20>::G;
    case 32: return CxGeo<32>::G;
    case 64: return CxGeo<64>::G;
    default: return 1;
  }
}

int launch_acc_cx(const KParams &p, int A, bool pb, const float *sa, const float *sb, int c_base, int c_count,
                  int grid, cudaStream_t s) {
  switch (A) {
    case 4: return cx_launch_pb<4>(p, pb, sa, sb, c_base, c_count, grid, s);
    case 8: return cx_launch_pb<8>(p, pb, sa, sb, c_base, c_count, grid, s);
    case 16: return cx_launch_pb<16>(p, pb, sa, sb, c_base, c_count, grid, s);
    case 20: return cx_launch_pb<20>(p, pb, sa, sb, c_base, c_count, grid, s);
    case 32: return cx_launch_pb<32>(p, pb, sa, sb, c_base, c_count, grid, s);
    case 64: return cx_launch_pb<64>(p, pb, sa, sb, c_base, c_count, grid, s);
    default: return -1;
  }
}

}  // namespace subby
