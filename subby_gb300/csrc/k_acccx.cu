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
// Per-branch models run one launch per group of branches sharing a system
// (P.cx_tab, P.cx_br), the summed counts accumulating in the output.
//
// Layout: a CTA of 256 threads holds G columns; the A^2 complex entries of a
// column's C are split over TPC = A^2 / 16 threads (16 entries each, in
// registers).  Per branch the CTA projects its columns' D and U into shared
// memory (double-buffered and software-pipelined: branch n + 1 is loaded
// and projected while branch n accumulates; one barrier per branch) and each
// thread updates its 16 entries with J_n, staged in shared memory once per
// CTA and branch.  The epilogue forms T = C Vinv and
// V T through shared memory.  Complex tables (P.cx): J (R x A x A), V, Vinv,
// R, Vinv^T, V^T (A x A each), FP32 pairs; then V, Vinv, Vinv^T, V^T in FP64
// pairs for the FP64 back-transform (k_bt_cx).  P.cx_exact selects the
// pair (Vinv^T, V^T) in place of (V, Vinv): the expected counts of the
// process M(t) = e^{Qt} itself (D~ = D V, U~ = Vinv U, Vinv^T C V^T), which
// differ from the reference's formula for non-reversible Q.
//
// A = 64: the back-transform cancels strongly (|C| is a few hundred times
// the counts when V is far from orthogonal), so k_acc_cx writes C (FP32) to
// a buffer and k_bt_cx back-transforms it in FP64 with V, Vinv in shared
// memory.
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
  return (size_t)(2 * A * A + 2 * Gm::G * 2 * A + Gm::G * A * A + (Gm::G > 1 ? 2 * A * A : 0)) * sizeof(float2);
}

// Branches: P.cx_br[n_lo .. n_hi) (the branches of one system).  PB:
// per-branch counts (R, A, A, C) instead of their sum; CBUF: write the
// summed C to cbuf ([column][A*A] complex) instead of back-transforming it;
// P.cx_accum: add the summed counts to the output.
template <int A, bool PB, bool CBUF>
__global__ void __launch_bounds__(kCxThreads) k_acc_cx(const KParams P, const float *__restrict__ sa,
                                                       const float *__restrict__ sb, int c_base, int c_count,
                                                       int n_lo, int n_hi, float2 *__restrict__ cbuf) {
  using Gm = CxGeo<A>;
  constexpr int TPC = Gm::TPC, G = Gm::G;
  extern __shared__ __align__(16) float2 s_cx[];
  float2 *sV = s_cx;                  // A x A: V[i][k]
  float2 *sVi = sV + A * A;           // A x A: Vinv[k][j]
  // column-minor layouts (consecutive columns in consecutive words: no bank
  // conflicts when a warp spans several columns)
  float2 *sP = sVi + A * A;           // [2][2A][G]: D~ (k < A), U~ (A + l)
  float2 *sC = sP + 2 * G * 2 * A;    // [A*A][G]: C, then T = C Vinv
  float2 *sJ = sC + G * A * A;        // [2][16][TPC]: J_n, entry p*16+i at i*TPC+p
  const float2 *J = P.cx;
  const float2 *T0 = P.cx_tab;  // V, Vinv, R, Vinv^T, V^T
  const float2 *Vg = T0 + (P.cx_exact ? 3 : 0) * A * A;
  const float2 *Vig = Vg + A * A;
  const float2 *Rg = T0 + 2 * A * A;
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
  auto cC = [&](int e) -> float2 & { return sC[(size_t)e * G + g]; };

  // back-transform of the thread's 16 entries and the stores (row: branch
  // n for PB, else 0); every thread calls it (barriers inside)
  auto epilogue = [&](const float2 (&acc)[kCxE], int row, bool valid, size_t col) {
    __syncthreads();  // earlier readers of sC are done
    if (busy)
#pragma unroll
      for (int i = 0; i < kCxE; ++i) cC(p * kCxE + i) = acc[i];
    __syncthreads();
    float2 T[kCxE];
    if (busy)
#pragma unroll
      for (int i = 0; i < kCxE; ++i) {
        const int e = p * kCxE + i, k = e / A, j = e % A;
        float2 s = make_float2(0.f, 0.f);
#pragma unroll 4
        for (int l = 0; l < A; ++l) s = cfma(cC(k * A + l), sVi[l * A + j], s);
        T[i] = s;
      }
    __syncthreads();
    if (busy)
#pragma unroll
      for (int i = 0; i < kCxE; ++i) cC(p * kCxE + i) = T[i];
    __syncthreads();
    if (busy && valid) {
      float *out = P.counts + (size_t)row * A * A * C + col;
#pragma unroll
      for (int i = 0; i < kCxE; ++i) {
        const int e = p * kCxE + i, ii = e / A, j = e % A;
        float2 s = make_float2(0.f, 0.f);
#pragma unroll 4
        for (int k = 0; k < A; ++k) s = cfma(sV[ii * A + k], cC(k * A + j), s);
        const float v = (ii == j) ? s.x : cmul(__ldg(Rg + e), s).x;
        if (!PB && P.cx_accum) out[(size_t)e * C] += v;
        else out[(size_t)e * C] = v;
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
    // projections of branch slot bi into buffer bi & 1
    auto project = [&](int bi) {
      const int n = __ldg(P.cx_br + bi);
      if constexpr (G > 1) {
        // J_n into shared memory once per CTA (not once per column); the
        // stores run over the shared layout so that they do not conflict
        float2 *dj = sJ + (size_t)(bi & 1) * A * A;
        const float2 *Jn = J + (size_t)n * A * A;
        for (int d = t; d < A * A; d += blockDim.x) dj[d] = __ldg(Jn + (d % TPC) * kCxE + d / TPC);
      }
      if (!busy) return;
      float2 *buf = sP + (size_t)(bi & 1) * 2 * A * G + g;   // element o at buf[o * G]
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
        buf[(size_t)o * G] = s;
      }
    };
    // software pipeline: branch bi + 1 is projected (its staged rows loaded)
    // while branch bi accumulates; one barrier per branch
    if (n_lo < n_hi) project(n_lo);
    __syncthreads();
    for (int bi = n_lo; bi < n_hi; ++bi) {
      const int n = __ldg(P.cx_br + bi);
      if (bi + 1 < n_hi) project(bi + 1);
      if (busy) {
        const float2 *buf = sP + (size_t)(bi & 1) * 2 * A * G + g;
        // one column per CTA (A = 64): no reuse, J_n read through L1
        const float2 *Jn = (G > 1) ? sJ + (size_t)(bi & 1) * A * A + p : J + (size_t)n * A * A + p * kCxE;
        constexpr int js = (G > 1) ? TPC : 1;
#pragma unroll
        for (int i = 0; i < kCxE; ++i) {
          const int e = p * kCxE + i, k = e / A, l = e % A;
          const float2 x = cmul(buf[(size_t)k * G], (G > 1) ? Jn[i * js] : __ldg(Jn + i));
          const float2 u = buf[(size_t)(A + l) * G];
          acc[i] = PB ? cmul(x, u) : cfma(x, u, acc[i]);
        }
      }
      if constexpr (PB) {
        epilogue(acc, n, valid, col);
      }
      __syncthreads();
    }
    if constexpr (CBUF) {
      if (valid) {
        float2 *o = cbuf + (size_t)ccl * A * A + p * kCxE;
#pragma unroll
        for (int i = 0; i < kCxE; ++i) o[i] = acc[i];
      }
    } else if constexpr (!PB) {
      epilogue(acc, 0, valid, col);
    }
  }
}

// FP64 back-transform of buffered C (A = 64): per column, T = C Vinv and
// V T in FP64 with V, Vinv, T in shared memory (224 KB at A = 64); output
// row `row` of counts.
template <int A>
__global__ void __launch_bounds__(1024) k_bt_cx(const KParams P, const float2 *__restrict__ cbuf, int c_base,
                                                      int c_count, int row) {
  extern __shared__ __align__(16) double2 s_bt[];
  double2 *sV = s_bt;           // A x A
  double2 *sVi = sV + A * A;    // A x A
  double2 *sT = sVi + A * A;    // A x A
  float2 *sCc = reinterpret_cast<float2 *>(sT + A * A);  // A x A
  const double2 *D0 = reinterpret_cast<const double2 *>(P.cx_tab + (size_t)5 * A * A);  // V, Vinv, Vinv^T, V^T
  const double2 *Vg = D0 + (P.cx_exact ? 2 : 0) * A * A;
  const double2 *Vig = Vg + A * A;
  const float2 *Rg = P.cx_tab + (size_t)2 * A * A;
  const int t = threadIdx.x;
  for (int e = t; e < A * A; e += blockDim.x) {
    sV[e] = Vg[e];
    sVi[e] = Vig[e];
  }
  constexpr int EPT = A * A / kCxThreads > 0 ? A * A / kCxThreads : 1;  // entries per thread
  const int C = P.C;
  for (int cc = blockIdx.x; cc < c_count; cc += gridDim.x) {
    __syncthreads();  // tables loaded / previous column's reads done
    for (int e = t; e < A * A; e += blockDim.x) sCc[e] = cbuf[(size_t)cc * A * A + e];
    __syncthreads();
    for (int e = t; e < A * A; e += blockDim.x) {
      const int k = e / A, j = e % A;
      double2 s = make_double2(0.0, 0.0);
      for (int l = 0; l < A; ++l) {
        const float2 c = sCc[k * A + l];
        const double2 v = sVi[l * A + j];
        s.x = fma((double)c.x, v.x, fma(-(double)c.y, v.y, s.x));
        s.y = fma((double)c.x, v.y, fma((double)c.y, v.x, s.y));
      }
      sT[e] = s;
    }
    __syncthreads();
    float *out = P.counts + (size_t)row * A * A * C + (size_t)c_base + cc;
    for (int e = t; e < A * A; e += blockDim.x) {
      const int i = e / A, j = e % A;
      double2 s = make_double2(0.0, 0.0);
      for (int k = 0; k < A; ++k) {
        const double2 v = sV[i * A + k], x = sT[k * A + j];
        s.x = fma(v.x, x.x, fma(-v.y, x.y, s.x));
        s.y = fma(v.x, x.y, fma(v.y, x.x, s.y));
      }
      double r = s.x;
      if (i != j) {
        const float2 q = __ldg(Rg + e);
        r = (double)q.x * s.x - (double)q.y * s.y;
      }
      out[(size_t)e * C] = (float)r;
    }
    (void)EPT;
  }
}

template <int A, bool PB, bool CBUF>
int cx_launch(const KParams &p, const float *sa, const float *sb, int c_base, int c_count, int n_lo, int n_hi,
              float2 *cbuf, int grid, cudaStream_t s) {
  const size_t smem = cx_smem<A>();
  cudaError_t e =
      cudaFuncSetAttribute(k_acc_cx<A, PB, CBUF>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return (int)e;
  k_acc_cx<A, PB, CBUF><<<grid, kCxThreads, smem, s>>>(p, sa, sb, c_base, c_count, n_lo, n_hi, cbuf);
  return (int)cudaGetLastError();
}

template <int A>
int cx_launch_any(const KParams &p, bool pb, const float *sa, const float *sb, int c_base, int c_count, int n_lo,
                  int n_hi, float2 *cbuf, int grid, cudaStream_t s) {
  if (cbuf) return cx_launch<A, false, true>(p, sa, sb, c_base, c_count, n_lo, n_hi, cbuf, grid, s);
  return pb ? cx_launch<A, true, false>(p, sa, sb, c_base, c_count, n_lo, n_hi, cbuf, grid, s)
            : cx_launch<A, false, false>(p, sa, sb, c_base, c_count, n_lo, n_hi, cbuf, grid, s);
}

template <int A>
int bt_launch(const KParams &p, const float2 *cbuf, int c_base, int c_count, int row, int grid, cudaStream_t s) {
  const size_t smem = (size_t)3 * A * A * sizeof(double2) + (size_t)A * A * sizeof(float2);
  cudaError_t e = cudaFuncSetAttribute(k_bt_cx<A>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return (int)e;
  k_bt_cx<A><<<grid, 1024, smem, s>>>(p, cbuf, c_base, c_count, row);  // 32 warps: FP64 latency
  return (int)cudaGetLastError();
}

// Distance gradient (subby/jax/vjp.py:62-133) from the walk's raw staging:
// per (branch n, 128-column tile), with G_n = dM_n/dt in shared memory,
// v_c = g_c (D_n s_n)^T G_n U_n reduced over the tile in FP64 and added to
// grad_t[n] (one atomic per tile).
template <int A>
__global__ void __launch_bounds__(128) k_grad_cx(const KParams P, const float *__restrict__ sa,
                                                 const float *__restrict__ sb, const float *__restrict__ gq,
                                                 const float *__restrict__ g, int c_base, int c_count,
                                                 double *__restrict__ grad_t) {
  __shared__ __align__(16) float sG[A * A];
  __shared__ double s_red[4];
  const int t = threadIdx.x;
  const int ntiles = (c_count + 127) / 128;
  const long long items = (long long)(P.R - 1) * ntiles;
  for (long long it = blockIdx.x; it < items; it += gridDim.x) {
    const int n = 1 + (int)(it / ntiles);
    const int tile = (int)(it % ntiles);
    __syncthreads();
    for (int e = t; e < A * A; e += 128) sG[e] = __ldg(gq + (size_t)n * A * A + e);
    __syncthreads();
    const int cc = tile * 128 + t;
    double v = 0.0;
    if (cc < c_count) {
      const size_t row = ((size_t)(n - 1) * c_count + cc) * A;
      float u[A];
#pragma unroll
      for (int q = 0; q < A / 4; ++q) {
        const float4 x = __ldg(reinterpret_cast<const float4 *>(sb + row) + q);
        u[4 * q] = x.x, u[4 * q + 1] = x.y, u[4 * q + 2] = x.z, u[4 * q + 3] = x.w;
      }
      float acc = 0.f;
#pragma unroll 4
      for (int a = 0; a < A; ++a) {
        float y = 0.f;
#pragma unroll
        for (int b = 0; b < A; ++b) y = fmaf(sG[a * A + b], u[b], y);
        acc = fmaf(__ldg(sa + row + a), y, acc);
      }
      v = (double)acc * (g ? (double)__ldg(g + c_base + cc) : 1.0);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((t & 31) == 0) s_red[t >> 5] = v;
    __syncthreads();
    if (t == 0) atomicAdd(grad_t + n, (s_red[0] + s_red[1]) + (s_red[2] + s_red[3]));
  }
}

}  // namespace

int launch_grad_cx(const KParams &p, int A, const float *sa, const float *sb, const float *gq, const float *g,
                   int c_base, int c_count, double *grad_t, int grid, cudaStream_t s) {
  switch (A) {
    case 4: k_grad_cx<4><<<grid, 128, 0, s>>>(p, sa, sb, gq, g, c_base, c_count, grad_t); break;
    case 8: k_grad_cx<8><<<grid, 128, 0, s>>>(p, sa, sb, gq, g, c_base, c_count, grad_t); break;
    case 16: k_grad_cx<16><<<grid, 128, 0, s>>>(p, sa, sb, gq, g, c_base, c_count, grad_t); break;
    case 20: k_grad_cx<20><<<grid, 128, 0, s>>>(p, sa, sb, gq, g, c_base, c_count, grad_t); break;
    case 32: k_grad_cx<32><<<grid, 128, 0, s>>>(p, sa, sb, gq, g, c_base, c_count, grad_t); break;
    case 64: k_grad_cx<64><<<grid, 128, 0, s>>>(p, sa, sb, gq, g, c_base, c_count, grad_t); break;
    default: return -1;
  }
  return (int)cudaGetLastError();
}

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

bool cx_bt64(int A) { return A == 64; }

int launch_acc_cx(const KParams &p, int A, bool pb, const float *sa, const float *sb, int c_base, int c_count,
                  int n_lo, int n_hi, float2 *cbuf, int grid, cudaStream_t s) {
  switch (A) {
    case 4: return cx_launch_any<4>(p, pb, sa, sb, c_base, c_count, n_lo, n_hi, cbuf, grid, s);
    case 8: return cx_launch_any<8>(p, pb, sa, sb, c_base, c_count, n_lo, n_hi, cbuf, grid, s);
    case 16: return cx_launch_any<16>(p, pb, sa, sb, c_base, c_count, n_lo, n_hi, cbuf, grid, s);
    case 20: return cx_launch_any<20>(p, pb, sa, sb, c_base, c_count, n_lo, n_hi, cbuf, grid, s);
    case 32: return cx_launch_any<32>(p, pb, sa, sb, c_base, c_count, n_lo, n_hi, cbuf, grid, s);
    case 64: return cx_launch_any<64>(p, pb, sa, sb, c_base, c_count, n_lo, n_hi, cbuf, grid, s);
    default: return -1;
  }
}

int launch_bt_cx(const KParams &p, int A, const float2 *cbuf, int c_base, int c_count, int row, int grid,
                 cudaStream_t s) {
  if (A == 64) return bt_launch<64>(p, cbuf, c_base, c_count, row, grid, s);
  return -1;
}

}  // namespace subby
