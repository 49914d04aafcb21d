// F81 fast-path accumulation at A = 64 on the tensor cores.
//
// The F81 counts of one column (subby/oracle/oracle.py:1190-1256) are
//   I_ij = G_ij + h_i + pi_i (g_j + z),
//   G = sum_n alpha_n (s D_n) (x) U_n,  h = sum_n beta_n (pi . U_n) s D_n,
//   g = sum_n beta_n sum(s D_n) U_n,    z = sum_n gamma_n sum(s D_n) (pi . U_n),
// with dwell = I_ii and substitutions mu pi_j I_ij.  G is a product of two
// (A x (R-1)) matrices per column — a GEMM over the branches — so it runs as
// tcgen05.mma (kind::f16, BF16 operands split into three terms, six products,
// FP32 accumulation in TMEM): per CTA a group of 8 columns, two columns per
// M = N = 128 product (rows 0-63 column 2p, rows 64-127 column 2p+1; the
// cross blocks are not used), 16 branches per K step.  All terms of G are
// non-negative, so the split keeps FP32-level accuracy.  The staged s D and
// U (written by k_walk, F81 staging) are read from global memory by all
// threads, split and stored into the canonical K-major tiles of a double
// buffer while the tensor cores work on the other buffer; h, g, z are
// accumulated on the CUDA cores from the same loads and the per-branch
// scalars (pi . U, sum s D) that k_walk staged beside the vectors.
#include <cuda_bf16.h>

#include "common.cuh"

namespace subby {
namespace {

constexpr int kA = 64;         // alphabet
constexpr int kG = 8;          // columns per group
constexpr int kKC = 16;        // branches per K step
constexpr uint32_t kTileB = 4096;          // one BF16 term of a 128 x 16 tile
constexpr uint32_t kPairB = 6 * kTileB;    // A (3 terms) + B (3 terms)
constexpr uint32_t kBufB = 4 * kPairB;     // four column pairs
constexpr uint32_t kDynB = 2 * kBufB;      // double buffer (reused for the output staging)
constexpr int kWaitLimitT = 1 << 24;

constexpr uint32_t kIdesc128 = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(128 >> 3) << 17) |
                               ((uint32_t)(128 >> 4) << 24);

__device__ __forceinline__ bool mbar_wait_t(uint32_t mb, uint32_t phase) {
  for (int it = 0; it < kWaitLimitT; ++it) {
    uint32_t done;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
                 : "=r"(done)
                 : "r"(mb), "r"(phase)
                 : "memory");
    if (done) return true;
  }
  return false;
}
// canonical K-major tile with K = 16 and no swizzle: element (r, k) at byte
// (r&7)*16 + (r>>3)*256 + (k&7)*2 + (k>>3)*128 (core-matrix strides: 128 B
// along K, 256 B along M/N)
__device__ __forceinline__ uint32_t off16(int r, int k) {
  return (uint32_t)((r & 7) * 16 + (r >> 3) * 256 + (k & 7) * 2 + (k >> 3) * 128);
}
__device__ __forceinline__ uint64_t desc16(uint32_t saddr) {
  return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(256 >> 4) << 32) |
         ((uint64_t)1 << 46);
}

__global__ void __launch_bounds__(256, 1) k_acc_f81_tc(const KParams P, const float *__restrict__ sa,
                                                       const float *__restrict__ sb,
                                                       const float2 *__restrict__ sc, int c_base,
                                                       int c_count) {
  extern __shared__ __align__(1024) unsigned char dyn[];
  __shared__ __align__(8) uint64_t mbar[2];
  __shared__ uint32_t s_taddr;
  __shared__ int s_err;
  __shared__ float Hs[kG][kA], Gv[kG][kA], Zs[kG], pis[kA];
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const float *F8 = P.tab + P.off.F81;
  const int C = P.C, nbr = P.R - 1;
  const int NK = (nbr + kKC - 1) / kKC;
  const int ngroups = (c_count + kG - 1) / kG;
  if (warp == 0) {
    const uint32_t dst = (uint32_t)__cvta_generic_to_shared(&s_taddr);
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst), "r"(512)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (t == 0) {
    s_err = 0;
    for (int i = 0; i < 2; ++i) {
      const uint32_t mb = (uint32_t)__cvta_generic_to_shared(&mbar[i]);
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb) : "memory");
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncwarp();  // warp-aligned barriers below need warp 0 whole
  if (t < kA) pis[t] = __ldg(P.tab + P.off.pi + t);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = s_taddr;
  const uint32_t base = (uint32_t)__cvta_generic_to_shared(dyn);
  const uint32_t mbs[2] = {(uint32_t)__cvta_generic_to_shared(&mbar[0]),
                           (uint32_t)__cvta_generic_to_shared(&mbar[1])};
  uint32_t nph0 = 0, nph1 = 0;   // phases of each barrier waited so far
  auto wait_buf = [&](int b) {
    const uint32_t ph = b ? nph1 : nph0;
    if (!mbar_wait_t(mbs[b], ph & 1)) s_err = 1;
    if (b) ++nph1;
    else ++nph0;
    __syncwarp();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  };
  // this thread's tile row r (state ii of column 2p + ci) and K half kh
  const int r = t >> 1, kh = t & 1, ci = r >> 6, ii = r & 63;
  const float mu = P.f81_mu;

  for (int gi = blockIdx.x; gi < ngroups; gi += gridDim.x) {
    const int g0 = gi * kG;
    const int gcols = min(kG, c_count - g0);
    float hacc[4] = {0.f, 0.f, 0.f, 0.f}, gacc[4] = {0.f, 0.f, 0.f, 0.f}, zacc = 0.f;
    for (int kc = 0; kc < NK; ++kc) {
      const int b = kc & 1;
      if (t < kG * kKC) {
        // z: thread t takes column t / 16 and branch kc * 16 + t % 16
        const int c = t >> 4, nn = kc * kKC + (t & 15);
        if (c < gcols && nn < nbr) {
          const float2 q = __ldg(sc + ((size_t)nn * c_count + g0 + c));
          zacc = fmaf(__ldg(F8 + 4 * (nn + 1) + 2) * q.y, q.x, zacc);
        }
      }
      if (kc >= 2) wait_buf(b);   // the MMAs of chunk kc - 2 have read this buffer
      const uint32_t buf = base + (uint32_t)b * kBufB;
      const int n0 = kc * kKC + 8 * kh;
      float4 abg[8];
#pragma unroll
      for (int k = 0; k < 8; ++k)
        abg[k] = (n0 + k < nbr) ? __ldg(reinterpret_cast<const float4 *>(F8) + n0 + k + 1)
                                : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
      for (int p = 0; p < 4; ++p) {
        const int c = 2 * p + ci;
        const bool cin = c < gcols;
        float va[8], vb[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
          const int n = n0 + k;
          const bool in = cin && n < nbr;
          const size_t row = ((size_t)n * c_count + g0 + c);
          const float d = in ? __ldg(sa + row * kA + ii) : 0.f;
          const float u = in ? __ldg(sb + row * kA + ii) : 0.f;
          const float2 pd = in ? __ldg(sc + row) : make_float2(0.f, 0.f);  // (pi . U, sum s D)
          va[k] = abg[k].x * d;
          vb[k] = u;
          hacc[p] = fmaf(abg[k].y * pd.x, d, hacc[p]);
          gacc[p] = fmaf(abg[k].y * pd.y, u, gacc[p]);
        }
        // three BF16 terms of the 8 values -> one 16-byte row per term
        uint32_t ta[3][4], tb[3][4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
#pragma unroll
          for (int w2 = 0; w2 < 2; ++w2) {
            const float x0 = w2 ? vb[2 * q] : va[2 * q], x1 = w2 ? vb[2 * q + 1] : va[2 * q + 1];
            const __nv_bfloat162 b1 = __floats2bfloat162_rn(x0, x1);
            const float2 f1 = __bfloat1622float2(b1);
            const float r0 = x0 - f1.x, r1 = x1 - f1.y;
            const __nv_bfloat162 b2 = __floats2bfloat162_rn(r0, r1);
            const float2 f2 = __bfloat1622float2(b2);
            const __nv_bfloat162 b3 = __floats2bfloat162_rn(r0 - f2.x, r1 - f2.y);
            uint32_t(*dst)[4] = w2 ? tb : ta;
            dst[0][q] = *reinterpret_cast<const uint32_t *>(&b1);
            dst[1][q] = *reinterpret_cast<const uint32_t *>(&b2);
            dst[2][q] = *reinterpret_cast<const uint32_t *>(&b3);
          }
        }
        const uint32_t o = off16(r, 8 * kh);
#pragma unroll
        for (int term = 0; term < 3; ++term) {
          const uint32_t pa = buf + (uint32_t)p * kPairB + (uint32_t)term * kTileB + o;
          const uint32_t pb = pa + 3 * kTileB;
          asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(pa), "r"(ta[term][0]), "r"(ta[term][1]),
                       "r"(ta[term][2]), "r"(ta[term][3]) : "memory");
          asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(pb), "r"(tb[term][0]), "r"(tb[term][1]),
                       "r"(tb[term][2]), "r"(tb[term][3]) : "memory");
        }
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncthreads();
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      if (t == 0) {
        constexpr int pa6[6] = {0, 0, 1, 0, 1, 2}, pb6[6] = {0, 1, 0, 2, 1, 0};
#pragma unroll
        for (int p = 0; p < 4; ++p) {
#pragma unroll
          for (int prod = 0; prod < 6; ++prod) {
            const uint32_t a = buf + (uint32_t)p * kPairB + (uint32_t)pa6[prod] * kTileB;
            const uint32_t bb = buf + (uint32_t)p * kPairB + 3 * kTileB + (uint32_t)pb6[prod] * kTileB;
            const uint32_t accum = (kc | prod) != 0;
            asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                         " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}"
                         ::"r"(tmem + 128u * p), "l"(desc16(a)), "l"(desc16(bb)), "r"(kIdesc128), "r"(accum)
                         : "memory");
          }
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbs[b])
                     : "memory");
      }
      __syncwarp();
    }
    // the last two chunks' products
    if (NK >= 2) wait_buf((NK - 2) & 1);
    wait_buf((NK - 1) & 1);
    // ------------------------------------------------------------ epilogue
    // h, g: combine the two K halves; z: one thread per column
#pragma unroll
    for (int p = 0; p < 4; ++p) {
      const float hf = hacc[p] + __shfl_xor_sync(0xffffffffu, hacc[p], 1);
      const float gf = gacc[p] + __shfl_xor_sync(0xffffffffu, gacc[p], 1);
      if (kh == 0) {
        Hs[2 * p + ci][ii] = hf;
        Gv[2 * p + ci][ii] = gf;
      }
    }
    // z: sum the 16 partials of each column (lanes 16 apart hold other columns)
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) zacc += __shfl_xor_sync(0xffffffffu, zacc, o);
    if (t < kG * kKC && (t & 15) == 0) Zs[t >> 4] = zacc;
    // G out of TMEM into the shared staging [c][i][j] (the operand buffers are idle)
    float *Gs = reinterpret_cast<float *>(dyn);
    {
      const int sub = warp & 3, row = 32 * sub + lane;
      const int cg = row >> 6, i = row & 63, j0 = 32 * (warp >> 2);
#pragma unroll
      for (int p = 0; p < 4; ++p) {
        uint32_t v[32];
        const uint32_t ta = tmem + ((uint32_t)(32 * sub) << 16) + 128u * p + 64u * cg + (uint32_t)j0;
        asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,"
                     "%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
                 "tcgen05.wait::ld.sync.aligned;"
                     : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
                       "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
                       "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]),
                       "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]),
                       "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
                     : "r"(ta)
                     : "memory");
        float *dst = Gs + ((size_t)(2 * p + cg) * kA + i) * kA + j0;
#pragma unroll
        for (int q = 0; q < 8; ++q)
          *reinterpret_cast<float4 *>(dst + 4 * q) =
              make_float4(__uint_as_float(v[4 * q]), __uint_as_float(v[4 * q + 1]), __uint_as_float(v[4 * q + 2]),
                          __uint_as_float(v[4 * q + 3]));
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    // I = G + h_i + pi_i (g_j + z); dwell I_ii, substitutions mu pi_j I_ij;
    // thread t: the 4 x 4 block (k0, l0) of (i, j) for all 8 columns
    {
      const int k0 = 4 * (t >> 4), l0 = 4 * (t & 15);
      const int col0 = c_base + g0;
      const bool vec = (C & 3) == 0 && (col0 & 3) == 0 && gcols == kG;
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          const int i = k0 + a, j = l0 + b;
          const float f = (i == j) ? 1.f : mu * pis[j];
          float v[kG];
#pragma unroll
          for (int q = 0; q < kG; ++q)
            v[q] = f * (Gs[((size_t)q * kA + i) * kA + j] + Hs[q][i] + pis[i] * (Gv[q][j] + Zs[q]));
          float *o = P.counts + (size_t)(i * kA + j) * C + col0;
          if (vec) {
            *reinterpret_cast<float4 *>(o) = make_float4(v[0], v[1], v[2], v[3]);
            *reinterpret_cast<float4 *>(o + 4) = make_float4(v[4], v[5], v[6], v[7]);
          } else {
#pragma unroll
            for (int q = 0; q < kG; ++q)
              if (q < gcols) o[q] = v[q];
          }
        }
    }
    __syncthreads();
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512) : "memory");
  if (t == 0 && s_err && P.err) atomicAdd(P.err, 1);
}

}  // namespace

int launch_acc_f81_tc(const KParams &p, const float *sa, const float *sb, const float2 *sc, int c_base,
                      int c_count, int grid, cudaStream_t s) {
  cudaError_t e = cudaFuncSetAttribute(k_acc_f81_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kDynB);
  if (e != cudaSuccess) return (int)e;
  k_acc_f81_tc<<<grid, 256, kDynB, s>>>(p, sa, sb, sc, c_base, c_count);
  return (int)cudaGetLastError();
}

}  // namespace subby
