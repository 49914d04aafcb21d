// Large-alphabet path (A = 16, 20, 32, 64): tree walk + staged accumulation.
//
// Kernel 1, k_walk<A> (walk.cuh): the tree program of k_tree.cu (stored / derived
// nodes; subby/oracle/oracle.py:784-924) for a tile of 128 columns per CTA.
// Thread (c, h) owns column c of the tile and states [32h, 32h + S) of every
// vector (S = min(A, 32); h < H = ceil(A / 32)), so a length-A vector lives
// in S registers of each of H threads.  Matrix-vector products
// y_b = sum_j T[j][b] x_j read T rows with warp-uniform broadcast loads and
// keep x in registers; with H = 2 each thread forms partial sums over its own
// inputs for all A outputs and the pair exchanges halves through shared
// memory.  Stored-node slots live in a per-tile region of global memory.
//   * LogLike / RootProb come out of the inside pass.
//   * For Counts the outside pass stages, per branch n and column c, the two
//     vectors the accumulation needs: eigen path D~ = s Vd^T D and
//     U~ = Vu^T U (subby/oracle/oracle.py:966-1003; s = the branch weight
//     exp(lnD + lnU - lnL) = 2^(eD+eU-eRoot)/P, zero for masked branches),
//     F81 path s D and U (oracle.py:1190-1256).
// Kernel 2, k_acc<A, F81>: per group of G columns, accumulates
// C_kl += D~_k J_kl U~_l over all branches (oracle.py:1010-1044) — or the
// F81 rank-3 terms — with 4 x 4 (k, l) register blocks, J rows and staged
// vectors double-buffered through shared memory, then back-transforms
// V C V^T (oracle.py:1087-1137) through shared memory and writes counts.
#include <cuda_bf16.h>

#include "common.cuh"
#include "walk.cuh"

namespace subby {
namespace {

// ---------------------------------------------------------------------------
// Kernel 2: accumulation over branches + back-transform, G columns per CTA.
// Thread t: 4 x 4 block b = t % NB of (k, l), column group t / NB of 8 columns.
template <int A>
struct AccGeo {
  static constexpr int KB = A / 4;          // blocks per side
  static constexpr int NB = KB * KB;        // (k, l) blocks
  static constexpr int GROUPS = 256 / NB;   // column groups of 8
  static constexpr int G = GROUPS * 8;      // columns per CTA
  static constexpr int THREADS = NB * GROUPS;
};

// Stages of the k_acc ring: as many (J_n, a, b) buffers as fit in the
// G x A x A floats of the back-transform buffer, at most 8.
template <int A>
struct AccRing {
  static constexpr int STAGE = A * A + 2 * AccGeo<A>::G * A;       // floats per stage
  static constexpr int CBUF = AccGeo<A>::G * A * A;                // back-transform buffer
  static constexpr int S = (CBUF / STAGE) < 8 ? (CBUF / STAGE) : 8;
  static constexpr int SCAL = (S * STAGE > CBUF ? S * STAGE : CBUF);  // F81 scalars after both
  static_assert(S >= 3, "ring too short");
};

// Shared-memory float offset of the static [V ; V] operand tile of the
// tensor-core back-transform (A = 64), 1 KB aligned.
template <int A>
__host__ __device__ constexpr int acc_vv_offset() {
  return ((AccRing<A>::SCAL + 2 * AccGeo<A>::G + 2 * A * A + A + 2 * AccGeo<A>::G * A + AccGeo<A>::G) + 255) / 256 *
         256;
}

// TCB: back-transform V C V^T on the tensor cores (A = 64 eigen path of the
// tensor-core Counts); otherwise on CUDA cores.
// PB: per-branch counts — each work item is one (branch, column group) and
// writes that branch's counts (R, A, A, C layout) instead of summing.
template <int A, bool F81, bool TCB, bool PB = false>
__global__ void __launch_bounds__(256, 1) k_acc(const KParams P, const float *__restrict__ stage_a,
                                                 const float *__restrict__ stage_b, int c_base, int c_count) {
  using Gm = AccGeo<A>;
  using Rg = AccRing<A>;
  static_assert(!(PB && TCB), "per-branch counts use the CUDA-core back-transform");
  static_assert(!TCB || (A == 64 && !F81), "tensor-core back-transform is A = 64 eigen");
  constexpr int G = Gm::G;
  constexpr int S = Rg::S;
  extern __shared__ __align__(128) float sm[];
  // ring of S stages, each J_n (A*A, eigen path) + a (G*A) + b (G*A), filled
  // by bulk copies that complete on one mbarrier per stage; the space is
  // reused for C / T by the back-transform.
  __shared__ __align__(8) uint64_t mbar[S];
  __shared__ int s_err;
  const int t = threadIdx.x;
  const bool active = t < Gm::THREADS;
  const int blk = t % Gm::NB, grp = t / Gm::NB;
  const int k0 = 4 * (blk / Gm::KB), l0 = 4 * (blk % Gm::KB);
  const float *J = P.tab + P.off.J;
  const float *F8 = P.tab + P.off.F81;
  const float *pig = P.tab + P.off.pi;
  const int C = P.C;
  const int nbr = P.R - 1;
  const int ngroups = (c_count + G - 1) / G;
  const int nitems = PB ? ngroups * nbr : ngroups;
  float *cbase = P.counts;   // PB: the current branch's slab
  // V, S (eigen path) and pi, copied once per CTA behind the F81 scalars
  float *Vs = sm + Rg::SCAL + 2 * G, *Ss = Vs + A * A, *pis = Ss + A * A;
  if (!F81)
    for (int i = t; i < A * A; i += blockDim.x) {
      Vs[i] = __ldg(P.tab + P.off.V + i);
      Ss[i] = __ldg(P.tab + P.off.S + i);
    }
  for (int i = t; i < A; i += blockDim.x) pis[i] = __ldg(pig + i);
  // output row r, the 8 columns col0.. of this thread's group: two 16-byte
  // stores when the rows are 16-byte aligned and all 8 columns exist
  const bool vec_out = (C & 3) == 0 && (c_base & 3) == 0;
  auto store8 = [&](size_t r, const float (&v)[8], int col0, int ncols) {
    float *o = cbase + r * C + col0;
    if (vec_out && ncols >= 8) {
      *reinterpret_cast<float4 *>(o) = make_float4(v[0], v[1], v[2], v[3]);
      *reinterpret_cast<float4 *>(o + 4) = make_float4(v[4], v[5], v[6], v[7]);
    } else {
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (q < ncols) o[q] = v[q];
    }
  };
  if (t == 0) {
    s_err = 0;
    for (int i = 0; i < S; ++i) {
      const uint32_t mb = (uint32_t)__cvta_generic_to_shared(&mbar[i]);
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb) : "memory");
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncwarp();  // warp-aligned barriers below need warp 0 whole
  // tensor-core back-transform: TMEM (the four pairs' V C V^T in columns
  // 0-255, T = C V^T in 256-383), one mbarrier per product kind, and the
  // static A operand [V ; V] (three BF16 terms)
  __shared__ uint32_t s_tm;
  __shared__ __align__(8) uint64_t mbT[2];   // D1 products, D2 products
  if constexpr (TCB) {
    if ((t >> 5) == 0) {
      asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                   ::"r"((uint32_t)__cvta_generic_to_shared(&s_tm)), "r"(512) : "memory");
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (t == 0) {
      for (int i = 0; i < 2; ++i)
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"((uint32_t)__cvta_generic_to_shared(&mbT[i]))
                     : "memory");
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();
    __syncthreads();   // Vs is loaded
    unsigned char *vv = reinterpret_cast<unsigned char *>(sm + acc_vv_offset<A>());
    for (int idx = t; idx < 128 * 64; idx += blockDim.x) {
      const int m = idx >> 6, l = idx & 63;
      const float v = Vs[(m & 63) * 64 + l];
      const __nv_bfloat16 b1 = __float2bfloat16_rn(v);
      const float r1 = v - __bfloat162float(b1);
      const __nv_bfloat16 b2 = __float2bfloat16_rn(r1);
      const __nv_bfloat16 b3 = __float2bfloat16_rn(r1 - __bfloat162float(b2));
      const uint32_t o = kmaj_off(m, l);
      *reinterpret_cast<__nv_bfloat16 *>(vv + o) = b1;
      *reinterpret_cast<__nv_bfloat16 *>(vv + 16384 + o) = b2;
      *reinterpret_cast<__nv_bfloat16 *>(vv + 32768 + o) = b3;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  }
  __syncthreads();
  if constexpr (TCB) asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  uint32_t nT[2] = {0, 0};  // completed phases of mbT[0] (D1) and mbT[1] (D2)
  uint32_t it = 0;  // ring position of the next branch to consume (all groups)

  for (int wi = blockIdx.x; wi < nitems; wi += gridDim.x) {
    const int gi = PB ? wi % ngroups : wi;
    const int n_lo = PB ? wi / ngroups : 0, n_hi = PB ? n_lo + 1 : nbr;   // branches of this item
    if constexpr (PB) cbase = P.counts + (size_t)(n_lo + 1) * A * A * C;
    const int g0 = gi * G;                       // first column (chunk-relative)
    const int gcols = min(G, c_count - g0);
    // accumulators: ac2[a][p][q] = (C[k0+a][l0+2p], C[k0+a][l0+2p+1]) of column q
    float2 ac2[4][2][8];
#define ACC(a, b, q) (((b) & 1) ? ac2[a][(b) >> 1][q].y : ac2[a][(b) >> 1][q].x)
    // F81: per-column h (rows), g (columns) and z, one element set per thread
    constexpr int NE = (G * A + 255) / 256;
    float hreg[NE], greg[NE], zreg = 0.f;
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int pp = 0; pp < 2; ++pp)
#pragma unroll
        for (int q = 0; q < 8; ++q) ac2[a][pp][q] = make_float2(0.f, 0.f);
    if (F81) {
#pragma unroll
      for (int r = 0; r < NE; ++r) hreg[r] = greg[r] = 0.f;
    }
    // a short last group: zero the unused column rows of every stage once
    // (the copies below fill only gcols rows)
    if (gcols < G) {
      for (int i = t; i < S * 2 * (G - gcols) * A; i += blockDim.x) {
        const int st = i / (2 * (G - gcols) * A), r = i % (2 * (G - gcols) * A);
        const int half = r / ((G - gcols) * A), e = r % ((G - gcols) * A);
        sm[st * Rg::STAGE + (F81 ? 0 : A * A) + half * G * A + gcols * A + e] = 0.f;
      }
      __syncthreads();
    }
    // J_n (eigen path) and the staged vectors of branch n for this group's
    // columns: three bulk copies issued by one thread, completing on the
    // stage's mbarrier
    const uint32_t vbytes = (uint32_t)gcols * A * 4;
    auto load = [&](int n, uint32_t pos) {
      const int st = (int)(pos % S);
      float *dst = sm + st * Rg::STAGE;
      const uint32_t mb = (uint32_t)__cvta_generic_to_shared(&mbar[st]);
      const uint32_t jb = F81 ? 0u : (uint32_t)(A * A * 4);
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mb), "r"(jb + 2 * vbytes)
                   : "memory");
      if (!F81)
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                     ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(J + (size_t)(n + 1) * A * A), "r"(jb),
                     "r"(mb) : "memory");
      const size_t off = ((size_t)n * c_count + g0) * A;
      float *da = dst + (F81 ? 0 : A * A), *db = da + G * A;
      asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                   ::"r"((uint32_t)__cvta_generic_to_shared(da)), "l"(stage_a + off), "r"(vbytes), "r"(mb)
                   : "memory");
      asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                   ::"r"((uint32_t)__cvta_generic_to_shared(db)), "l"(stage_b + off), "r"(vbytes), "r"(mb)
                   : "memory");
    };
    if (t == 0)
      for (int n = n_lo; n < n_lo + S - 1 && n < n_hi; ++n) load(n, it + (n - n_lo));
    __syncwarp();
    float *scal = sm + Rg::SCAL;  // F81: piU, Dsum per column
    for (int n = n_lo; n < n_hi; ++n, ++it) {
      // every thread is done with the stage of branch n - 1: refill it
      __syncthreads();
      if (t == 0 && n + S - 1 < n_hi) load(n + S - 1, it + S - 1);
      __syncwarp();
      const int st = (int)(it % S);
      const float *cur = sm + st * Rg::STAGE;
      if (!mbar_wait((uint32_t)__cvta_generic_to_shared(&mbar[st]), (it / S) & 1)) s_err = 1;
      if (F81) {
        // pi . U and sum(s D) per column: one warp per column, shuffle sums
        const int warp = t >> 5, lane = t & 31;
        for (int c = warp; c < G; c += 8) {
          const float *Ds = cur + c * A, *U = cur + G * A + c * A;
          float piU = 0.f, dsum = 0.f;
          for (int a = lane; a < A; a += 32) {
            piU = fmaf(pis[a], U[a], piU);
            dsum += Ds[a];
          }
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) {
            piU += __shfl_xor_sync(0xffffffffu, piU, o);
            dsum += __shfl_xor_sync(0xffffffffu, dsum, o);
          }
          if (lane == 0) {
            scal[2 * c] = piU;
            scal[2 * c + 1] = dsum;
          }
        }
        __syncthreads();
        // h_i += beta piU (s D)_i, g_j += beta sum(s D) U_j, z += gamma sum(s D) piU
        const float4 abg = __ldg(reinterpret_cast<const float4 *>(F8) + n + 1);
#pragma unroll
        for (int r = 0; r < NE; ++r) {
          const int e = t + 256 * r;
          if (NE * 256 == G * A || e < G * A) {
            const int c = e / A;
            hreg[r] = fmaf(abg.y * scal[2 * c], cur[e], hreg[r]);
            greg[r] = fmaf(abg.y * scal[2 * c + 1], cur[G * A + e], greg[r]);
          }
        }
        if (t < G) zreg = fmaf(abg.z * scal[2 * t + 1], scal[2 * t], zreg);
      }
      if (active) {
        const float *da = cur + (F81 ? 0 : A * A), *db = da + G * A;
        if (!F81) {
          // packed FP32x2: (d_k J_kl) for two l at once, then fma with (u_l, u_l+1)
          float2 jp[4][2];
#pragma unroll
          for (int a = 0; a < 4; ++a) {
            const float4 r = *reinterpret_cast<const float4 *>(cur + (k0 + a) * A + l0);
            jp[a][0] = make_float2(r.x, r.y);
            jp[a][1] = make_float2(r.z, r.w);
          }
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            const int cc = grp * 8 + q;
            const float4 d = *reinterpret_cast<const float4 *>(da + cc * A + k0);
            const float4 u = *reinterpret_cast<const float4 *>(db + cc * A + l0);
            const float dk[4] = {d.x, d.y, d.z, d.w};
            const float2 up[2] = {make_float2(u.x, u.y), make_float2(u.z, u.w)};
#pragma unroll
            for (int a = 0; a < 4; ++a) {
              const float2 dd = make_float2(dk[a], dk[a]);
#pragma unroll
              for (int pp = 0; pp < 2; ++pp)
                ac2[a][pp][q] = __ffma2_rn(__fmul2_rn(dd, jp[a][pp]), up[pp], ac2[a][pp][q]);
            }
          }
        } else {
          const float4 abg = __ldg(reinterpret_cast<const float4 *>(F8) + n + 1);
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            const int cc = grp * 8 + q;
            const float4 d = *reinterpret_cast<const float4 *>(da + cc * A + k0);
            const float4 u = *reinterpret_cast<const float4 *>(db + cc * A + l0);
            const float dk[4] = {d.x, d.y, d.z, d.w};
            const float2 up[2] = {make_float2(u.x, u.y), make_float2(u.z, u.w)};
#pragma unroll
            for (int a = 0; a < 4; ++a) {
              const float ad = abg.x * dk[a];
              const float2 dd = make_float2(ad, ad);
#pragma unroll
              for (int pp = 0; pp < 2; ++pp) ac2[a][pp][q] = __ffma2_rn(dd, up[pp], ac2[a][pp][q]);
            }
          }
        }
      }
    }
    __syncthreads();
    // ------------------------------------------------------------- epilogue
    const int col0 = c_base + g0 + grp * 8, ncols = gcols - grp * 8;
    if (F81) {
      // h, g, z of every column through shared memory to the (k, l) blocks
      float *Hs = pis + A, *Gs = Hs + G * A, *Zs = Gs + G * A;
#pragma unroll
      for (int r = 0; r < NE; ++r) {
        const int e = t + 256 * r;
        if (NE * 256 == G * A || e < G * A) {
          Hs[e] = hreg[r];
          Gs[e] = greg[r];
        }
      }
      if (t < G) Zs[t] = zreg;
      __syncthreads();
      if (active && ncols > 0) {
        const float mu = P.f81_mu;
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int b = 0; b < 4; ++b) {
            const int i = k0 + a, j = l0 + b;
            const float pi_i = pis[i], f = (i == j) ? 1.f : mu * pis[j];
            float v[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) {
              const int cc = grp * 8 + q;
              v[q] = f * (ACC(a, b, q) + Hs[cc * A + i] + pi_i * (Gs[cc * A + j] + Zs[cc]));
            }
            store8((size_t)(i * A + j), v, col0, ncols);
          }
      }
      __syncthreads();
      continue;
    }
    if constexpr (TCB) {
      // Per column pair (p, p+4): B1 = [C_p ; C_p+4] (rows (c, k), K = l);
      // D1 = [V ; V] B1^T holds T_c^T (lane (c, j), column k) in its
      // diagonal blocks; A2 = those rows (K = k); D2 = A2 V^T holds
      // (V C V^T)_c[i][j] at lane (c, j), column i.  D1 sits in tensor-memory
      // columns 256-383; each pair's D2 stays in columns 64p.. until all four
      // are formed, so a pair's D2 product runs while the next pair's B1 is
      // built and its D1 issued, and the eight columns go out together:
      // lane (c, j) holds columns 4c .. 4c+3 of the group, one 16-byte store.
      const uint32_t base = (uint32_t)__cvta_generic_to_shared(sm);
      const uint32_t B1 = base, A2 = base + 49152;
      const uint32_t VV = base + 4u * acc_vv_offset<A>();
      const uint32_t tm = s_tm, tmD1 = s_tm + 256u;
      const int warp = t >> 5, lane = t & 31, sub = warp & 3, hh = warp >> 2;
      const int m = 32 * sub + lane, cg = m >> 6, jj = m & 63;
      // each kind of product commits to its own mbarrier, so a wait never
      // has two phases of one barrier outstanding (a parity wait cannot tell
      // them apart)
      auto mma6 = [&](uint32_t d, uint32_t a, uint32_t b, uint32_t idesc, int kind) {
        constexpr int pa[6] = {0, 0, 1, 0, 1, 2}, pb[6] = {0, 1, 0, 2, 1, 0};
#pragma unroll
        for (int ks = 0; ks < 4; ++ks)
#pragma unroll
          for (int prod = 0; prod < 6; ++prod) {
            const uint32_t accum = (ks | prod) != 0;
            asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                         " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}"
                         ::"r"(d), "l"(umma_desc(a + pa[prod] * 16384 + ks * 256)),
                         "l"(umma_desc(b + pb[prod] * 16384 + ks * 256)), "r"(idesc), "r"(accum) : "memory");
          }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                     ::"r"((uint32_t)__cvta_generic_to_shared(&mbT[kind])) : "memory");
      };
      auto sync_tc = [&]() {
        __syncwarp();
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      };
      auto wait_t = [&](int kind) {
        if (!mbar_wait((uint32_t)__cvta_generic_to_shared(&mbT[kind]), nT[kind] & 1)) s_err = 1;
        ++nT[kind];
        __syncwarp();
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      };
      auto ld32 = [&](uint32_t col, uint32_t (&r)[32]) {
        asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,"
                     "%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
                     "tcgen05.wait::ld.sync.aligned;"
                     : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                       "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
                       "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]),
                       "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]),
                       "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                     : "r"(col + ((uint32_t)(32 * sub) << 16))
                     : "memory");
      };
      auto split3 = [](float x0, float x1, uint32_t &t1, uint32_t &t2, uint32_t &t3) {
        const __nv_bfloat162 b1 = __floats2bfloat162_rn(x0, x1);
        const float2 f1 = __bfloat1622float2(b1);
        const float r0 = x0 - f1.x, r1 = x1 - f1.y;
        const __nv_bfloat162 b2 = __floats2bfloat162_rn(r0, r1);
        const float2 f2 = __bfloat1622float2(b2);
        const __nv_bfloat162 b3 = __floats2bfloat162_rn(r0 - f2.x, r1 - f2.y);
        t1 = *reinterpret_cast<const uint32_t *>(&b1);
        t2 = *reinterpret_cast<const uint32_t *>(&b2);
        t3 = *reinterpret_cast<const uint32_t *>(&b3);
      };
#pragma unroll
      for (int p = 0; p < 4; ++p) {
        // (a) B1 rows of this thread's 4 x 4 block for columns p and p + 4
        // (B1 is free: the previous pair's D1 has completed)
#pragma unroll
        for (int h2 = 0; h2 < 2; ++h2) {
          const int q = p + 4 * h2;
#pragma unroll
          for (int a = 0; a < 4; ++a) {
            uint32_t u1[2], u2[2], u3[2];
            split3(ac2[a][0][q].x, ac2[a][0][q].y, u1[0], u2[0], u3[0]);
            split3(ac2[a][1][q].x, ac2[a][1][q].y, u1[1], u2[1], u3[1]);
            const uint32_t o = B1 + kmaj_off(64 * h2 + k0 + a, l0);
            asm volatile("st.shared.v2.b32 [%0], {%1, %2};" ::"r"(o), "r"(u1[0]), "r"(u1[1]) : "memory");
            asm volatile("st.shared.v2.b32 [%0], {%1, %2};" ::"r"(o + 16384), "r"(u2[0]), "r"(u2[1]) : "memory");
            asm volatile("st.shared.v2.b32 [%0], {%1, %2};" ::"r"(o + 32768), "r"(u3[0]), "r"(u3[1]) : "memory");
          }
        }
        sync_tc();
        if (t == 0) mma6(tmD1, VV, B1, kIdesc128, 0);
        __syncwarp();
        if (p > 0) wait_t(1);   // the previous pair's D2
        wait_t(0);              // this pair's D1
        // (e) T_c^T rows (lane (cg, jj), k in [32 hh, 32 hh + 32)) into A2
        // (A2 is free: the previous pair's D2 has completed)
        {
          uint32_t r[32];
          ld32(tmD1 + 64u * cg + 32u * hh, r);
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            uint32_t w1[4], w2[4], w3[4];
#pragma unroll
            for (int pp = 0; pp < 4; ++pp)
              split3(__uint_as_float(r[8 * q + 2 * pp]), __uint_as_float(r[8 * q + 2 * pp + 1]), w1[pp], w2[pp], w3[pp]);
            const uint32_t o = A2 + kmaj_off(m, 32 * hh + 8 * q);
            asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(o), "r"(w1[0]), "r"(w1[1]), "r"(w1[2]),
                         "r"(w1[3]) : "memory");
            asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(o + 16384), "r"(w2[0]), "r"(w2[1]),
                         "r"(w2[2]), "r"(w2[3]) : "memory");
            asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(o + 32768), "r"(w3[0]), "r"(w3[1]),
                         "r"(w3[2]), "r"(w3[3]) : "memory");
          }
        }
        sync_tc();   // D1's tensor-memory loads are done before the next pair's D1 overwrites it
        if (t == 0) mma6(tm + 64u * p, A2, VV, kIdesc, 1);
        __syncwarp();
      }
      wait_t(1);   // the last pair's D2
      // (k) counts rows (i, j = jj) of columns 4 cg .. 4 cg + 3, i in [32 hh, 32 hh + 32)
      {
        const int col0 = c_base + g0 + 4 * cg;
        const int ncol = min(4, gcols - 4 * cg);
        const bool vec4 = (C & 3) == 0 && (col0 & 3) == 0 && ncol == 4;
        if (ncol > 0) {
#pragma unroll 1
          for (int h16 = 0; h16 < 2; ++h16) {
            const int i0 = 32 * hh + 16 * h16;
            uint32_t v[4][16];
#pragma unroll
            for (int p = 0; p < 4; ++p)
              asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
                           "%14,%15}, [%16];\n"
                           "tcgen05.wait::ld.sync.aligned;"
                           : "=r"(v[p][0]), "=r"(v[p][1]), "=r"(v[p][2]), "=r"(v[p][3]), "=r"(v[p][4]),
                             "=r"(v[p][5]), "=r"(v[p][6]), "=r"(v[p][7]), "=r"(v[p][8]), "=r"(v[p][9]),
                             "=r"(v[p][10]), "=r"(v[p][11]), "=r"(v[p][12]), "=r"(v[p][13]), "=r"(v[p][14]),
                             "=r"(v[p][15])
                           : "r"(tm + ((uint32_t)(32 * sub) << 16) + 64u * p + (uint32_t)i0)
                           : "memory");
#pragma unroll
            for (int i2 = 0; i2 < 16; ++i2) {
              const int i = i0 + i2;
              const float f = (i == jj) ? 1.f : Ss[i * A + jj];
              const float4 o4 = make_float4(f * __uint_as_float(v[0][i2]), f * __uint_as_float(v[1][i2]),
                                            f * __uint_as_float(v[2][i2]), f * __uint_as_float(v[3][i2]));
              float *o = P.counts + (size_t)(i * A + jj) * C + col0;
              if (vec4) {
                *reinterpret_cast<float4 *>(o) = o4;
              } else {
                o[0] = o4.x;
                if (ncol > 1) o[1] = o4.y;
                if (ncol > 2) o[2] = o4.z;
                if (ncol > 3) o[3] = o4.w;
              }
            }
          }
        }
      }
      // every tensor-memory read done before the next group's products
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncthreads();
      continue;
    }
    // back-transform: C -> T = C V^T -> VCV = V T, through shared memory [c][k][l]
    float *Cs = sm;  // G * A * A floats
    const float *V = Vs;
    if (active) {
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int cc = grp * 8 + q;
#pragma unroll
        for (int a = 0; a < 4; ++a)
          *reinterpret_cast<float4 *>(Cs + ((size_t)cc * A + k0 + a) * A + l0) =
              make_float4(ac2[a][0][q].x, ac2[a][0][q].y, ac2[a][1][q].x, ac2[a][1][q].y);
      }
    }
    __syncthreads();
    // T[c][k][j] = sum_l C[c][k][l] V[j][l]   (block (k0.., j0 = l0..))
    if (active) {
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int pp = 0; pp < 2; ++pp)
#pragma unroll
          for (int q = 0; q < 8; ++q) ac2[a][pp][q] = make_float2(0.f, 0.f);
      for (int l = 0; l < A; l += 4) {
        float2 vjp[2][4];  // (V[j][l+m], V[j+1][l+m]) for the two j pairs of this block
#pragma unroll
        for (int pp = 0; pp < 2; ++pp) {
          const float4 r0 = *reinterpret_cast<const float4 *>(V + (l0 + 2 * pp) * A + l);
          const float4 r1 = *reinterpret_cast<const float4 *>(V + (l0 + 2 * pp + 1) * A + l);
          vjp[pp][0] = make_float2(r0.x, r1.x);
          vjp[pp][1] = make_float2(r0.y, r1.y);
          vjp[pp][2] = make_float2(r0.z, r1.z);
          vjp[pp][3] = make_float2(r0.w, r1.w);
        }
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int cc = grp * 8 + q;
#pragma unroll
          for (int a = 0; a < 4; ++a) {
            const float4 cr = *reinterpret_cast<const float4 *>(Cs + ((size_t)cc * A + k0 + a) * A + l);
            const float cv[4] = {cr.x, cr.y, cr.z, cr.w};
#pragma unroll
            for (int m = 0; m < 4; ++m) {
              const float2 cc2 = make_float2(cv[m], cv[m]);
#pragma unroll
              for (int pp = 0; pp < 2; ++pp) ac2[a][pp][q] = __ffma2_rn(cc2, vjp[pp][m], ac2[a][pp][q]);
            }
          }
        }
      }
    }
    __syncthreads();
    if (active) {
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int cc = grp * 8 + q;
#pragma unroll
        for (int a = 0; a < 4; ++a)
          *reinterpret_cast<float4 *>(Cs + ((size_t)cc * A + k0 + a) * A + l0) =
              make_float4(ac2[a][0][q].x, ac2[a][0][q].y, ac2[a][1][q].x, ac2[a][1][q].y);
      }
    }
    __syncthreads();
    // VCV[c][i][j] = sum_k V[i][k] T[c][k][j]   (block (i0 = k0.., j0 = l0..))
    if (active) {
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int pp = 0; pp < 2; ++pp)
#pragma unroll
          for (int q = 0; q < 8; ++q) ac2[a][pp][q] = make_float2(0.f, 0.f);
      for (int k = 0; k < A; ++k) {
        float2 vi2[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) {
          const float v = V[(k0 + a) * A + k];
          vi2[a] = make_float2(v, v);
        }
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int cc = grp * 8 + q;
          const float4 tr = *reinterpret_cast<const float4 *>(Cs + ((size_t)cc * A + k) * A + l0);
          const float2 tp[2] = {make_float2(tr.x, tr.y), make_float2(tr.z, tr.w)};
#pragma unroll
          for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int pp = 0; pp < 2; ++pp) ac2[a][pp][q] = __ffma2_rn(vi2[a], tp[pp], ac2[a][pp][q]);
        }
      }
      if (ncols > 0) {
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int b = 0; b < 4; ++b) {
            const int i = k0 + a, j = l0 + b;
            const float f = (i == j) ? 1.f : Ss[i * A + j];
            float v[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) v[q] = f * ACC(a, b, q);
            store8((size_t)(i * A + j), v, col0, ncols);
          }
      }
    }
    __syncthreads();
  }
  if constexpr (TCB) {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if ((t >> 5) == 0)
      asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(s_tm), "r"(512) : "memory");
  }
  if (t == 0 && s_err && P.err) atomicAdd(P.err, 1);
}
#undef ACC


// The closed-form F81 walk serves the inside-only and F81-staging modes;
// eigen staging of an F81 model keeps the general products.
template <int A, bool TC>
int walk_launch_tc(const KParams &p, int mode, float *sa, float *sb, int c_base, int c_count, int grid,
                   cudaStream_t s) {
  const bool f = !TC && p.f81_model != 0;   // (the tensor-core walk is never F81-specialised)
  constexpr bool kF = !TC;
  if (mode == 0)
    return f ? walk_launch1<A, 0, TC, kF>(p, sa, sb, c_base, c_count, grid, s)
             : walk_launch1<A, 0, TC, false>(p, sa, sb, c_base, c_count, grid, s);
  if (mode == 1) return walk_launch1<A, 1, TC, false>(p, sa, sb, c_base, c_count, grid, s);
  return f ? walk_launch1<A, 2, TC, kF>(p, sa, sb, c_base, c_count, grid, s)
           : walk_launch1<A, 2, TC, false>(p, sa, sb, c_base, c_count, grid, s);
}

template <int A>
int walk_launch(const KParams &p, int mode, bool tc, float *sa, float *sb, int c_base, int c_count, int grid,
                cudaStream_t s) {
  if constexpr (A == 64) {
    // the closed-form F81 walk has no matrix products for the tensor cores
    if (tc && !(p.f81_model && mode != 1)) return walk_launch_tc<A, true>(p, mode, sa, sb, c_base, c_count, grid, s);
  }
  return walk_launch_tc<A, false>(p, mode, sa, sb, c_base, c_count, grid, s);
}

template <int A, bool F81, bool TCB, bool PB = false>
int acc_launch1(const KParams &p, const float *sa, const float *sb, int c_base, int c_count, int grid,
                cudaStream_t s) {
  using Gm = AccGeo<A>;
  const size_t smem = TCB ? (size_t)acc_vv_offset<A>() * sizeof(float) + 49152
                          : (size_t)(AccRing<A>::SCAL + 2 * Gm::G + 2 * A * A + A + 2 * Gm::G * A + Gm::G) *
                                sizeof(float);
  cudaError_t e =
      cudaFuncSetAttribute(k_acc<A, F81, TCB, PB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return (int)e;
  k_acc<A, F81, TCB, PB><<<grid, 256, smem, s>>>(p, sa, sb, c_base, c_count);
  return (int)cudaGetLastError();
}

template <int A>
int acc_launch(const KParams &p, bool f81, bool tc, const float *sa, const float *sb, int c_base, int c_count,
               int grid, cudaStream_t s) {
  if (p.mode & kModeBranch)
    return f81 ? acc_launch1<A, true, false, true>(p, sa, sb, c_base, c_count, grid, s)
               : acc_launch1<A, false, false, true>(p, sa, sb, c_base, c_count, grid, s);
  if (f81) return acc_launch1<A, true, false>(p, sa, sb, c_base, c_count, grid, s);
  if constexpr (A == 64) {
    if (tc) return acc_launch1<A, false, true>(p, sa, sb, c_base, c_count, grid, s);
  }
  return acc_launch1<A, false, false>(p, sa, sb, c_base, c_count, grid, s);
}

}  // namespace

bool big_supported(int A) { return A == 16 || A == 20 || A == 32 || A == 64; }
int big_tile() { return kTile; }
int big_acc_group(int A) {
  switch (A) {
    case 16: return AccGeo<16>::G;
    case 20: return AccGeo<20>::G;
    case 32: return AccGeo<32>::G;
    case 64: return AccGeo<64>::G;
    default: return 0;
  }
}

int launch_walk(const KParams &p, int A, int mode, bool tc, float *sa, float *sb, int c_base, int c_count,
                int grid, cudaStream_t s) {
  switch (A) {
    case 16: return walk_launch<16>(p, mode, false, sa, sb, c_base, c_count, grid, s);
    case 20: return walk_launch<20>(p, mode, false, sa, sb, c_base, c_count, grid, s);
    case 32: return walk_launch<32>(p, mode, false, sa, sb, c_base, c_count, grid, s);
    case 64: return walk_launch<64>(p, mode, tc, sa, sb, c_base, c_count, grid, s);
    default: return -1;
  }
}

int launch_acc(const KParams &p, int A, bool f81, bool tc, const float *sa, const float *sb, int c_base,
               int c_count, int grid, cudaStream_t s) {
  switch (A) {
    case 16: return acc_launch<16>(p, f81, false, sa, sb, c_base, c_count, grid, s);
    case 20: return acc_launch<20>(p, f81, false, sa, sb, c_base, c_count, grid, s);
    case 32: return acc_launch<32>(p, f81, false, sa, sb, c_base, c_count, grid, s);
    case 64: return acc_launch<64>(p, f81, tc, sa, sb, c_base, c_count, grid, s);
    default: return -1;
  }
}

}  // namespace subby
