// Tree walk of the large-alphabet path (A = 4 .. 64): k_walk<A, MODE, TC, F81M>
// and its launcher, shared by the count path (k_big.cu) and the posterior
// path (k_walkpost.cu).
//
// Kernel 1, k_walk<A>: the tree program of k_tree.cu (stored / derived
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
#pragma once
#include <cuda_bf16.h>

#include "common.cuh"

namespace subby {
namespace {


constexpr double kLn2b = 0.69314718055994530942;
constexpr int kTile = 128;  // columns per CTA tile of k_walk

__device__ __forceinline__ int btcode(int tok, int A) { return (int)min((unsigned)tok, (unsigned)A); }
__device__ __forceinline__ int btung(int tok, int A) { return (unsigned)tok <= (unsigned)A; }

template <int A>
struct Geo {
  static constexpr int H = (A + 31) / 32;      // threads per column
  static constexpr int S = A < 32 ? A : 32;    // states per thread
  static_assert(A % 4 == 0, "A must be a multiple of 4");
};

template <int A>
struct BV {
  float v[Geo<A>::S];
};

// Pair barrier: the two warps (w, w + 4) that share columns.
__device__ __forceinline__ void pair_sync(int warp) {
  asm volatile("bar.sync %0, 64;" ::"r"(1 + (warp & 3)) : "memory");
}

// ---- tensor-core (tcgen05) helpers for the A = 64 walk -------------------
// Operands use the canonical K-major layout without swizzle: element (r, k)
// of a tile with K = 64 sits at byte (r&7)*16 + (r>>3)*1024 + (k&7)*2 +
// (k>>3)*128 (8 x 16-byte core matrices; 128 B between K-adjacent and
// 1024 B between M/N-adjacent core matrices).
__device__ __forceinline__ uint32_t kmaj_off(int r, int k) {
  return (uint32_t)((r & 7) * 16 + (r >> 3) * 1024 + (k & 7) * 2 + (k >> 3) * 128);
}
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr) {
  return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46);
}
// kind::f16, BF16 x BF16 -> F32, K-major A and B, M = 128, N = 64
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(64 >> 3) << 17) |
                            ((uint32_t)(128 >> 4) << 24);
constexpr uint32_t kIdesc128 = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(128 >> 3) << 17) |
                               ((uint32_t)(128 >> 4) << 24);
constexpr int kWaitLimit = 1 << 24;  // bounded mbarrier waits

__device__ __forceinline__ bool mbar_wait(uint32_t mb, uint32_t phase, int limit = kWaitLimit) {
  for (int it = 0; it < limit; ++it) {
    uint32_t done;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
                 : "=r"(done)
                 : "r"(mb), "r"(phase)
                 : "memory");
    if (done) return true;
  }
  return false;
}

// Shared-memory operand layout of the tensor-core walk (dynamic, 168 KB):
//   sA   [0,   48K)  A operand 0: three BF16 terms of 16 KB (128 columns x 64)
//   sA1  [48K, 96K)  A operand 1 (the U of an outside-pass product)
//   sB2  [96K,144K)  three terms of 16 KB, each [per-node matrix 8 KB | Vd 8 KB]:
//                    a stacked 128 x 64 B operand [MN_n ; Vd^T-tile] (N = 128)
//   sBu  [144K,168K) Vu tile, three terms of 8 KB
// Vd and Vu are loaded once per CTA; per-node matrices per product.
constexpr uint32_t kSA1 = 49152, kSB2 = 98304, kSBu = 147456, kTcDyn = 172032;
struct TcState {
  uint32_t tmem;    // accumulators: 128 lanes x 192 fp32 columns (O | dt | ut)
  uint32_t sA;      // shared address of the operand area
  uint32_t mbB, mbM;
  uint32_t nB, nM;  // completed phases of the copy and MMA mbarriers
  int *err;         // shared: set when a bounded wait gives up
};

template <int A>
struct Walk {
  static constexpr int H = Geo<A>::H;
  static constexpr int S = Geo<A>::S;
  int c, h, warp;
  float *xch;     // shared exchange buffer: [2][32 states][128 cols] floats
  int *xmax;      // shared [2][128] ints (exponent-field exchange)
  TcState tcs;    // tensor-core state (per thread copy; used when use_tc)
  bool use_tc;

  // y = (B x) on the tensor cores for the 128 columns of the tile at once:
  // D[c][b] = sum_j X[c][j] B[b][j].  X and B are each split into three
  // BF16 terms (v = v1 + v2 + v3, v2 = bf16(v - v1), v3 = bf16(v - v1 - v2))
  // and the six products with combined order <= 4 (1.1, 1.2, 2.1, 1.3, 2.2,
  // 3.1) accumulate in FP32 in TMEM, which keeps FP32-level accuracy (the
  // two-term split measured 1.5e-4 column-wise counts error at A = 64).
  // Bg: the B tile's three terms (4096 elements each) in the canonical
  // layout in global memory, brought in by bulk copies.
  // x (this thread's 32 states of column c) as three BF16 terms into the
  // canonical K-major A tile at shared address base
  __device__ __forceinline__ void stage_x(const BV<A> &x, uint32_t base) const {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      uint32_t t1[4], t2[4], t3[4];
#pragma unroll
      for (int pp = 0; pp < 4; ++pp) {
        const float a0 = x.v[8 * q + 2 * pp], a1 = x.v[8 * q + 2 * pp + 1];
        const __nv_bfloat162 b1 = __floats2bfloat162_rn(a0, a1);
        const float2 f1 = __bfloat1622float2(b1);
        const float r0 = a0 - f1.x, r1 = a1 - f1.y;
        const __nv_bfloat162 b2 = __floats2bfloat162_rn(r0, r1);
        const float2 f2 = __bfloat1622float2(b2);
        const __nv_bfloat162 b3 = __floats2bfloat162_rn(r0 - f2.x, r1 - f2.y);
        t1[pp] = *reinterpret_cast<const uint32_t *>(&b1);
        t2[pp] = *reinterpret_cast<const uint32_t *>(&b2);
        t3[pp] = *reinterpret_cast<const uint32_t *>(&b3);
      }
      const uint32_t off = kmaj_off(c, 32 * h + 8 * q);
      asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(base + off), "r"(t1[0]), "r"(t1[1]), "r"(t1[2]),
                   "r"(t1[3]) : "memory");
      asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(base + 16384 + off), "r"(t2[0]), "r"(t2[1]),
                   "r"(t2[2]), "r"(t2[3]) : "memory");
      asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(base + 32768 + off), "r"(t3[0]), "r"(t3[1]),
                   "r"(t3[2]), "r"(t3[3]) : "memory");
    }
  }
  // bring a per-node B tile (three terms) into the matrix slots of sB2
  __device__ __forceinline__ void load_node_B(const uint16_t *Bg) {
    TcState &T = tcs;
    if (threadIdx.x == 0) {
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(T.mbB), "r"(3 * 8192) : "memory");
#pragma unroll
      for (int part = 0; part < 3; ++part)
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                     ::"r"(T.sA + kSB2 + part * 16384), "l"(Bg + part * 4096), "r"(8192), "r"(T.mbB) : "memory");
    }
    __syncwarp();  // warp 0 whole again before the next warp-collective step
  }
  // A-tile stores visible to the tensor cores, then every thread past the barrier
  // (__syncwarp first: bar.sync is warp-aligned, and a warp that reaches it
  // diverged may be counted as arrived before all its lanes stored)
  __device__ __forceinline__ void tc_sync() const {
    __syncwarp();
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  }
  // the six (A term, B term) products with combined order <= 4 over K = 64
  __device__ __forceinline__ static void mma6(uint32_t d, uint32_t a, uint32_t astride, uint32_t b,
                                              uint32_t bstride, uint32_t idesc) {
    constexpr int pa[6] = {0, 0, 1, 0, 1, 2}, pb[6] = {0, 1, 0, 2, 1, 0};
#pragma unroll
    for (int ks = 0; ks < 4; ++ks) {
#pragma unroll
      for (int prod = 0; prod < 6; ++prod) {
        const uint32_t accum = (ks | prod) != 0;
        asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                     " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}"
                     ::"r"(d), "l"(umma_desc(a + pa[prod] * astride + ks * 256)),
                     "l"(umma_desc(b + pb[prod] * bstride + ks * 256)), "r"(idesc), "r"(accum) : "memory");
      }
    }
  }
  // wait for the MMAs of this round trip.  Lane 0 of warp 0 arrives here
  // after issuing them while the other lanes poll already; the __syncwarp
  // reconverges the warp before the warp-collective (.sync.aligned)
  // tensor-memory loads that follow.
  __device__ __forceinline__ void mma_wait() {
    TcState &T = tcs;
    if (!mbar_wait(T.mbM, T.nM & 1)) *T.err = 1;
    T.nM += 1;
    __syncwarp();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  }
  // this thread's 32 FP32 accumulator columns [col, col + 32) of its lane
  __device__ __forceinline__ void tm_ld32(BV<A> &y, uint32_t col) const {
    uint32_t r[32];
    const uint32_t ta = tcs.tmem + ((uint32_t)(32 * (warp & 3)) << 16) + col;
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                 "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
                 "tcgen05.wait::ld.sync.aligned;"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                   "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
                   "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
                   "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                 : "r"(ta)
                 : "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) y.v[i] = __uint_as_float(r[i]);
  }

  // y = (B x) on the tensor cores for the 128 columns of the tile at once:
  // D[c][b] = sum_j X[c][j] B[b][j].  X and B are each split into three
  // BF16 terms (v = v1 + v2 + v3, v2 = bf16(v - v1), v3 = bf16(v - v1 - v2))
  // and the six products with combined order <= 4 (1.1, 1.2, 2.1, 1.3, 2.2,
  // 3.1) accumulate in FP32 in TMEM, which keeps FP32-level accuracy (the
  // two-term split measured 1.5e-4 column-wise counts error at A = 64).
  // Bg: the B tile's three terms (4096 elements each) in the canonical
  // layout in global memory, brought in by bulk copies.
  __device__ __forceinline__ void matvec_tc(BV<A> &y, const BV<A> &x, const uint16_t *Bg) {
    static_assert(A == 64, "tensor-core walk is A = 64");
    TcState &T = tcs;
    load_node_B(Bg);
    stage_x(x, T.sA);
    tc_sync();
    if (threadIdx.x == 0) {
      if (!mbar_wait(T.mbB, T.nB & 1)) *T.err = 1;
      mma6(T.tmem, T.sA, 16384, T.sA + kSB2, 16384, kIdesc);
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(T.mbM)
                   : "memory");
    }
    __syncwarp();
    T.nB += 1;
    mma_wait();
    tm_ld32(y, 32u * h);
  }

  // Outside-pass products of one branch in a single round trip:
  //   O = MN_n-product of D and dt = Vd-product of D (stacked, N = 128) when
  //   MNg is given, dt alone (N = 64) otherwise; ut = Vu-product of U when U
  //   is given.  dt is scaled by s and stored to pa, ut to pb (when store).
  __device__ __forceinline__ void outside_tc(BV<A> &O, const BV<A> &D, const BV<A> *U, const uint16_t *MNg,
                                             float s, float *pa, float *pb, bool store) {
    TcState &T = tcs;
    const bool wantO = MNg != nullptr, wantU = U != nullptr;
    if (wantO) load_node_B(MNg);
    stage_x(D, T.sA);
    if (wantU) stage_x(*U, T.sA + kSA1);
    tc_sync();
    if (threadIdx.x == 0) {
      if (wantO) {
        if (!mbar_wait(T.mbB, T.nB & 1)) *T.err = 1;
        mma6(T.tmem, T.sA, 16384, T.sA + kSB2, 16384, kIdesc128);
      } else {
        mma6(T.tmem + 64, T.sA, 16384, T.sA + kSB2 + 8192, 16384, kIdesc);
      }
      if (wantU) mma6(T.tmem + 128, T.sA + kSA1, 16384, T.sA + kSBu, 8192, kIdesc);
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(T.mbM)
                   : "memory");
    }
    __syncwarp();
    if (wantO) T.nB += 1;
    mma_wait();
    {
      BV<A> t;
      tm_ld32(t, 64u + 32u * h);
#pragma unroll
      for (int i = 0; i < 32; ++i) t.v[i] *= s;
      if (store) st(pa, t);
    }
    if (wantU) {
      BV<A> t;
      tm_ld32(t, 128u + 32u * h);
      if (store) st(pb, t);
    }
    if (wantO) tm_ld32(O, 32u * h);
  }

  __device__ __forceinline__ void ld(BV<A> &o, const float *p) const {  // S contiguous floats
#pragma unroll
    for (int q = 0; q < S / 4; ++q) {
      const float4 t = *reinterpret_cast<const float4 *>(p + 4 * q);
      o.v[4 * q] = t.x, o.v[4 * q + 1] = t.y, o.v[4 * q + 2] = t.z, o.v[4 * q + 3] = t.w;
    }
  }
  __device__ __forceinline__ void st(float *p, const BV<A> &x) const {
#pragma unroll
    for (int q = 0; q < S / 4; ++q)
      *reinterpret_cast<float4 *>(p + 4 * q) = make_float4(x.v[4 * q], x.v[4 * q + 1], x.v[4 * q + 2], x.v[4 * q + 3]);
  }
  __device__ __forceinline__ void obs(BV<A> &x, int code) const {
    if (code < A) {
#pragma unroll
      for (int i = 0; i < S; ++i) x.v[i] = (32 * h + i == code) ? x.v[i] : 0.f;
    }
  }
  __device__ __forceinline__ void fill(BV<A> &x, float s) const {
#pragma unroll
    for (int i = 0; i < S; ++i) x.v[i] = s;
  }
  // exponent field of the column max (combined over the H threads)
  __device__ __forceinline__ int maxfield(const BV<A> &x) const {
    float m = x.v[0];
#pragma unroll
    for (int i = 1; i < S; ++i) m = fmaxf(m, x.v[i]);
    int E = __float_as_int(m) >> 23;
    if constexpr (H == 2) {
      xmax[h * kTile + c] = E;
      pair_sync(warp);
      E = max(E, xmax[(1 - h) * kTile + c]);
      pair_sync(warp);
    }
    return E;
  }
  // multiply by 2^-e, e = floor(log2 max); returns e (zero vector: -127)
  __device__ __forceinline__ int rescale(BV<A> &x) const {
    const int E = maxfield(x);
    const float s = __int_as_float((254 - E) << 23);
#pragma unroll
    for (int i = 0; i < S; ++i) x.v[i] *= s;
    return E - 127;
  }
  // F81 / JC closed form of the two products with M = e I + (1 - e) 1 pi^T:
  //   M u     : y_a = e u_a + (1 - e) (pi . u)
  //   D^T M   : y_b = e D_b + (1 - e) pi_b (sum_a D_a)        (trans)
  // The column's dot product is combined over its H threads.
  __device__ __forceinline__ void f81prod(BV<A> &y, const BV<A> &x, float e, float ome, bool trans,
                                          const BV<A> &piv) const {
    float sd = 0.f;
#pragma unroll
    for (int i = 0; i < S; ++i) sd = trans ? sd + x.v[i] : fmaf(piv.v[i], x.v[i], sd);
    if constexpr (H == 2) {
      xch[h * kTile + c] = sd;
      pair_sync(warp);
      sd += xch[(1 - h) * kTile + c];
      pair_sync(warp);
    }
    const float q = ome * sd;
#pragma unroll
    for (int i = 0; i < S; ++i) y.v[i] = fmaf(e, x.v[i], trans ? q * piv.v[i] : q);
  }
  // y_b = sum_j T[j][b] x_j over all A inputs j (T rows contiguous, stride A);
  // on the tensor cores when enabled, with Bg the same product's B tile.
  __device__ __forceinline__ void matvec(BV<A> &y, const BV<A> &x, const float *__restrict__ T,
                                         const uint16_t *Bg = nullptr) {
    if constexpr (A == 64) {
      if (use_tc) {
        matvec_tc(y, x, Bg);
        return;
      }
    }
    if constexpr (H == 1) {
#pragma unroll
      for (int i = 0; i < S; ++i) y.v[i] = 0.f;
#pragma unroll 4
      for (int j = 0; j < A; ++j) {
        const float xj = x.v[j];
#pragma unroll
        for (int q = 0; q < A / 4; ++q) {
          const float4 t = __ldg(reinterpret_cast<const float4 *>(T + j * A) + q);
          y.v[4 * q] = fmaf(t.x, xj, y.v[4 * q]);
          y.v[4 * q + 1] = fmaf(t.y, xj, y.v[4 * q + 1]);
          y.v[4 * q + 2] = fmaf(t.z, xj, y.v[4 * q + 2]);
          y.v[4 * q + 3] = fmaf(t.w, xj, y.v[4 * q + 3]);
        }
      }
    } else {
      // partial sums over my 32 inputs for all 64 outputs, then swap halves
      float p[64];
#pragma unroll
      for (int b = 0; b < 64; ++b) p[b] = 0.f;
#pragma unroll 2
      for (int i = 0; i < 32; ++i) {
        const float xj = x.v[i];
        const float4 *row = reinterpret_cast<const float4 *>(T + (32 * h + i) * 64);
#pragma unroll
        for (int q = 0; q < 16; ++q) {
          const float4 t = __ldg(row + q);
          p[4 * q] = fmaf(t.x, xj, p[4 * q]);
          p[4 * q + 1] = fmaf(t.y, xj, p[4 * q + 1]);
          p[4 * q + 2] = fmaf(t.z, xj, p[4 * q + 2]);
          p[4 * q + 3] = fmaf(t.w, xj, p[4 * q + 3]);
        }
      }
      // hand the partner its half: xch[dst h][i][c]
      float *out = xch + (1 - h) * 32 * kTile;
#pragma unroll
      for (int i = 0; i < 32; ++i) out[i * kTile + c] = h ? p[i] : p[32 + i];
      pair_sync(warp);
      const float *in = xch + h * 32 * kTile;
#pragma unroll
      for (int i = 0; i < 32; ++i) y.v[i] = (h ? p[32 + i] : p[i]) + in[i * kTile + c];
      pair_sync(warp);
    }
  }
};

template <int A>
struct BN {
  BV<A> cc;
  int e, hh, init, code;
};

// MODE: 0 inside only, 1 eigen staging, 2 F81 (raw) staging, 3 node
// posteriors (and raw staging when stage_a is given); F81M: the model is
// F81 / JC and the M products take the closed form; ND: the program has no
// derived nodes (every internal node stored), so the derived-node paths are
// not compiled (fewer live registers)
template <int A, int MODE, bool TC, bool F81M, bool ND = false>
__global__ void __launch_bounds__(128 * Geo<A>::H, 1) k_walk(const KParams P, float *__restrict__ stage_a,
                                                              float *__restrict__ stage_b, int c_base,
                                                              int c_count) {
  constexpr int S = Geo<A>::S;
  __shared__ __align__(16) float s_xch[(Geo<A>::H == 2 && !TC) ? 2 * 32 * kTile : 2 * kTile];
  __shared__ int s_xmax[2 * kTile];
  Walk<A> wk;
  wk.use_tc = TC;
  __shared__ TcState s_tc;
  __shared__ __align__(8) uint64_t s_mbar[2];
  __shared__ uint32_t s_taddr;
  __shared__ int s_err;
  __shared__ int s_skip;
  extern __shared__ __align__(1024) unsigned char s_dyn[];  // TC: operand tiles (layout at TcState)
  if constexpr (TC) {
    if ((threadIdx.x >> 5) == 0) {
      const uint32_t dst = (uint32_t)__cvta_generic_to_shared(&s_taddr);
      asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst), "r"(256)
                   : "memory");
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (threadIdx.x == 0) {
      s_err = 0;
      for (int i = 0; i < 2; ++i) {
        const uint32_t mb = (uint32_t)__cvta_generic_to_shared(&s_mbar[i]);
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb) : "memory");
      }
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (threadIdx.x == 0) {
      s_tc.tmem = s_taddr;
      s_tc.sA = (uint32_t)__cvta_generic_to_shared(s_dyn);
      s_tc.mbB = (uint32_t)__cvta_generic_to_shared(&s_mbar[0]);
      s_tc.mbM = (uint32_t)__cvta_generic_to_shared(&s_mbar[1]);
      s_tc.nB = 0;
      s_tc.nM = 0;
      s_tc.err = &s_err;
      // Test hook of the failure path: wait on the MMA mbarrier, which
      // nothing has armed yet (no copy or MMA is in flight), for a few
      // polls; the wait gives up and the CTA skips its work.
      s_skip = P.dbg_wait_polls > 0 && !mbar_wait(s_tc.mbM, 0, P.dbg_wait_polls);
      if (MODE == 1 && !s_skip) {
        // Vd (stacked behind the per-node matrix slots) and Vu, once per CTA
        const uint16_t *Vg = P.tab16 + (size_t)P.R * 24576;
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(s_tc.mbB), "r"(6 * 8192)
                     : "memory");
        for (int part = 0; part < 3; ++part) {
          asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                       ::"r"(s_tc.sA + kSB2 + part * 16384 + 8192), "l"(Vg + part * 4096), "r"(8192),
                       "r"(s_tc.mbB) : "memory");
          asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                       ::"r"(s_tc.sA + kSBu + part * 8192), "l"(Vg + 12288 + part * 4096), "r"(8192),
                       "r"(s_tc.mbB) : "memory");
        }
        if (!mbar_wait(s_tc.mbB, 0)) s_err = 1;
        s_tc.nB = 1;
      }
    }
    __syncwarp();
    __syncthreads();
    wk.tcs = s_tc;
    if (s_skip) {
      // the test hook's wait gave up (nothing in flight): free the tensor
      // memory, record the failure in the status word, leave the outputs
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncthreads();
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      if ((threadIdx.x >> 5) == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(s_tc.tmem), "r"(256) : "memory");
      if (threadIdx.x == 0 && P.err) atomicAdd(P.err, 1);
      return;
    }
  }
  wk.warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  wk.c = lane + 32 * (wk.warp & 3);
  wk.h = wk.warp >> 2;
  wk.xch = s_xch;
  wk.xmax = s_xmax;
  const int h = wk.h, cl = wk.c;

  const float *MT = P.tab + P.off.MT;
  const float *MN = P.tab + P.off.MN;
  const float *Vu = P.tab + P.off.Vu;
  const float *Vd = P.tab + P.off.Vd;
  const float *Ut = P.tab + P.off.Ut;
  const float *pig = P.tab + P.off.pi;
  const float *pr0g = P.tab + P.off.pi0;   // root prior
  const int4 *prog = P.prog;
  const int C = P.C;
  const size_t tile_slots = (size_t)P.nslots * kTile;
  float *svec = P.scrV + (size_t)blockIdx.x * tile_slots * A;  // [slot][c][A]
  // slot words (exponent, mask flags) [h][slot][c]: each half of a column
  // keeps its own copy, so no word crosses warps between barriers
  int *sword = P.scrW + (size_t)blockIdx.x * tile_slots * Geo<A>::H;
  BV<A> piv;
  wk.ld(piv, pig + 32 * h);
  const float *EF = P.tab + P.off.EF;
  constexpr bool f81m = F81M;
  // the walk's M products: y = M_n x (inside) or y = x^T M_n (outside, trans)
  auto mprod = [&](BV<A> &y, const BV<A> &x, int n, bool trans) {
    if constexpr (f81m) {
      wk.f81prod(y, x, __ldg(EF + 2 * n), __ldg(EF + 2 * n + 1), trans, piv);
    } else if (trans) {
      wk.matvec(y, x, MN + (size_t)n * A * A, P.tab16 + (size_t)n * 24576 + 12288);
    } else {
      wk.matvec(y, x, MT + (size_t)n * (A + 1) * A, P.tab16 + (size_t)n * 24576);
    }
  };

  const int ntiles = (c_count + kTile - 1) / kTile;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int cc0 = tile * kTile + cl;              // column within the chunk
    const bool valid = cc0 < c_count;
    const int col = c_base + (valid ? cc0 : c_count - 1);
    const int32_t *alnc = P.aln + col;
    auto tok = [&](int n) { return __ldg(alnc + (size_t)n * C); };
    auto slotv = [&](int s) { return svec + ((size_t)s * kTile + cl) * A + 32 * h; };
    auto slotw = [&](int s) -> int & { return sword[(size_t)h * tile_slots + (size_t)s * kTile + cl]; };
    auto leaf = [&](BN<A> &o, int n) {
      const int t = tok(n);
      o.code = btcode(t, A);
      wk.ld(o.cc, MT + ((size_t)n * (A + 1) + o.code) * A + 32 * h);
      o.e = 0;
      o.hh = o.init = btung(t, A);
    };
    auto stored = [&](BN<A> &o, int s) {
      wk.ld(o.cc, slotv(s));
      const int w = slotw(s);
      o.e = w >> 2, o.hh = (w >> 1) & 1, o.init = w & 1, o.code = -1;
    };
    auto basic = [&](BN<A> &o, int n, int ks) {
      if (ks < 0) leaf(o, n);
      else stored(o, ks);
    };
    // derived node n (children leaves or stored): CC, and its U / children
    auto derive = [&](BN<A> &o, BV<A> &u, BN<A> &k0, BN<A> &k1, int &codec, int n, int4 sc, int ksl, int ksr) {
      basic(k0, sc.z, ksl);
      basic(k1, sc.w, ksr);
      codec = btcode(tok(n), A);
#pragma unroll
      for (int i = 0; i < S; ++i) u.v[i] = k0.cc.v[i] * k1.cc.v[i];
      wk.obs(u, codec);
      o.e = k0.e + k1.e + wk.rescale(u);
      o.hh = k0.hh | k1.hh;
      o.init = k0.hh & k1.hh;
      o.code = -1;
      mprod(o.cc, u, n, false);
    };

    // ---------------------------------------------------------------- inside
    BV<A> ur;
    int eRoot = 0, iRoot = 0;
    if (P.root_is_leaf) {
      wk.fill(ur, 1.f);
      wk.obs(ur, btcode(tok(0), A));
    }
    for (int i = 0; i < P.nsteps; ++i) {
      const int4 s0 = prog[4 * i], s1 = prog[4 * i + 1], s2 = prog[4 * i + 2], s3 = prog[4 * i + 3];
      BN<A> nl, nr;
      {
        BV<A> u;
        BN<A> k0, k1;
        int cd;
        if (!ND && s1.y == -2) derive(nl, u, k0, k1, cd, s1.x, s1, s3.x, s3.y);
        else basic(nl, s1.x, s1.y);
        if (!ND && s2.y == -2) derive(nr, u, k0, k1, cd, s2.x, s2, s3.z, s3.w);
        else basic(nr, s2.x, s2.y);
      }
      BV<A> u;
#pragma unroll
      for (int q = 0; q < S; ++q) u.v[q] = nl.cc.v[q] * nr.cc.v[q];
      wk.obs(u, btcode(tok(s0.x), A));
      const int eU = nl.e + nr.e + wk.rescale(u);
      const int hh = nl.hh | nr.hh, init = nl.hh & nr.hh;
      if (s0.z) {
        ur = u;
        eRoot = eU;
        iRoot = init;
      } else {
        BV<A> cc;
        mprod(cc, u, s0.x, false);
        wk.st(slotv(s0.y), cc);
        slotw(s0.y) = (eU << 2) | (hh << 1) | init;
      }
    }
    // P = pi . U_root (combined over the pair)
    float pp = 0.f;
#pragma unroll
    for (int q = 0; q < S; ++q) pp = fmaf(__ldg(pr0g + 32 * h + q), ur.v[q], pp);
    if constexpr (Geo<A>::H == 2) {
      s_xch[h * kTile + cl] = pp;
      pair_sync(wk.warp);
      pp += s_xch[(1 - h) * kTile + cl];
      pair_sync(wk.warp);
    }
    const float Pp = pp;
    if ((P.mode & kModeLogLike) && valid && h == 0)
      P.logL[col] = (float)((double)eRoot * kLn2b + (double)logf(Pp));
    const float invP = 1.0f / Pp;
    if ((P.mode & kModeRootProb) && valid) {
#pragma unroll
      for (int q = 0; q < S; ++q) P.rootp[(size_t)(32 * h + q) * C + col] = __ldg(pr0g + 32 * h + q) * ur.v[q] * invP;
    }
    if (MODE == 0 || P.nsteps == 0) continue;

    // ---------------------------------------------------------------- outside
    // stage the two vectors of the branch above node n for column cc0
    // DM: D^T M_n when the caller has it (mode 3 node posteriors)
    auto emit = [&](int n, const BV<A> &D, const BV<A> &U, int leafcode, int eDU, int active,
                    const BV<A> *DM = nullptr) {
      float s = invP * __int_as_float((max(-127, min(127, eDU - eRoot)) + 127) << 23);
      s = active ? s : 0.f;
      float *pa = stage_a + ((size_t)(n - 1) * c_count + (valid ? cc0 : c_count - 1)) * A + 32 * h;
      float *pb = stage_b + ((size_t)(n - 1) * c_count + (valid ? cc0 : c_count - 1)) * A + 32 * h;
      if constexpr (MODE == 2 || MODE == 3) {
        BV<A> Ds;
#pragma unroll
        for (int q = 0; q < S; ++q) Ds.v[q] = D.v[q] * s;
        if ((MODE == 2 || stage_a) && valid) {
          wk.st(pa, Ds);
          wk.st(pb, U);
        }
        if constexpr (MODE == 3) {
          // node posterior (D^T M_n) o U normalised over the states
          // (oracle.py:1755-1831); the scale s cancels
          if (P.npost && (P.npost_node < 0 || n == P.npost_node)) {
            // posterior from Y = D^T M_n without copying Y (register pressure)
            auto post = [&](const BV<A> &Y) {
              float z = 0.f;
#pragma unroll
              for (int q = 0; q < S; ++q) z += __fmul_rn(Y.v[q], U.v[q]);
              if constexpr (Geo<A>::H == 2) {
                s_xch[h * kTile + cl] = z;
                pair_sync(wk.warp);
                z += s_xch[(1 - h) * kTile + cl];
                pair_sync(wk.warp);
              }
              const float inv = z > 0.f ? 1.0f / z : 1.0f;
              if (valid) {
                float *o = P.npost + ((size_t)(P.npost_node < 0 ? n : 0) * A + 32 * h) * C + col;
#pragma unroll
                for (int q = 0; q < S; ++q) __stcs(o + (size_t)q * C, __fmul_rn(Y.v[q], U.v[q]) * inv);
              }
            };
            if (DM) {
              post(*DM);
            } else {
              BV<A> y;
              mprod(y, D, n, true);
              post(y);
            }
          }
        } else if (P.stage_c) {
          // the branch's scalars pi . U and sum(s D), combined over the pair
          float pu = 0.f, ds = 0.f;
#pragma unroll
          for (int q = 0; q < S; ++q) {
            pu = fmaf(piv.v[q], U.v[q], pu);
            ds += Ds.v[q];
          }
          if constexpr (Geo<A>::H == 2) {
            s_xch[h * kTile + cl] = pu;
            pair_sync(wk.warp);
            pu += s_xch[(1 - h) * kTile + cl];
            pair_sync(wk.warp);
            s_xch[h * kTile + cl] = ds;
            pair_sync(wk.warp);
            ds += s_xch[(1 - h) * kTile + cl];
            pair_sync(wk.warp);
          }
          if (valid && h == 0) P.stage_c[(size_t)(n - 1) * c_count + cc0] = make_float2(pu, ds);
        }
      } else {
        BV<A> Ds, dt, ut;
#pragma unroll
        for (int q = 0; q < S; ++q) Ds.v[q] = D.v[q] * s;
        wk.matvec(dt, Ds, Vd, P.tab16 + (size_t)P.R * 24576);
        if (leafcode >= 0) wk.ld(ut, Ut + leafcode * A + 32 * h);
        else wk.matvec(ut, U, Vu, P.tab16 + (size_t)P.R * 24576 + 12288);
        if (valid) {
          wk.st(pa, dt);
          wk.st(pb, ut);
        }
      }
    };
    // tensor-core walk, eigen staging: the branch's products in one round
    // trip (Walk::outside_tc); O receives the MN product when MNg is given
    BV<A> Onone;
    auto emit_tc = [&](int n, const BV<A> &D, const BV<A> *U, int leafcode, int eDU, int active, BV<A> &O,
                       const uint16_t *MNg) {
      float s = invP * __int_as_float((max(-127, min(127, eDU - eRoot)) + 127) << 23);
      s = active ? s : 0.f;
      float *pa = stage_a + ((size_t)(n - 1) * c_count + (valid ? cc0 : c_count - 1)) * A + 32 * h;
      float *pb = stage_b + ((size_t)(n - 1) * c_count + (valid ? cc0 : c_count - 1)) * A + 32 * h;
      wk.outside_tc(O, D, leafcode >= 0 ? nullptr : U, MNg, s, pa, pb, valid);
      if (leafcode >= 0 && valid) {
        BV<A> ut;
        wk.ld(ut, Ut + leafcode * A + 32 * h);
        wk.st(pb, ut);
      }
    };
    constexpr bool kFuse = TC && MODE == 1;
    auto act_of = [&](int n, int stn, int stpar) -> int {
      if (P.mask_mode == kMaskAuto) return stn & stpar;
      if (P.mask_mode == kMaskGiven) return P.mask[(size_t)n * C + col] != 0;
      return 1;
    };
    for (int i = P.nsteps - 1; i >= 0; --i) {
      const int4 s0 = prog[4 * i], s1 = prog[4 * i + 1], s2 = prog[4 * i + 2], s3 = prog[4 * i + 3];
      BN<A> nl, nr;
      {
        // derived children's U and children are recomputed when they are
        // processed below instead of being held here (register pressure)
        BV<A> u;
        BN<A> k0, k1;
        int cd;
        if (!ND && s1.y == -2) derive(nl, u, k0, k1, cd, s1.x, s1, s3.x, s3.y);
        else basic(nl, s1.x, s1.y);
        if (!ND && s2.y == -2) derive(nr, u, k0, k1, cd, s2.x, s2, s3.z, s3.w);
        else basic(nr, s2.x, s2.y);
      }
      const int codep = btcode(tok(s0.x), A);
      BV<A> O;
      int eO, stp;
      if (s0.z) {
        wk.ld(O, pr0g + 32 * h);
        wk.obs(O, codep);
        eO = 0;
        stp = iRoot;
      } else {
        BV<A> D, U;
        wk.ld(D, slotv(s0.y));
        const int wd = slotw(s0.y);
        const int eD = wd >> 2;
        stp = (wd >> 1) & 1;
        const int actp = wd & 1;
#pragma unroll
        for (int q = 0; q < S; ++q) U.v[q] = nl.cc.v[q] * nr.cc.v[q];
        wk.obs(U, codep);
        const int eUp = nl.e + nr.e + wk.rescale(U);
        if constexpr (kFuse) {
          if constexpr (f81m) {
            mprod(O, D, s0.x, true);
            emit_tc(s0.x, D, &U, -1, eD + eUp, actp, Onone, nullptr);
          } else {
            emit_tc(s0.x, D, &U, -1, eD + eUp, actp, O, P.tab16 + (size_t)s0.x * 24576 + 12288);
          }
        } else if constexpr (MODE == 3) {
          mprod(O, D, s0.x, true);
          emit(s0.x, D, U, -1, eD + eUp, actp, &O);
        } else {
          emit(s0.x, D, U, -1, eD + eUp, actp);
          mprod(O, D, s0.x, true);
        }
        wk.obs(O, codep);
        eO = eD + wk.rescale(O);
      }
#pragma unroll
#pragma unroll
      for (int side = 0; side < 2; ++side) {
        const BN<A> &me = side ? nr : nl;
        const BN<A> &sib = side ? nl : nr;
        const int4 sc = side ? s2 : s1;
        BV<A> Dc;
#pragma unroll
        for (int q = 0; q < S; ++q) Dc.v[q] = O.v[q] * sib.cc.v[q];
        const int eDc = eO + sib.e;
        const int stc = me.init | (stp & me.hh);
        const int actc = act_of(sc.x, stc, stp);
        if (sc.y == -1) {
          if constexpr (kFuse) {
            emit_tc(sc.x, Dc, nullptr, me.code, eDc, actc, Onone, nullptr);
          } else {
            BV<A> U;
            wk.fill(U, 1.f);
            wk.obs(U, me.code);
            emit(sc.x, Dc, U, me.code, eDc, actc);
          }
        } else if (ND || sc.y >= 0) {
          __syncwarp();
          wk.st(slotv(sc.y), Dc);
          slotw(sc.y) = (eDc << 2) | (stc << 1) | actc;
        } else {
          const int gks[2] = {side ? s3.z : s3.x, side ? s3.w : s3.y};
          const int gn[2] = {sc.z, sc.w};
          BN<A> kk[2];
          basic(kk[0], gn[0], gks[0]);
          basic(kk[1], gn[1], gks[1]);
          const int dcode = btcode(tok(sc.x), A);
          BV<A> Oc;
          {
            BV<A> du;
#pragma unroll
            for (int q = 0; q < S; ++q) du.v[q] = kk[0].cc.v[q] * kk[1].cc.v[q];
            wk.obs(du, dcode);
            wk.rescale(du);  // same exponent as in the gather: eU_c = me.e
            if constexpr (kFuse) {
              if constexpr (f81m) emit_tc(sc.x, Dc, &du, -1, eDc + me.e, actc, Onone, nullptr);
              else emit_tc(sc.x, Dc, &du, -1, eDc + me.e, actc, Oc, P.tab16 + (size_t)sc.x * 24576 + 12288);
            } else if constexpr (MODE == 3) {
              mprod(Oc, Dc, sc.x, true);
              emit(sc.x, Dc, du, -1, eDc + me.e, actc, &Oc);
            } else {
              emit(sc.x, Dc, du, -1, eDc + me.e, actc);
            }
          }
          if constexpr ((!kFuse || f81m) && MODE != 3) mprod(Oc, Dc, sc.x, true);
          wk.obs(Oc, dcode);
          const int eOc = eDc + wk.rescale(Oc);
#pragma unroll
          for (int gs = 0; gs < 2; ++gs) {
            const BN<A> &g = kk[gs];
            const BN<A> &gsib = kk[1 - gs];
            BV<A> Dg;
#pragma unroll
            for (int q = 0; q < S; ++q) Dg.v[q] = Oc.v[q] * gsib.cc.v[q];
            const int eDg = eOc + gsib.e;
            const int stg = g.init | (stc & g.hh);
            const int actg = act_of(gn[gs], stg, stc);
            if (gks[gs] == -1) {
              if constexpr (kFuse) {
                emit_tc(gn[gs], Dg, nullptr, g.code, eDg, actg, Onone, nullptr);
              } else {
                BV<A> U;
                wk.fill(U, 1.f);
                wk.obs(U, g.code);
                emit(gn[gs], Dg, U, g.code, eDg, actg);
              }
            } else {
              wk.st(slotv(gks[gs]), Dg);
              slotw(gks[gs]) = (eDg << 2) | (stg << 1) | actg;
            }
          }
        }
      }
    }
  }
  if constexpr (TC) {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if ((threadIdx.x >> 5) == 0)
      asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(wk.tcs.tmem), "r"(256) : "memory");
    if (threadIdx.x == 0 && s_err && P.err) atomicAdd(P.err, 1);
  }
}


template <int A, int MODE, bool TC, bool F81M, bool ND>
int walk_launch_nd(const KParams &p, float *sa, float *sb, int c_base, int c_count, int grid, cudaStream_t s) {
  const int threads = 128 * Geo<A>::H;
  const size_t dyn = TC ? kTcDyn + 1024 : 0;
  if (TC) {
    cudaError_t e = cudaFuncSetAttribute(k_walk<A, MODE, TC, F81M, ND>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)dyn);
    if (e != cudaSuccess) return (int)e;
  }
  k_walk<A, MODE, TC, F81M, ND><<<grid, threads, dyn, s>>>(p, sa, sb, c_base, c_count);
  return (int)cudaGetLastError();
}
// the eigen-staging walk (Counts, gradients) in its derived-node-free form
// when the program has no derived nodes
template <int A, int MODE, bool TC, bool F81M>
int walk_launch1(const KParams &p, float *sa, float *sb, int c_base, int c_count, int grid, cudaStream_t s) {
  if constexpr (MODE == 1) {
    if (p.noderiv) return walk_launch_nd<A, MODE, TC, F81M, true>(p, sa, sb, c_base, c_count, grid, s);
  }
  return walk_launch_nd<A, MODE, TC, F81M, false>(p, sa, sb, c_base, c_count, grid, s);
}

}  // namespace
}  // namespace subby
