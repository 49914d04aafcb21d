// Tree-program kernel for small even alphabets (A = 2, 4, 6, 8).
//
// One thread owns one alignment column and runs the host-compiled tree
// program for it (subby/oracle/oracle.py:784-1137 and 1190-1256 restated):
//
//   * Every internal non-root node is either STORED (its child contribution
//     CC_n = M_n U_n gets a per-column slot) or DERIVED (both its children
//     are leaves or stored, so CC_n is recomputed from them when needed).
//     The program has one step per stored node plus the root, in postorder.
//     About half of the internal nodes are derived, which halves the
//     per-column state so it fits in shared memory for a whole CTA.
//   * Inside pass (steps forward): U_p = CC_l o CC_r o L(x_p), rescaled by an
//     exact power of two, CC_p = M_p U_p into p's slot.
//   * Outside pass (steps backward = right-first preorder): D_p from its slot,
//     U_p recomputed, branch-p counts, O_p = (D_p^T M_p) o L(x_p), then
//     D_c = O_p o CC_sibling for both children: a leaf child's branch counts
//     are accumulated at once, a stored child's D goes into its slot (the CC
//     it replaces is dead), and a derived child is processed inline.
//   * Branch counts: eigenbasis projection + J-weighted outer product
//     (oracle.py:966-1044) or the F81 closed form (oracle.py:1190-1256), with
//     the Steiner mask bits (oracle.py:1372-1435) riding along.
//   * Epilogue: back-transform V C V^T (FP64 or FP32) and S-weighting
//     (oracle.py:1087-1137).
//
// Vector arithmetic on state pairs uses the packed FP32x2 instructions of
// sm_100+ (__ffma2_rn / __fmul2_rn), halving the issue count of the
// projections and accumulations.  Slots live in shared memory when the
// per-column state fits, otherwise in a per-CTA region of global memory.
#include "common.cuh"

namespace subby {
namespace {

constexpr double kLn2t = 0.69314718055994530942;

template <int A>
struct V {
  static_assert(A % 2 == 0, "even alphabets only");
  float2 p[A / 2];
};

template <int A>
__device__ __forceinline__ float at(const V<A> &x, int a) {
  return (a & 1) ? x.p[a >> 1].y : x.p[a >> 1].x;
}

template <int A>
__device__ __forceinline__ void vld(V<A> &o, const float *s) {
  if constexpr (A % 4 == 0) {
#pragma unroll
    for (int q = 0; q < A / 4; ++q) {
      const float4 t = reinterpret_cast<const float4 *>(s)[q];
      o.p[2 * q] = make_float2(t.x, t.y);
      o.p[2 * q + 1] = make_float2(t.z, t.w);
    }
  } else {
#pragma unroll
    for (int q = 0; q < A / 2; ++q) o.p[q] = reinterpret_cast<const float2 *>(s)[q];
  }
}

template <int A>
__device__ __forceinline__ void vst(float *s, const V<A> &x) {
  if constexpr (A % 4 == 0) {
#pragma unroll
    for (int q = 0; q < A / 4; ++q)
      reinterpret_cast<float4 *>(s)[q] = make_float4(x.p[2 * q].x, x.p[2 * q].y, x.p[2 * q + 1].x,
                                                     x.p[2 * q + 1].y);
  } else {
#pragma unroll
    for (int q = 0; q < A / 2; ++q) reinterpret_cast<float2 *>(s)[q] = x.p[q];
  }
}

template <int A>
__device__ __forceinline__ void vmul(V<A> &o, const V<A> &a, const V<A> &b) {
#pragma unroll
  for (int q = 0; q < A / 2; ++q) o.p[q] = __fmul2_rn(a.p[q], b.p[q]);
}

template <int A>
__device__ __forceinline__ void vscale(V<A> &o, float s) {
  const float2 ss = make_float2(s, s);
#pragma unroll
  for (int q = 0; q < A / 2; ++q) o.p[q] = __fmul2_rn(o.p[q], ss);
}

template <int A>
__device__ __forceinline__ void vfill(V<A> &o, float s) {
#pragma unroll
  for (int q = 0; q < A / 2; ++q) o.p[q] = make_float2(s, s);
}

// token -> code 0..A-1 (observed) or A (unobserved / gap / any other value)
__device__ __forceinline__ int tcode(int tok, int A) {
  return (int)min((unsigned)tok, (unsigned)A);
}
__device__ __forceinline__ int tungapped(int tok, int A) { return (unsigned)tok <= (unsigned)A; }

template <int A>
__device__ __forceinline__ void vobs(V<A> &u, int code) {
  if (code < A) {
#pragma unroll
    for (int a = 0; a < A; ++a) {
      float &r = (a & 1) ? u.p[a >> 1].y : u.p[a >> 1].x;
      r = (a == code) ? r : 0.f;
    }
  }
}

__device__ __forceinline__ float tpow2(int k) {
  k = max(-127, min(127, k));
  return __int_as_float((k + 127) << 23);
}

// Multiply by 2^-e so that max(u) lands in [1, 2); returns e.
template <int A>
__device__ __forceinline__ int vrescale(V<A> &u) {
  float m = fmaxf(u.p[0].x, u.p[0].y);
#pragma unroll
  for (int q = 1; q < A / 2; ++q) m = fmaxf(m, fmaxf(u.p[q].x, u.p[q].y));
  if (!(m > 0.f) || !(m < 3.0e38f)) return 0;
  int e = ((__float_as_int(m) >> 23) & 0xff) - 127;
  if (e == -127) {
    int ee;
    frexpf(m, &ee);
    e = ee - 1;
#pragma unroll
    for (int q = 0; q < A / 2; ++q) u.p[q] = make_float2(ldexpf(u.p[q].x, -e), ldexpf(u.p[q].y, -e));
    return e;
  }
  vscale<A>(u, __int_as_float((127 - e) << 23));
  return e;
}

// y_b = sum_j T[j][b] x_j  (T row-major A x A in shared memory)
template <int A>
__device__ __forceinline__ void vmat(V<A> &y, const V<A> &x, const float *T) {
  V<A> row;
  vld<A>(row, T);
  const float x0 = at<A>(x, 0);
#pragma unroll
  for (int q = 0; q < A / 2; ++q) y.p[q] = __fmul2_rn(row.p[q], make_float2(x0, x0));
#pragma unroll
  for (int j = 1; j < A; ++j) {
    vld<A>(row, T + j * A);
    const float xj = at<A>(x, j);
#pragma unroll
    for (int q = 0; q < A / 2; ++q) y.p[q] = __ffma2_rn(row.p[q], make_float2(xj, xj), y.p[q]);
  }
}

// y_a = sum_i x_i T[a][i]  (rows of T dotted with x)
template <int A>
__device__ __forceinline__ void vmatT(V<A> &y, const V<A> &x, const float *T) {
#pragma unroll
  for (int a = 0; a < A; ++a) {
    V<A> row;
    vld<A>(row, T + a * A);
    float2 t = __fmul2_rn(row.p[0], x.p[0]);
#pragma unroll
    for (int q = 1; q < A / 2; ++q) t = __ffma2_rn(row.p[q], x.p[q], t);
    float &r = (a & 1) ? y.p[a >> 1].y : y.p[a >> 1].x;
    r = t.x + t.y;
  }
}

template <int A>
struct Node {
  V<A> cc;  // child contribution (leaf: column of M)
  int e;    // cumulative exponent of U
  int h;    // subtree holds an ungapped leaf
  int init; // Steiner seed: ungapped leaf, or both children have ungapped leaves
  int code; // leaf token code, -1 for internal nodes
};

template <int A>
struct Derived {
  V<A> u;       // rescaled U of the derived node
  int codec;    // its token code
  Node<A> k[2]; // its children (leaves or stored)
};

// Where the per-column slot vectors live.
enum : int { kStSmem = 0, kStGlobal = 1, kStTmem = 2 };

// Tensor memory as per-thread scratch: with the 32x32b access shape each
// thread of a warp owns one TMEM lane (lanes 32*(warp%4) ..), and warps
// w and w+4 use disjoint column halves.  Every access is warp-uniform.
__device__ __forceinline__ void tm_st4(uint32_t ta, float a, float b, float c, float d) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x4.b32 [%0], {%1, %2, %3, %4};" ::"r"(ta),
               "r"(__float_as_uint(a)), "r"(__float_as_uint(b)), "r"(__float_as_uint(c)),
               "r"(__float_as_uint(d))
               : "memory");
}
__device__ __forceinline__ void tm_ld4(uint32_t ta, float &a, float &b, float &c, float &d) {
  uint32_t x, y, z, w;
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0, %1, %2, %3}, [%4];"
               : "=r"(x), "=r"(y), "=r"(z), "=r"(w)
               : "r"(ta)
               : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" : "+r"(x), "+r"(y), "+r"(z), "+r"(w)::"memory");
  a = __uint_as_float(x);
  b = __uint_as_float(y);
  c = __uint_as_float(z);
  d = __uint_as_float(w);
}
__device__ __forceinline__ void tm_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

template <int A, int ST>
struct Ctx {
  const int32_t *alnc;
  int C;
  const float *MT;
  float *svec;   // this thread's slot 0 vector (shared or global memory)
  uint32_t tb;   // this thread's slot 0 vector (tensor memory address)
  int *sword;    // this thread's slot 0 word
  int vstride;   // floats between consecutive slots of one thread
  int wstride;   // ints between consecutive slots of one thread

  __device__ __forceinline__ void vload(V<A> &o, int slot) const {
    if constexpr (ST == kStTmem) {
      static_assert(A == 4, "tensor-memory slots hold 4 states");
      tm_ld4(tb + 4 * slot, o.p[0].x, o.p[0].y, o.p[1].x, o.p[1].y);
    } else {
      vld<A>(o, svec + slot * vstride);
    }
  }
  __device__ __forceinline__ void vstore(int slot, const V<A> &v) const {
    if constexpr (ST == kStTmem) {
      tm_st4(tb + 4 * slot, v.p[0].x, v.p[0].y, v.p[1].x, v.p[1].y);
    } else {
      vst<A>(svec + slot * vstride, v);
    }
  }

  __device__ __forceinline__ int tok(int n) const { return __ldg(alnc + (size_t)n * C); }

  __device__ __forceinline__ void leaf(Node<A> &o, int n, int t) const {
    o.code = tcode(t, A);
    vld<A>(o.cc, MT + (n * (A + 1) + o.code) * A);
    o.e = 0;
    o.h = o.init = tungapped(t, A);
  }
  __device__ __forceinline__ void stored(Node<A> &o, int slot) const {
    vload(o.cc, slot);
    const int w = sword[slot * wstride];
    o.e = w >> 2;
    o.h = (w >> 1) & 1;
    o.init = w & 1;
    o.code = -1;
  }
  __device__ __forceinline__ void basic(Node<A> &o, int n, int ks, int t) const {
    if (ks < 0) leaf(o, n, t);
    else stored(o, ks);
  }
  // Recompute a derived node n from its children (leaves or stored); t, tl,
  // tr are the tokens of n and of its two children.
  __device__ __forceinline__ void derive(Node<A> &o, Derived<A> &d, int n, int nl, int nr, int ksl,
                                         int ksr, int t, int tl, int tr) const {
    basic(d.k[0], nl, ksl, tl);
    basic(d.k[1], nr, ksr, tr);
    d.codec = tcode(t, A);
    vmul<A>(d.u, d.k[0].cc, d.k[1].cc);
    vobs<A>(d.u, d.codec);
    o.e = d.k[0].e + d.k[1].e + vrescale<A>(d.u);
    o.h = d.k[0].h | d.k[1].h;
    o.init = d.k[0].h & d.k[1].h;
    o.code = -1;
    vmat<A>(o.cc, d.u, MT + n * (A + 1) * A);
  }
  __device__ __forceinline__ void put(int slot, const V<A> &v, int w) const {
    vstore(slot, v);
    sword[slot * wstride] = w;
  }
};

// Tokens one program step reads: p, l, r and the children of l and r
// (used when l / r is derived).  Loaded one step ahead of their use.
struct Tok7 {
  int t[7];
};

__device__ __forceinline__ void load_tok7(Tok7 &o, const int32_t *alnc, int C, int4 s0, int4 s1, int4 s2) {
  const int n[7] = {s0.x, s1.x, s2.x, max(s1.z, 0), max(s1.w, 0), max(s2.z, 0), max(s2.w, 0)};
#pragma unroll
  for (int i = 0; i < 7; ++i) o.t[i] = __ldg(alnc + (size_t)n[i] * C);
}

template <int A>
struct Acc {
  float2 c[A][A / 2];  // eigen C_kl or F81 G_ij
  float2 h[A / 2];
  float2 g[A / 2];
  float z;
  __device__ __forceinline__ void zero() {
#pragma unroll
    for (int k = 0; k < A; ++k)
#pragma unroll
      for (int q = 0; q < A / 2; ++q) c[k][q] = make_float2(0.f, 0.f);
#pragma unroll
    for (int q = 0; q < A / 2; ++q) h[q] = g[q] = make_float2(0.f, 0.f);
    z = 0.f;
  }
};

template <int A, int ST>
__global__ void __launch_bounds__(256, 1) k_tree(const KParams P) {
  extern __shared__ __align__(16) float sm[];
  for (int t = 0; t < P.ntab; ++t) {
    const SmemTable tb = P.stab[t];
    for (int i = threadIdx.x; i < tb.n; i += blockDim.x) sm[tb.sofs + i] = P.tab[tb.gofs + i];
  }
  {
    int4 *dst = reinterpret_cast<int4 *>(sm + P.smem_steps);
    for (int i = threadIdx.x; i < 4 * P.nsteps; i += blockDim.x) dst[i] = P.prog[i];
  }
  __syncthreads();

  const float *MT = sm + P.stab[0].sofs;
  const float *small = sm + P.stab[1].sofs;
  const float *Vu = small;
  const float *Vd = Vu + A * A;
  const float *Ut = Vd + A * A;
  const float *pi = Ut + (A + 1) * A;
  const float *S32 = pi + A;
  const float *V32 = S32 + A * A;
  const float *TB = (P.ntab > 2) ? sm + P.stab[2].sofs : nullptr;  // J (eigen) or F81 coefs
  const int4 *prog = reinterpret_cast<const int4 *>(sm + P.smem_steps);

  const int nb = blockDim.x;
  const int lane = threadIdx.x & 31;
  const int C = P.C;
  const bool counts = (P.mode & kModeCounts) != 0;
  const bool f81 = (P.mode & kModeF81) != 0;

  Ctx<A, ST> cx;
  cx.C = C;
  cx.MT = MT;
  cx.tb = 0;
  cx.svec = nullptr;
  if (ST == kStGlobal) {
    const size_t per_cta = (size_t)P.nslots * nb;
    cx.svec = P.scrV + ((size_t)blockIdx.x * per_cta + threadIdx.x) * A;
    cx.sword = P.scrW + (size_t)blockIdx.x * per_cta + threadIdx.x;
  } else {
    if (ST == kStSmem) cx.svec = sm + P.smem_slots + threadIdx.x * A;
    cx.sword = reinterpret_cast<int *>(sm + P.smem_words) + threadIdx.x;
  }
  cx.vstride = nb * A;
  cx.wstride = nb;
  uint32_t tmem_base = 0;
  if constexpr (ST == kStTmem) {
    // One CTA per SM owns all 512 TMEM columns (blockDim 128 or 256).
    __shared__ uint32_t s_taddr;
    const int warp = threadIdx.x >> 5;
    if (warp == 0) {
      const uint32_t dst = (uint32_t)__cvta_generic_to_shared(&s_taddr);
      asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst), "r"(512)
                   : "memory");
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    tmem_base = s_taddr;
    const uint32_t cols_per_thread = 512u / (uint32_t)(nb >> 7);
    cx.tb = tmem_base + (((uint32_t)(warp & 3) * 32u) << 16) + (uint32_t)(warp >> 2) * cols_per_thread;
  }

  V<A> piv;
  vld<A>(piv, pi);
  const int stride = gridDim.x * nb;
  for (int c0 = blockIdx.x * nb + threadIdx.x - lane; c0 < C; c0 += stride) {
    const bool valid = c0 + lane < C;
    const int col = valid ? c0 + lane : C - 1;
    cx.alnc = P.aln + col;
    {
      // Pull this thread's next column into L2 while this one is processed.
      const int nxt = c0 + stride + lane;
      if (nxt < C)
        for (int n = 0; n < P.R; ++n) asm volatile("prefetch.global.L2 [%0];" ::"l"(P.aln + (size_t)n * C + nxt));
    }
    // ---------------------------------------------------------------- inside
    V<A> ur;
    int eRoot = 0, iRoot = 0;
    if (P.root_is_leaf) {
      vfill<A>(ur, 1.f);
      vobs<A>(ur, tcode(__ldg(cx.alnc), A));
    }
    Tok7 tk, tn;
    if (P.nsteps > 0) load_tok7(tk, cx.alnc, C, prog[0], prog[1], prog[2]);
    for (int i = 0; i < P.nsteps; ++i) {
      const int4 s0 = prog[4 * i], s1 = prog[4 * i + 1], s2 = prog[4 * i + 2], s3 = prog[4 * i + 3];
      if (i + 1 < P.nsteps) load_tok7(tn, cx.alnc, C, prog[4 * i + 4], prog[4 * i + 5], prog[4 * i + 6]);
      if constexpr (ST == kStTmem) tm_wait_st();
      Node<A> nl, nr;
      Derived<A> dl, dr;
      if (s1.y == -2) cx.derive(nl, dl, s1.x, s1.z, s1.w, s3.x, s3.y, tk.t[1], tk.t[3], tk.t[4]);
      else cx.basic(nl, s1.x, s1.y, tk.t[1]);
      if (s2.y == -2) cx.derive(nr, dr, s2.x, s2.z, s2.w, s3.z, s3.w, tk.t[2], tk.t[5], tk.t[6]);
      else cx.basic(nr, s2.x, s2.y, tk.t[2]);
      V<A> u;
      vmul<A>(u, nl.cc, nr.cc);
      vobs<A>(u, tcode(tk.t[0], A));
      const int eU = nl.e + nr.e + vrescale<A>(u);
      const int h = nl.h | nr.h, init = nl.h & nr.h;
      if (s0.z) {
        ur = u;
        eRoot = eU;
        iRoot = init;
      } else {
        V<A> cc;
        vmat<A>(cc, u, MT + s0.x * (A + 1) * A);
        cx.put(s0.y, cc, (eU << 2) | (h << 1) | init);
      }
      tk = tn;
    }
    float Pp = 0.f;
#pragma unroll
    for (int a = 0; a < A; ++a) Pp = fmaf(at<A>(piv, a), at<A>(ur, a), Pp);
    if ((P.mode & kModeLogLike) && valid) P.logL[col] = (float)((double)eRoot * kLn2t + (double)logf(Pp));
    const float invP = 1.0f / Pp;
    if ((P.mode & kModeRootProb) && valid) {
#pragma unroll
      for (int a = 0; a < A; ++a) P.rootp[(size_t)a * C + col] = at<A>(piv, a) * at<A>(ur, a) * invP;
    }
    if (!counts) continue;
    if (P.nsteps == 0) {
      if (valid)
#pragma unroll
        for (int i = 0; i < A * A; ++i) P.counts[(size_t)i * C + col] = 0.f;
      continue;
    }
    // ---------------------------------------------------------------- outside
    Acc<A> acc;
    acc.zero();

    // Branch contribution for the branch above node n.
    auto branch = [&](int n, const V<A> &D, const V<A> &U, int leafcode, int eDU, int active) {
      const float s = active ? invP * tpow2(eDU - eRoot) : 0.f;
      if (f81) {
        const float4 abg = *reinterpret_cast<const float4 *>(TB + n * 4);
        float piU = 0.f, ds = 0.f;
#pragma unroll
        for (int a = 0; a < A; ++a) {
          piU = fmaf(at<A>(piv, a), at<A>(U, a), piU);
          ds += at<A>(D, a);
        }
        ds *= s;
        const float as = abg.x * s, bh = abg.y * piU * s, bg = abg.y * ds;
#pragma unroll
        for (int i2 = 0; i2 < A; ++i2) {
          const float ai = as * at<A>(D, i2);
#pragma unroll
          for (int q = 0; q < A / 2; ++q) acc.c[i2][q] = __ffma2_rn(make_float2(ai, ai), U.p[q], acc.c[i2][q]);
        }
#pragma unroll
        for (int q = 0; q < A / 2; ++q) {
          acc.h[q] = __ffma2_rn(make_float2(bh, bh), D.p[q], acc.h[q]);
          acc.g[q] = __ffma2_rn(make_float2(bg, bg), U.p[q], acc.g[q]);
        }
        acc.z = fmaf(abg.z * ds, piU, acc.z);
        return;
      }
      V<A> ut, dt;
      if (leafcode >= 0) vld<A>(ut, Ut + leafcode * A);
      else vmat<A>(ut, U, Vu);
      vmat<A>(dt, D, Vd);
      vscale<A>(dt, s);
      const float *Jn = TB + n * A * A;
#pragma unroll
      for (int k = 0; k < A; ++k) {
        V<A> jr;
        vld<A>(jr, Jn + k * A);
        const float dk = at<A>(dt, k);
        const float2 d2 = make_float2(dk, dk);
#pragma unroll
        for (int q = 0; q < A / 2; ++q)
          acc.c[k][q] = __ffma2_rn(__fmul2_rn(jr.p[q], d2), ut.p[q], acc.c[k][q]);
      }
    };
    auto mask_of = [&](int n, int stn, int stpar) -> int {
      if (P.mask_mode == kMaskAuto) return stn & stpar;
      if (P.mask_mode == kMaskGiven) return P.mask[(size_t)n * C + col] != 0;
      return 1;
    };
    // Outside step of an internal node given its D (shared by scheduled and
    // derived nodes): O_n = (D^T M_n) o L(x_n), rescaled.
    auto outside_of = [&](V<A> &O, const V<A> &D, int n, int code) -> int {
      vmatT<A>(O, D, MT + n * (A + 1) * A);
      vobs<A>(O, code);
      return vrescale<A>(O);
    };

    {
      const int j = P.nsteps - 1;
      load_tok7(tk, cx.alnc, C, prog[4 * j], prog[4 * j + 1], prog[4 * j + 2]);
    }
    for (int i = P.nsteps - 1; i >= 0; --i) {
      const int4 s0 = prog[4 * i], s1 = prog[4 * i + 1], s2 = prog[4 * i + 2], s3 = prog[4 * i + 3];
      if (i > 0) load_tok7(tn, cx.alnc, C, prog[4 * i - 4], prog[4 * i - 3], prog[4 * i - 2]);
      if constexpr (ST == kStTmem) tm_wait_st();
      Node<A> nl, nr;
      Derived<A> dl, dr;
      if (s1.y == -2) cx.derive(nl, dl, s1.x, s1.z, s1.w, s3.x, s3.y, tk.t[1], tk.t[3], tk.t[4]);
      else cx.basic(nl, s1.x, s1.y, tk.t[1]);
      if (s2.y == -2) cx.derive(nr, dr, s2.x, s2.z, s2.w, s3.z, s3.w, tk.t[2], tk.t[5], tk.t[6]);
      else cx.basic(nr, s2.x, s2.y, tk.t[2]);
      const int codep = tcode(tk.t[0], A);
      V<A> O;
      int eO, stp;
      if (s0.z) {
        O = piv;
        vobs<A>(O, codep);
        eO = 0;
        stp = iRoot;
      } else {
        V<A> D;
        cx.vload(D, s0.y);
        const int wd = cx.sword[s0.y * cx.wstride];
        const int eD = wd >> 2;
        stp = (wd >> 1) & 1;
        const int actp = wd & 1;
        V<A> U;
        vmul<A>(U, nl.cc, nr.cc);
        vobs<A>(U, codep);
        const int eUp = nl.e + nr.e + vrescale<A>(U);
        branch(s0.x, D, U, -1, eD + eUp, actp);
        eO = eD + outside_of(O, D, s0.x, codep);
      }
      // children: D_c = O o CC_sibling
#pragma unroll
      for (int side = 0; side < 2; ++side) {
        const Node<A> &me = side ? nr : nl;
        const Node<A> &sib = side ? nl : nr;
        const int4 sc = side ? s2 : s1;
        V<A> Dc;
        vmul<A>(Dc, O, sib.cc);
        const int eDc = eO + sib.e;
        const int stc = me.init | (stp & me.h);
        const int actc = mask_of(sc.x, stc, stp);
        if (sc.y == -1) {  // leaf
          V<A> U;
          vfill<A>(U, 1.f);
          vobs<A>(U, me.code);
          branch(sc.x, Dc, U, me.code, eDc, actc);
        } else if (sc.y >= 0) {  // stored: D into its slot
          cx.put(sc.y, Dc, (eDc << 2) | (stc << 1) | actc);
        } else {  // derived: processed inline
          const Derived<A> &d = side ? dr : dl;
          branch(sc.x, Dc, d.u, -1, eDc + me.e, actc);
          V<A> Oc;
          const int eOc = eDc + outside_of(Oc, Dc, sc.x, d.codec);
          const int gks[2] = {side ? s3.z : s3.x, side ? s3.w : s3.y};
          const int gn[2] = {sc.z, sc.w};
#pragma unroll
          for (int gs = 0; gs < 2; ++gs) {
            const Node<A> &g = d.k[gs];
            const Node<A> &gsib = d.k[1 - gs];
            V<A> Dg;
            vmul<A>(Dg, Oc, gsib.cc);
            const int eDg = eOc + gsib.e;
            const int stg = g.init | (stc & g.h);
            const int actg = mask_of(gn[gs], stg, stc);
            if (gks[gs] == -1) {
              V<A> U;
              vfill<A>(U, 1.f);
              vobs<A>(U, g.code);
              branch(gn[gs], Dg, U, g.code, eDg, actg);
            } else {
              cx.put(gks[gs], Dg, (eDg << 2) | (stg << 1) | actg);
            }
          }
        }
      }
      tk = tn;
    }
    // ---------------------------------------------------------------- epilogue
    if (!valid) continue;
    float *out = P.counts + col;
    if (f81) {
      const float mu = P.f81_mu;
#pragma unroll
      for (int i2 = 0; i2 < A; ++i2)
#pragma unroll
        for (int j = 0; j < A; ++j) {
          const float2 cq = acc.c[i2][j >> 1];
          const float I = ((j & 1) ? cq.y : cq.x) + ((i2 & 1) ? acc.h[i2 >> 1].y : acc.h[i2 >> 1].x) +
                          at<A>(piv, i2) * (((j & 1) ? acc.g[j >> 1].y : acc.g[j >> 1].x) + acc.z);
          out[(size_t)(i2 * A + j) * C] = (i2 == j) ? I : mu * at<A>(piv, j) * I;
        }
    } else if (P.mode & kModeBT64) {
      const double *Vg = P.tab64;
      const double *Sg = P.tab64 + A * A;
      double T[A][A];
#pragma unroll
      for (int k = 0; k < A; ++k)
#pragma unroll
        for (int j = 0; j < A; ++j) {
          double v = 0.0;
#pragma unroll
          for (int l = 0; l < A; ++l) {
            const float2 cq = acc.c[k][l >> 1];
            v = fma((double)((l & 1) ? cq.y : cq.x), __ldg(Vg + j * A + l), v);
          }
          T[k][j] = v;
        }
#pragma unroll
      for (int i2 = 0; i2 < A; ++i2)
#pragma unroll
        for (int j = 0; j < A; ++j) {
          double v = 0.0;
#pragma unroll
          for (int k = 0; k < A; ++k) v = fma(__ldg(Vg + i2 * A + k), T[k][j], v);
          out[(size_t)(i2 * A + j) * C] = (float)((i2 == j) ? v : __ldg(Sg + i2 * A + j) * v);
        }
    } else {
      float T[A][A];
#pragma unroll
      for (int k = 0; k < A; ++k)
#pragma unroll
        for (int j = 0; j < A; ++j) {
          float v = 0.f;
#pragma unroll
          for (int l = 0; l < A; ++l) {
            const float2 cq = acc.c[k][l >> 1];
            v = fmaf((l & 1) ? cq.y : cq.x, V32[j * A + l], v);
          }
          T[k][j] = v;
        }
#pragma unroll
      for (int i2 = 0; i2 < A; ++i2)
#pragma unroll
        for (int j = 0; j < A; ++j) {
          float v = 0.f;
#pragma unroll
          for (int k = 0; k < A; ++k) v = fmaf(V32[i2 * A + k], T[k][j], v);
          out[(size_t)(i2 * A + j) * C] = (i2 == j) ? v : S32[i2 * A + j] * v;
        }
    }
  }
  if constexpr (ST == kStTmem) {
    tm_wait_st();
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if ((threadIdx.x >> 5) == 0)
      asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base), "r"(512)
                   : "memory");
  }
}

template <int A, int ST>
int tlaunch(const KParams &p, int grid, int block, size_t smem, cudaStream_t s) {
  cudaError_t e = cudaFuncSetAttribute(k_tree<A, ST>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return (int)e;
  k_tree<A, ST><<<grid, block, smem, s>>>(p);
  return (int)cudaGetLastError();
}

}  // namespace

bool tree_supported(int A) { return A == 2 || A == 4 || A == 6 || A == 8; }

int launch_tree(const KParams &p, int A, int store, int grid, int block, size_t smem,
                cudaStream_t s) {
  if (store == kStTmem) {
    if (A != 4) return -1;
    return tlaunch<4, kStTmem>(p, grid, block, smem, s);
  }
  const bool g = store == kStGlobal;
  switch (A) {
    case 2: return g ? tlaunch<2, kStGlobal>(p, grid, block, smem, s) : tlaunch<2, kStSmem>(p, grid, block, smem, s);
    case 4: return g ? tlaunch<4, kStGlobal>(p, grid, block, smem, s) : tlaunch<4, kStSmem>(p, grid, block, smem, s);
    case 6: return g ? tlaunch<6, kStGlobal>(p, grid, block, smem, s) : tlaunch<6, kStSmem>(p, grid, block, smem, s);
    case 8: return g ? tlaunch<8, kStGlobal>(p, grid, block, smem, s) : tlaunch<8, kStSmem>(p, grid, block, smem, s);
    default: return -1;
  }
}

}  // namespace subby
