// A = 4 specialisation of the tree-program kernel (k_tree.cu), the path of
// the 4-state (DNA) workloads.  Same program and algorithm (inside pass,
// LogLike / root posterior, outside pass fused with the eigenbasis or F81
// count accumulation, Steiner mask, back-transform; subby/oracle/oracle.py
// :784-1256, 1372-1435), specialised for issue efficiency:
//
//  * compile-time counts kind (eigen / F81) and mask mode, so the loop body
//    carries no mode branches;
//  * per-column slot vectors in tensor memory (one CTA of 256 threads per
//    SM owns all 512 TMEM columns, 64 slots per thread), slot words and all
//    tables in shared memory;
//  * all tensor-memory loads of a program step are issued before a single
//    wait, and tokens are fetched one step ahead;
//  * observation likelihoods, leaf projections and leaf-branch J-weights are
//    table lookups (L(code), U~(code), K_n(code) = J_n o U~(code)), so leaf
//    branches need no selects and one multiply less per weight;
//  * branch-free power-of-two rescaling from the exponent bits of the max.
#include "common.cuh"

namespace subby {
namespace {

constexpr double kLn2q = 0.69314718055994530942;

struct F4 {
  float2 a, b;
};

__device__ __forceinline__ F4 ld4s(const float *p) {
  const float4 t = *reinterpret_cast<const float4 *>(p);
  return F4{make_float2(t.x, t.y), make_float2(t.z, t.w)};
}
__device__ __forceinline__ F4 mul4(const F4 &x, const F4 &y) {
  return F4{__fmul2_rn(x.a, y.a), __fmul2_rn(x.b, y.b)};
}
__device__ __forceinline__ F4 scale4(const F4 &x, float s) {
  const float2 ss = make_float2(s, s);
  return F4{__fmul2_rn(x.a, ss), __fmul2_rn(x.b, ss)};
}
__device__ __forceinline__ F4 fma4(float s, const F4 &y, const F4 &z) {
  const float2 ss = make_float2(s, s);
  return F4{__ffma2_rn(ss, y.a, z.a), __ffma2_rn(ss, y.b, z.b)};
}
__device__ __forceinline__ float sum4(const F4 &x) { return (x.a.x + x.a.y) + (x.b.x + x.b.y); }
__device__ __forceinline__ float dot4(const F4 &x, const F4 &y) {
  const float2 t = __ffma2_rn(x.b, y.b, __fmul2_rn(x.a, y.a));
  return t.x + t.y;
}

// Multiply by 2^-e with e = floor(log2(max)); returns e.  The scale factor is
// built from the exponent field of the max, so zero / subnormal maxima take
// e = -127 (scale 2^127): still an exact power of two, no branch.
__device__ __forceinline__ int rescale4(F4 &u) {
  const float m = fmaxf(fmaxf(u.a.x, u.a.y), fmaxf(u.b.x, u.b.y));
  const int E = __float_as_int(m) >> 23;  // m >= 0: sign bit clear
  const float s = __int_as_float((254 - E) << 23);
  u = scale4(u, s);
  return E - 127;
}

// y = M u  with MT rows (MT[j][b] = M[b][j])
__device__ __forceinline__ F4 matvec4(const float *MTn, const F4 &u) {
  F4 y = scale4(ld4s(MTn), u.a.x);
  y = fma4(u.a.y, ld4s(MTn + 4), y);
  y = fma4(u.b.x, ld4s(MTn + 8), y);
  y = fma4(u.b.y, ld4s(MTn + 12), y);
  return y;
}
// y_a = sum_i d_i M[i][a] = dot(MT row a, d)
__device__ __forceinline__ F4 vecmat4(const float *MTn, const F4 &d) {
  return F4{make_float2(dot4(ld4s(MTn), d), dot4(ld4s(MTn + 4), d)),
            make_float2(dot4(ld4s(MTn + 8), d), dot4(ld4s(MTn + 12), d))};
}

__device__ __forceinline__ int tcode4(int tok) { return (int)min((unsigned)tok, 4u); }
__device__ __forceinline__ int tung4(int tok) { return (unsigned)tok <= 4u; }

__device__ __forceinline__ void tmld(uint32_t ta, uint32_t (&r)[4]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0, %1, %2, %3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(ta)
               : "memory");
}
__device__ __forceinline__ void tmst(uint32_t ta, const F4 &v) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x4.b32 [%0], {%1, %2, %3, %4};" ::"r"(ta),
               "r"(__float_as_uint(v.a.x)), "r"(__float_as_uint(v.a.y)), "r"(__float_as_uint(v.b.x)),
               "r"(__float_as_uint(v.b.y))
               : "memory");
}
// Wait for all outstanding tensor-memory loads; the registers are passed
// through so that no use can be scheduled before the wait.
__device__ __forceinline__ void tmwait_ld(uint32_t (&a)[4], uint32_t (&b)[4], uint32_t (&c)[4]) {
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+r"(a[0]), "+r"(a[1]), "+r"(a[2]), "+r"(a[3]), "+r"(b[0]), "+r"(b[1]), "+r"(b[2]),
                 "+r"(b[3]), "+r"(c[0]), "+r"(c[1]), "+r"(c[2]), "+r"(c[3])::"memory");
}
__device__ __forceinline__ void tmwait_touch(uint32_t (&a)[4], uint32_t (&b)[4]) {
  asm volatile("" : "+r"(a[0]), "+r"(a[1]), "+r"(a[2]), "+r"(a[3]), "+r"(b[0]), "+r"(b[1]), "+r"(b[2]),
               "+r"(b[3])::"memory");
}
__device__ __forceinline__ F4 asF4(const uint32_t (&r)[4]) {
  return F4{make_float2(__uint_as_float(r[0]), __uint_as_float(r[1])),
            make_float2(__uint_as_float(r[2]), __uint_as_float(r[3]))};
}

struct N4 {
  F4 cc;
  int e, h, init, code;
};

// Shared-memory table layout (float offsets), set by the host in KParams:
//   stab[0] MT   R x 5 x 4      stab[1] small block (Vu, Vd, Ut, pi, S, V, root prior)
//   stab[2] J    R x 16 (eigen) or F81 R x 4
//   stab[3] K    R x 5 x 20 (eigen: K_n[code][k][l] = J_n[k][l] Ut[code][l], rows padded)
//   stab[4] LV   5 x 4 (observation rows), followed by piL[5] (pi . L(code))
// OUT: kOutSum, the counts summed over branches; kOutBranch, per-branch
// counts (R, 4, 4, C) written branch by branch; kOutPost, node posteriors
// (npost) and / or branch joint posteriors (bpost) of every non-root node
// (InsideOutside.node_posterior / branch_posterior, subby/oracle/oracle.py:
// 1755-1905), the root's row from RootProb.
constexpr int kOutSum = 0, kOutBranch = 1, kOutPost = 2;

// P's tables and tree program into shared memory, and the observation rows
// L(code) (all threads; the caller synchronises before t4_piL).
__device__ __forceinline__ void t4_load(const KParams &P, float *sm) {
  for (int t = 0; t < P.ntab; ++t) {
    const SmemTable tb = P.stab[t];
    for (int i = threadIdx.x; i < tb.n; i += blockDim.x) sm[tb.sofs + i] = P.tab[tb.gofs + i];
  }
  {
    int4 *dst = reinterpret_cast<int4 *>(sm + P.smem_steps);
    for (int i = threadIdx.x; i < 4 * P.nsteps; i += blockDim.x) dst[i] = P.prog[i];
  }
  float *LV = sm + P.stab[P.ntab - 1].sofs;
  if (threadIdx.x < 5) {
    const int c = threadIdx.x;
    for (int a = 0; a < 4; ++a) LV[c * 4 + a] = (c == 4 || c == a) ? 1.f : 0.f;
  }
}
// pi . L(code) behind the observation rows (after t4_load and a barrier).
__device__ __forceinline__ void t4_piL(const KParams &P, float *sm) {
  float *LV = sm + P.stab[P.ntab - 1].sofs;
  const float *pis = sm + P.stab[1].sofs + 52;
  if (threadIdx.x < 5) {
    float s = 0.f;
    for (int a = 0; a < 4; ++a) s = fmaf(pis[a], LV[threadIdx.x * 4 + a], s);
    LV[20 + threadIdx.x] = s;
  }
}

// The columns [c0, c0 + 32) of one warp (lane = column): inside pass,
// LogLike / root posterior, outside pass with the fused count accumulation
// and the epilogue.  sm holds P's tables (t4_load); tb is this warp's
// tensor-memory slot base.
template <bool F81, int MASK, int OUT>
__device__ __forceinline__ void t4_cols(const KParams &P, float *sm, const uint32_t tb, const int c0) {
  const float *LV = sm + P.stab[P.ntab - 1].sofs;
  const float *small = sm + P.stab[1].sofs;
  const float *Vu = small;
  const float *Vd = Vu + 16;
  const float *Ut = Vd + 16;
  const float *pis = Ut + 20;
  const float *S32 = pis + 4;
  const float *V32 = S32 + 16;
  (void)Ut;
  (void)S32;
  (void)V32;
  const int nb = blockDim.x;
  const float *MT = sm + P.stab[0].sofs;
  const float *TB = sm + P.stab[2].sofs;                      // J or F81 coefficients
  const float *KT = F81 ? nullptr : sm + P.stab[3].sofs;       // leaf J o Ut
  const float *piL = LV + 20;
  const int4 *prog = reinterpret_cast<const int4 *>(sm + P.smem_steps);
  int *swd = reinterpret_cast<int *>(sm + P.smem_words) + threadIdx.x;
  const int C = P.C;
  const int lane = threadIdx.x & 31;
  const F4 piv = ld4s(pis);           // the model's pi (F81 formulas)
  const F4 pr0 = ld4s(V32 + 16);      // root prior (pi unless the plan sets another)
  const float mu81 = P.f81_mu;
  const bool valid = c0 + lane < C;
  const int col = valid ? c0 + lane : C - 1;
  const int32_t *alnc = P.aln + col;
  auto tok = [&](int n) { return __ldg(alnc + (size_t)n * C); };
  int tk[7], tn[7];
  auto fetch = [&](int (&o)[7], int i) {
    const int4 s0 = prog[4 * i], s1 = prog[4 * i + 1], s2 = prog[4 * i + 2];
    o[0] = tok(s0.x);
    o[1] = tok(s1.x);
    o[2] = tok(s2.x);
    o[3] = tok(s1.z);  // grandchildren indices are 0 when absent
    o[4] = tok(s1.w);
    o[5] = tok(s2.z);
    o[6] = tok(s2.w);
  };
  // Gather the children of a step: leaves from tables, stored ones from
  // tensor memory (all loads issued before one wait), derived ones
  // recomputed.  dl/dr receive the derived nodes' U and children.
  struct Dv {
    F4 u;
    N4 k[2];
  };
  auto gather = [&](const int4 &s1, const int4 &s2, const int4 &s3, const int (&t)[7], N4 &nl, N4 &nr,
                    Dv &dl, Dv &dr, bool wantD, int slotD, F4 &D, int &wD) {
    // registers of loads that a step does not issue are never read
    uint32_t r0[4], r1[4], r2[4], r3[4], r4[4], r5[4], r6[4];
    // issue
    if (s1.y >= 0) tmld(tb + 4 * s1.y, r0);
    if (s2.y >= 0) tmld(tb + 4 * s2.y, r1);
    if (s1.y == -2) {
      if (s3.x >= 0) tmld(tb + 4 * s3.x, r2);
      if (s3.y >= 0) tmld(tb + 4 * s3.y, r3);
    }
    if (s2.y == -2) {
      if (s3.z >= 0) tmld(tb + 4 * s3.z, r4);
      if (s3.w >= 0) tmld(tb + 4 * s3.w, r5);
    }
    if (wantD) tmld(tb + 4 * slotD, r6);
    tmwait_ld(r0, r1, r2);
    tmwait_touch(r3, r4);
    tmwait_touch(r5, r6);
    auto basic = [&](N4 &o, int n, int ks, int tt, const uint32_t (&r)[4]) {
      if (ks < 0) {
        o.code = tcode4(tt);
        o.cc = ld4s(MT + (n * 5 + o.code) * 4);
        o.e = 0;
        o.h = o.init = tung4(tt);
      } else {
        o.cc = asF4(r);
        const int w = swd[ks * nb];
        o.e = w >> 2;
        o.h = (w >> 1) & 1;
        o.init = w & 1;
        o.code = -1;
      }
    };
    auto derive = [&](N4 &o, Dv &d, int n, int nl_, int nr_, int ksl, int ksr, int tt, int tl, int tr,
                      const uint32_t (&ra)[4], const uint32_t (&rb)[4]) {
      basic(d.k[0], nl_, ksl, tl, ra);
      basic(d.k[1], nr_, ksr, tr, rb);
      d.u = mul4(mul4(d.k[0].cc, d.k[1].cc), ld4s(LV + tcode4(tt) * 4));
      o.e = d.k[0].e + d.k[1].e + rescale4(d.u);
      o.h = d.k[0].h | d.k[1].h;
      o.init = d.k[0].h & d.k[1].h;
      o.code = -1;
      o.cc = matvec4(MT + n * 20, d.u);
    };
    if (s1.y == -2) derive(nl, dl, s1.x, s1.z, s1.w, s3.x, s3.y, t[1], t[3], t[4], r2, r3);
    else basic(nl, s1.x, s1.y, t[1], r0);
    if (s2.y == -2) derive(nr, dr, s2.x, s2.z, s2.w, s3.z, s3.w, t[2], t[5], t[6], r4, r5);
    else basic(nr, s2.x, s2.y, t[2], r1);
    if (wantD) {
      D = asF4(r6);
      wD = swd[slotD * nb];
    }
  };

  // ------------------------------------------------------------ inside
  F4 ur = F4{make_float2(1.f, 1.f), make_float2(1.f, 1.f)};
  int eRoot = 0, iRoot = 0;
  if (P.root_is_leaf) ur = ld4s(LV + tcode4(tok(0)) * 4);
  const int nst = P.nsteps;
  if (nst > 0) fetch(tk, 0);
  for (int i = 0; i < nst; ++i) {
    const int4 s0 = prog[4 * i], s1 = prog[4 * i + 1], s2 = prog[4 * i + 2], s3 = prog[4 * i + 3];
    if (i + 1 < nst) fetch(tn, i + 1);
    asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
    N4 nl, nr;
    Dv dl, dr;
    F4 Dd;
    int wd = 0;
    gather(s1, s2, s3, tk, nl, nr, dl, dr, false, 0, Dd, wd);
    F4 u = mul4(mul4(nl.cc, nr.cc), ld4s(LV + tcode4(tk[0]) * 4));
    const int eU = nl.e + nr.e + rescale4(u);
    const int h = nl.h | nr.h, init = nl.h & nr.h;
    if (s0.z) {
      ur = u;
      eRoot = eU;
      iRoot = init;
    } else {
      tmst(tb + 4 * s0.y, matvec4(MT + s0.x * 20, u));
      swd[s0.y * nb] = (eU << 2) | (h << 1) | init;
    }
#pragma unroll
    for (int q = 0; q < 7; ++q) tk[q] = tn[q];
  }
  const float Pp = dot4(pr0, ur);
  if ((P.mode & kModeLogLike) && valid) P.logL[col] = (float)((double)eRoot * kLn2q + (double)logf(Pp));
  const float invP = 1.0f / Pp;
  if ((P.mode & kModeRootProb) && valid) {
    const F4 q = scale4(mul4(pr0, ur), invP);
    P.rootp[col] = q.a.x;
    P.rootp[(size_t)C + col] = q.a.y;
    P.rootp[(size_t)2 * C + col] = q.b.x;
    P.rootp[(size_t)3 * C + col] = q.b.y;
  }
  if (!(P.mode & kModeCounts) && OUT != kOutPost) return;
  if (OUT == kOutPost && (nst == 0 || P.npost_node == 0)) return;
  if (nst == 0) {
    if (valid)
      for (int i = 0; i < 16; ++i) P.counts[(size_t)i * C + col] = 0.f;
    return;
  }
  // ------------------------------------------------------------ outside
  F4 acc[4];  // eigen C rows / F81 G rows
  F4 hacc = F4{make_float2(0.f, 0.f), make_float2(0.f, 0.f)}, gacc = hacc;
  float zacc = 0.f;
#pragma unroll
  for (int k = 0; k < 4; ++k) acc[k] = hacc;

  // branch above node n; for leaves `code` >= 0 selects the table rows
  // per-branch counts of branch n (kOutBranch): 16 values from the rows I_i
  auto put_branch = [&](int n, const F4 (&I)[4]) {
    float *o = P.counts + (size_t)n * 16 * C + col;
    const float r[4][4] = {{I[0].a.x, I[0].a.y, I[0].b.x, I[0].b.y}, {I[1].a.x, I[1].a.y, I[1].b.x, I[1].b.y},
                           {I[2].a.x, I[2].a.y, I[2].b.x, I[2].b.y}, {I[3].a.x, I[3].a.y, I[3].b.x, I[3].b.y}};
    if (valid)
#pragma unroll
      for (int i2 = 0; i2 < 4; ++i2)
#pragma unroll
        for (int j = 0; j < 4; ++j) __stcs(o + (size_t)(i2 * 4 + j) * C, r[i2][j]);  // streamed: written once
  };
  auto branch = [&](int n, const F4 &D, const F4 &U, int code, int eDU, int active) {
    float s = invP * __int_as_float((max(-127, min(127, eDU - eRoot)) + 127) << 23);
    if (MASK != kMaskNone) s = active ? s : 0.f;
    if constexpr (OUT == kOutPost) {
      // y = D^T M_n; node posterior y o U / Z, branch joint D_i M_n[i][j] U_j / Z
      (void)s;
      if (P.npost_node >= 0 && n != P.npost_node) return;
      const float *Mn = MT + n * 20;
      const F4 p = mul4(vecmat4(Mn, D), U);
      const float z = sum4(p);
      const float inv = z > 0.f ? 1.0f / z : 1.0f;
      if (!valid) return;
      const size_t row = P.npost_node < 0 ? (size_t)n : 0;
      if (P.npost) {
        // streamed stores: the posteriors are written once and not re-read here
        float *o = P.npost + row * 4 * C + col;
        __stcs(o, p.a.x * inv);
        __stcs(o + C, p.a.y * inv);
        __stcs(o + (size_t)2 * C, p.b.x * inv);
        __stcs(o + (size_t)3 * C, p.b.y * inv);
      }
      if (P.bpost) {
        float *o = P.bpost + row * 16 * C + col;
        const F4 ui = scale4(U, inv);
        const float dk[4] = {D.a.x, D.a.y, D.b.x, D.b.y};
#pragma unroll
        for (int i2 = 0; i2 < 4; ++i2) {
          // row i of M_n is column i of the MT rows: M_n[i][j] = MT[n][j][i]
          const F4 mi = F4{make_float2(Mn[i2], Mn[4 + i2]), make_float2(Mn[8 + i2], Mn[12 + i2])};
          const F4 r = scale4(mul4(mi, ui), dk[i2]);
          __stcs(o + (size_t)(4 * i2) * C, r.a.x);
          __stcs(o + (size_t)(4 * i2 + 1) * C, r.a.y);
          __stcs(o + (size_t)(4 * i2 + 2) * C, r.b.x);
          __stcs(o + (size_t)(4 * i2 + 3) * C, r.b.y);
        }
      }
      return;
    }
    const F4 Ds = scale4(D, s);
    if constexpr (OUT == kOutBranch) {
      F4 I[4];
      if constexpr (F81) {
        // I_ij = (alpha Ds_i + beta pi_i sum(Ds)) U_j + (beta Ds_i + gamma pi_i sum(Ds)) pi.U,
        // dwell I_ii, substitutions mu pi_j I_ij (subby/oracle/oracle.py:1259-1331)
        const float4 abg = *reinterpret_cast<const float4 *>(TB + n * 4);
        const float piU = (code >= 0) ? piL[code] : dot4(piv, U);
        const float dsum = sum4(Ds);
        const float dk[4] = {Ds.a.x, Ds.a.y, Ds.b.x, Ds.b.y}, pk[4] = {piv.a.x, piv.a.y, piv.b.x, piv.b.y};
#pragma unroll
        for (int i2 = 0; i2 < 4; ++i2) {
          const float cu = fmaf(abg.x, dk[i2], abg.y * pk[i2] * dsum);
          const float c1 = fmaf(abg.y, dk[i2], abg.z * pk[i2] * dsum) * piU;
          F4 row = fma4(cu, U, F4{make_float2(c1, c1), make_float2(c1, c1)});
          // substitutions: mu pi_j I_ij off the diagonal
          F4 f = scale4(piv, mu81);
          float *fe = i2 < 2 ? (i2 == 0 ? &f.a.x : &f.a.y) : (i2 == 2 ? &f.b.x : &f.b.y);
          *fe = 1.f;
          I[i2] = mul4(row, f);
        }
      } else {
        // eigenbasis C_kl = dt_k (J o U~)_l (leaves: K rows), then V C V^T and S
        F4 dt = scale4(ld4s(Vd), Ds.a.x);
        dt = fma4(Ds.a.y, ld4s(Vd + 4), dt);
        dt = fma4(Ds.b.x, ld4s(Vd + 8), dt);
        dt = fma4(Ds.b.y, ld4s(Vd + 12), dt);
        const float dk[4] = {dt.a.x, dt.a.y, dt.b.x, dt.b.y};
        F4 Cb[4];
        if (code >= 0) {
          const float *K = KT + (n * 5 + code) * 20;
#pragma unroll
          for (int k = 0; k < 4; ++k) Cb[k] = scale4(ld4s(K + 4 * k), dk[k]);
        } else {
          const F4 ut = matvec4(Vu, U);
          const float *Jn = TB + n * 16;
#pragma unroll
          for (int k = 0; k < 4; ++k) Cb[k] = scale4(mul4(ld4s(Jn + 4 * k), ut), dk[k]);
        }
        // T_k = C_k V^T (row k: T[k][j] = sum_l C[k][l] V[j][l]); VCV_i = sum_k V[i][k] T_k
        F4 T[4];
#pragma unroll
        for (int k = 0; k < 4; ++k)
          T[k] = F4{make_float2(dot4(Cb[k], ld4s(V32)), dot4(Cb[k], ld4s(V32 + 4))),
                    make_float2(dot4(Cb[k], ld4s(V32 + 8)), dot4(Cb[k], ld4s(V32 + 12)))};
#pragma unroll
        for (int i2 = 0; i2 < 4; ++i2) {
          const F4 vi = ld4s(V32 + 4 * i2);
          F4 row = scale4(T[0], vi.a.x);
          row = fma4(vi.a.y, T[1], row);
          row = fma4(vi.b.x, T[2], row);
          row = fma4(vi.b.y, T[3], row);
          F4 f = ld4s(S32 + 4 * i2);
          float *fe = i2 < 2 ? (i2 == 0 ? &f.a.x : &f.a.y) : (i2 == 2 ? &f.b.x : &f.b.y);
          *fe = 1.f;
          I[i2] = mul4(row, f);
        }
      }
      put_branch(n, I);
      return;
    }
    if constexpr (F81) {
      const float4 abg = *reinterpret_cast<const float4 *>(TB + n * 4);
      const float piU = (code >= 0) ? piL[code] : dot4(piv, U);
      const float dsum = sum4(Ds);
      const float bh = abg.y * piU, bg = abg.y * dsum;
      const F4 aD = scale4(Ds, abg.x);
      acc[0] = fma4(aD.a.x, U, acc[0]);
      acc[1] = fma4(aD.a.y, U, acc[1]);
      acc[2] = fma4(aD.b.x, U, acc[2]);
      acc[3] = fma4(aD.b.y, U, acc[3]);
      hacc = fma4(bh, Ds, hacc);
      gacc = fma4(bg, U, gacc);
      zacc = fmaf(abg.z * dsum, piU, zacc);
    } else {
      // D~ = Vd^T (s D): d_k = sum_a Ds_a Vd[a][k]
      F4 dt = scale4(ld4s(Vd), Ds.a.x);
      dt = fma4(Ds.a.y, ld4s(Vd + 4), dt);
      dt = fma4(Ds.b.x, ld4s(Vd + 8), dt);
      dt = fma4(Ds.b.y, ld4s(Vd + 12), dt);
      if (code >= 0) {
        const float *K = KT + (n * 5 + code) * 20;  // rows padded to 20: conflict-free
        acc[0] = fma4(dt.a.x, ld4s(K), acc[0]);
        acc[1] = fma4(dt.a.y, ld4s(K + 4), acc[1]);
        acc[2] = fma4(dt.b.x, ld4s(K + 8), acc[2]);
        acc[3] = fma4(dt.b.y, ld4s(K + 12), acc[3]);
      } else {
        const F4 ut = matvec4(Vu, U);  // U~_l = sum_b U_b Vu[b][l]
        const float *Jn = TB + n * 16;
        acc[0] = fma4(dt.a.x, mul4(ld4s(Jn), ut), acc[0]);
        acc[1] = fma4(dt.a.y, mul4(ld4s(Jn + 4), ut), acc[1]);
        acc[2] = fma4(dt.b.x, mul4(ld4s(Jn + 8), ut), acc[2]);
        acc[3] = fma4(dt.b.y, mul4(ld4s(Jn + 12), ut), acc[3]);
      }
    }
  };
  auto act_of = [&](int n, int stn, int stpar) -> int {
    if constexpr (MASK == kMaskAuto) return stn & stpar;
    else if constexpr (MASK == kMaskGiven) return P.mask[(size_t)n * C + col] != 0;
    else return 1;
  };

  fetch(tk, nst - 1);
  for (int i = nst - 1; i >= 0; --i) {
    const int4 s0 = prog[4 * i], s1 = prog[4 * i + 1], s2 = prog[4 * i + 2], s3 = prog[4 * i + 3];
    if (i > 0) fetch(tn, i - 1);
    asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
    N4 nl, nr;
    Dv dl, dr;
    F4 D;
    int wd = 0;
    const bool root = s0.z != 0;
    gather(s1, s2, s3, tk, nl, nr, dl, dr, !root, root ? 0 : s0.y, D, wd);
    const F4 Lp = ld4s(LV + tcode4(tk[0]) * 4);
    F4 O;
    int eO, stp;
    if (root) {
      O = mul4(pr0, Lp);
      eO = 0;
      stp = iRoot;
    } else {
      const int eD = wd >> 2;
      stp = (wd >> 1) & 1;
      const int actp = wd & 1;
      F4 U = mul4(mul4(nl.cc, nr.cc), Lp);
      const int eUp = nl.e + nr.e + rescale4(U);
      branch(s0.x, D, U, -1, eD + eUp, actp);
      O = mul4(vecmat4(MT + s0.x * 20, D), Lp);
      eO = eD + rescale4(O);
    }
#pragma unroll
    for (int side = 0; side < 2; ++side) {
      const N4 &me = side ? nr : nl;
      const N4 &sib = side ? nl : nr;
      const int4 sc = side ? s2 : s1;
      const F4 Dc = mul4(O, sib.cc);
      const int eDc = eO + sib.e;
      const int stc = me.init | (stp & me.h);
      const int actc = act_of(sc.x, stc, stp);
      if (sc.y == -1) {
        branch(sc.x, Dc, ld4s(LV + me.code * 4), me.code, eDc, actc);
      } else if (sc.y >= 0) {
        tmst(tb + 4 * sc.y, Dc);
        swd[sc.y * nb] = (eDc << 2) | (stc << 1) | actc;
      } else {
        const Dv &d = side ? dr : dl;
        branch(sc.x, Dc, d.u, -1, eDc + me.e, actc);
        F4 Oc = mul4(vecmat4(MT + sc.x * 20, Dc), ld4s(LV + tcode4(tk[1 + side]) * 4));
        const int eOc = eDc + rescale4(Oc);
        const int gks[2] = {side ? s3.z : s3.x, side ? s3.w : s3.y};
        const int gn[2] = {sc.z, sc.w};
#pragma unroll
        for (int gs = 0; gs < 2; ++gs) {
          const N4 &g = d.k[gs];
          const N4 &gsib = d.k[1 - gs];
          const F4 Dg = mul4(Oc, gsib.cc);
          const int eDg = eOc + gsib.e;
          const int stg = g.init | (stc & g.h);
          const int actg = act_of(gn[gs], stg, stc);
          if (gks[gs] == -1) {
            branch(gn[gs], Dg, ld4s(LV + g.code * 4), g.code, eDg, actg);
          } else {
            tmst(tb + 4 * gks[gs], Dg);
            swd[gks[gs] * nb] = (eDg << 2) | (stg << 1) | actg;
          }
        }
      }
    }
#pragma unroll
    for (int q = 0; q < 7; ++q) tk[q] = tn[q];
  }
  // ------------------------------------------------------------ epilogue
  if (OUT != kOutSum || !valid) return;
  float *out = P.counts + col;
  if constexpr (F81) {
    float pi_[4] = {piv.a.x, piv.a.y, piv.b.x, piv.b.y};
    float hh[4] = {hacc.a.x, hacc.a.y, hacc.b.x, hacc.b.y};
    float gg[4] = {gacc.a.x, gacc.a.y, gacc.b.x, gacc.b.y};
#pragma unroll
    for (int i2 = 0; i2 < 4; ++i2) {
      const float cr[4] = {acc[i2].a.x, acc[i2].a.y, acc[i2].b.x, acc[i2].b.y};
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const float I = cr[j] + hh[i2] + pi_[i2] * (gg[j] + zacc);
        out[(size_t)(i2 * 4 + j) * C] = (i2 == j) ? I : mu81 * pi_[j] * I;
      }
    }
  } else if (P.mode & kModeBT64) {
    const double *Vg = P.tab64;
    const double *Sg = P.tab64 + 16;
    double T[4][4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const float cr[4] = {acc[k].a.x, acc[k].a.y, acc[k].b.x, acc[k].b.y};
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        double v = 0.0;
#pragma unroll
        for (int l = 0; l < 4; ++l) v = fma((double)cr[l], __ldg(Vg + j * 4 + l), v);
        T[k][j] = v;
      }
    }
#pragma unroll
    for (int i2 = 0; i2 < 4; ++i2)
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        double v = 0.0;
#pragma unroll
        for (int k = 0; k < 4; ++k) v = fma(__ldg(Vg + i2 * 4 + k), T[k][j], v);
        out[(size_t)(i2 * 4 + j) * C] = (float)((i2 == j) ? v : __ldg(Sg + i2 * 4 + j) * v);
      }
  } else {
    float T[4][4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const float cr[4] = {acc[k].a.x, acc[k].a.y, acc[k].b.x, acc[k].b.y};
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        float v = 0.f;
#pragma unroll
        for (int l = 0; l < 4; ++l) v = fmaf(cr[l], V32[j * 4 + l], v);
        T[k][j] = v;
      }
    }
#pragma unroll
    for (int i2 = 0; i2 < 4; ++i2)
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        float v = 0.f;
#pragma unroll
        for (int k = 0; k < 4; ++k) v = fmaf(V32[i2 * 4 + k], T[k][j], v);
        out[(size_t)(i2 * 4 + j) * C] = (i2 == j) ? v : S32[i2 * 4 + j] * v;
      }
  }
}

template <bool F81, int MASK, int OUT>
__global__ void __launch_bounds__(256, 1) k_tree4(const KParams P) {
  extern __shared__ __align__(16) float sm[];
  t4_load(P, sm);
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
  t4_piL(P, sm);
  __syncthreads();
  const uint32_t tmem_base = s_taddr;
  const int nb = blockDim.x;
  const uint32_t tb =
      tmem_base + (((uint32_t)(warp & 3) * 32u) << 16) + (uint32_t)(warp >> 2) * (512u / (uint32_t)(nb >> 7));
  const int lane = threadIdx.x & 31;
  const int stride = gridDim.x * nb;
  const int C = P.C;
  for (int c0 = blockIdx.x * nb + threadIdx.x - lane; c0 < C; c0 += stride) {
    {
      // the token rows of this thread's column of the next tile, into L2
      const int nxt = c0 + stride + lane;
      if (nxt < C)
        for (int n = 0; n < P.R; ++n) asm volatile("prefetch.global.L2 [%0];" ::"l"(P.aln + (size_t)n * C + nxt));
    }
    t4_cols<F81, MASK, OUT>(P, sm, tb, c0);
  }
  asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base), "r"(512)
                 : "memory");
}

// Persistent serving kernel over a flattened (job, column-tile) queue: the
// columns of many small A = 4 jobs in one launch.  Each CTA owns all 512
// tensor-memory columns for its lifetime, claims work items one at a time,
// reloads the tables when the claimed item belongs to another job than the
// previous one, and runs the same per-warp column code as k_tree4, so every
// column's result equals that of a separate call.  A claim past the
// published items waits (bounded) for more until the queue is closed.
__device__ __forceinline__ int ld_acquire(const int *p) {
  int v;
  asm volatile("ld.acquire.sys.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

template <bool F81, int MASK>
__global__ void __launch_bounds__(256, 1) k_tree4_packed(const T4Queue Q) {
  extern __shared__ __align__(16) float sm[];
  __shared__ uint32_t s_taddr;
  __shared__ int s_item;
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
  const uint32_t tmem_base = s_taddr;
  const int nb = blockDim.x;
  const int lane = threadIdx.x & 31;
  const uint32_t tb =
      tmem_base + (((uint32_t)(warp & 3) * 32u) << 16) + (uint32_t)(warp >> 2) * (512u / (uint32_t)(nb >> 7));
  int loaded = -1;
  for (;;) {
    if (threadIdx.x == 0) {
      const int it = atomicAdd(Q.head, 1);
      int avail = ld_acquire(Q.published);
      for (int polls = 0; it >= avail && !ld_acquire(Q.closed) && polls < Q.wait_polls; ++polls) {
        __nanosleep(256);
        avail = ld_acquire(Q.published);
      }
      if (it < avail) {
        s_item = it;
      } else {
        // closed and drained: done; still open after the bounded wait: the
        // wait gave up, which the status word records
        if (!ld_acquire(Q.closed) && Q.err) atomicAdd(Q.err, 1);
        s_item = -1;
      }
    }
    __syncwarp();  // bar.sync is warp-aligned: warp 0 whole before it
    __syncthreads();
    const int it = s_item;
    if (it < 0) break;
    const int4 w = Q.items[it];
    const KParams &P = Q.jobs[w.x];
    if (w.x != loaded) {
      // every thread is past the previous item (barrier above)
      t4_load(P, sm);
      __syncthreads();
      t4_piL(P, sm);
      __syncthreads();
      loaded = w.x;
    }
    for (int c0 = w.y; c0 < w.z; c0 += nb) t4_cols<F81, MASK, kOutSum>(P, sm, tb, c0 + (int)threadIdx.x - lane);
    __syncthreads();  // s_item and, on a job change, the tables are rewritten next
  }
  asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base), "r"(512)
                 : "memory");
}

template <bool F, int M>
int t4packed(const T4Queue &q, int grid, int block, size_t smem, cudaStream_t s) {
  cudaError_t e = cudaFuncSetAttribute(k_tree4_packed<F, M>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return (int)e;
  k_tree4_packed<F, M><<<grid, block, smem, s>>>(q);
  return (int)cudaGetLastError();
}

template <bool F, int M, int O>
int t4launch(const KParams &p, int grid, int block, size_t smem, cudaStream_t s) {
  cudaError_t e = cudaFuncSetAttribute(k_tree4<F, M, O>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return (int)e;
  k_tree4<F, M, O><<<grid, block, smem, s>>>(p);
  return (int)cudaGetLastError();
}

template <int O>
int t4launch_m(const KParams &p, bool f81, int mask_mode, int grid, int block, size_t smem, cudaStream_t s) {
  if (f81) {
    if (mask_mode == kMaskAuto) return t4launch<true, kMaskAuto, O>(p, grid, block, smem, s);
    if (mask_mode == kMaskGiven) return t4launch<true, kMaskGiven, O>(p, grid, block, smem, s);
    return t4launch<true, kMaskNone, O>(p, grid, block, smem, s);
  }
  if (mask_mode == kMaskAuto) return t4launch<false, kMaskAuto, O>(p, grid, block, smem, s);
  if (mask_mode == kMaskGiven) return t4launch<false, kMaskGiven, O>(p, grid, block, smem, s);
  return t4launch<false, kMaskNone, O>(p, grid, block, smem, s);
}

}  // namespace

int launch_tree4(const KParams &p, bool f81, int mask_mode, int grid, int block, size_t smem,
                 cudaStream_t s) {
  return (p.mode & kModeBranch) ? t4launch_m<kOutBranch>(p, f81, mask_mode, grid, block, smem, s)
                                : t4launch_m<kOutSum>(p, f81, mask_mode, grid, block, smem, s);
}

int launch_tree4_packed(const T4Queue &q, bool f81, int mask_mode, int grid, int block, size_t smem,
                        cudaStream_t s) {
  if (f81) return mask_mode == kMaskAuto ? t4packed<true, kMaskAuto>(q, grid, block, smem, s)
                                         : t4packed<true, kMaskNone>(q, grid, block, smem, s);
  return mask_mode == kMaskAuto ? t4packed<false, kMaskAuto>(q, grid, block, smem, s)
                                : t4packed<false, kMaskNone>(q, grid, block, smem, s);
}

int preload_tree4() {
  cudaFuncAttributes a;
  const void *fns[] = {(const void *)k_tree4<false, kMaskAuto, kOutSum>, (const void *)k_tree4<false, kMaskGiven, kOutSum>,
                       (const void *)k_tree4<false, kMaskNone, kOutSum>, (const void *)k_tree4<true, kMaskAuto, kOutSum>,
                       (const void *)k_tree4<true, kMaskGiven, kOutSum>, (const void *)k_tree4<true, kMaskNone, kOutSum>};
  for (const void *f : fns) {
    const cudaError_t e = cudaFuncGetAttributes(&a, f);
    if (e != cudaSuccess) return (int)e;
  }
  return 0;
}

int launch_tree4_post(const KParams &p, int grid, int block, size_t smem, cudaStream_t s) {
  return t4launch<false, kMaskNone, kOutPost>(p, grid, block, smem, s);
}

}  // namespace subby
