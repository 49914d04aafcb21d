// Thread-per-column kernels for small alphabets (A <= 8).
//
// One thread owns one alignment column and walks the whole tree for it:
//   * inside pass over the postorder schedule (subby/oracle/oracle.py:784-838,
//     subby/jax/pruning.py:94-118),
//   * LogLike and root posterior (oracle.py:831-836, 1571-1595),
//   * outside pass over the same schedule backwards (oracle.py:845-924,
//     subby/jax/outside.py:94-126), fused with
//   * per-branch eigenbasis projection and J-weighted accumulation
//     (oracle.py:966-1044, subby/jax/eigensub.py:53-135) or the F81 closed
//     form (oracle.py:1190-1256, subby/jax/f81_fast.py:7-141),
//   * the Steiner-tree branch mask (oracle.py:1372-1435) as bit flags that
//     ride along with the two passes,
//   * and the back-transform to state counts (oracle.py:1087-1137).
//
// Rescaling: instead of dividing by the max component and adding log(max)
// (reference), every rescale multiplies by an exact power of two 2^-e that
// brings the max into [1, 2) and adds the integer e to the node's exponent.
// All outputs are invariant to the scale factors, so results equal the
// reference's up to FP32 rounding, the exponents sum exactly, and the
// per-branch posterior weight exp(lnD + lnU - lnL) becomes
// 2^(eD + eU - eRoot) / P with one reciprocal per column.
//
// Per-column state that must survive from the inside to the outside pass
// (the child contribution M_n U_n of every internal non-root node, its
// exponent and mask bits) lives in a per-thread scratch slice of global
// memory indexed [slot][thread]; leaves are recomputed from their token.
#include "common.cuh"

namespace subby {
namespace {

constexpr double kLn2 = 0.69314718055994530942;

__device__ __forceinline__ int tok_code(int tok, int A) { return (tok >= 0 && tok < A) ? tok : A; }
__device__ __forceinline__ int tok_ungapped(int tok, int A) { return (tok >= 0 && tok <= A) ? 1 : 0; }

// 2^k as float for k in [-126, 127]; k <= -127 gives +0.
__device__ __forceinline__ float pow2i(int k) {
  k = max(-127, min(127, k));
  return __int_as_float((k + 127) << 23);
}

template <int A>
__device__ __forceinline__ void ldv(float (&o)[A], const float *p) {
  if constexpr (A == 4) {
    float4 t = *reinterpret_cast<const float4 *>(p);
    o[0] = t.x; o[1] = t.y; o[2] = t.z; o[3] = t.w;
  } else if constexpr (A % 2 == 0) {
#pragma unroll
    for (int a = 0; a < A; a += 2) {
      float2 t = *reinterpret_cast<const float2 *>(p + a);
      o[a] = t.x; o[a + 1] = t.y;
    }
  } else {
#pragma unroll
    for (int a = 0; a < A; ++a) o[a] = p[a];
  }
}

template <int A>
__device__ __forceinline__ void stv(float *p, const float (&v)[A]) {
  if constexpr (A == 4) {
    *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
  } else if constexpr (A % 2 == 0) {
#pragma unroll
    for (int a = 0; a < A; a += 2) *reinterpret_cast<float2 *>(p + a) = make_float2(v[a], v[a + 1]);
  } else {
#pragma unroll
    for (int a = 0; a < A; ++a) p[a] = v[a];
  }
}

// Observation likelihood of token code `code` (A = all ones) applied in place.
template <int A>
__device__ __forceinline__ void apply_obs(float (&u)[A], int code) {
  if (code < A) {
#pragma unroll
    for (int a = 0; a < A; ++a) u[a] = (a == code) ? u[a] : 0.f;
  }
}

// Multiply by 2^-e so that max(u) lands in [1, 2); returns e (0 for a zero vector).
template <int A>
__device__ __forceinline__ int rescale(float (&u)[A]) {
  float m = u[0];
#pragma unroll
  for (int a = 1; a < A; ++a) m = fmaxf(m, u[a]);
  if (!(m > 0.f) || !(m < 3.0e38f)) return 0;
  int e = ((__float_as_int(m) >> 23) & 0xff) - 127;
  if (e == -127) {  // subnormal max: rare slow path
    int ee;
    frexpf(m, &ee);
    e = ee - 1;
#pragma unroll
    for (int a = 0; a < A; ++a) u[a] = ldexpf(u[a], -e);
    return e;
  }
  const float s = __int_as_float((127 - e) << 23);
#pragma unroll
  for (int a = 0; a < A; ++a) u[a] *= s;
  return e;
}

template <int A>
struct Acc {
  float c[A][A];   // eigenbasis C_kl (general) or G_ij (F81)
  float h[A];      // F81 only
  float g[A];      // F81 only
  float z;         // F81 only
};

// Branch counts contribution (general eigenbasis path).
template <int A>
__device__ __forceinline__ void branch_eigen(Acc<A> &acc, const float (&D)[A], const float (&ut)[A],
                                             float s, const float *__restrict__ Vd,
                                             const float *__restrict__ Jn) {
  float dt[A];
#pragma unroll
  for (int k = 0; k < A; ++k) {
    float v = 0.f;
#pragma unroll
    for (int a = 0; a < A; ++a) v = fmaf(D[a], Vd[a * A + k], v);
    dt[k] = v * s;
  }
#pragma unroll
  for (int k = 0; k < A; ++k) {
    float jr[A];
    ldv<A>(jr, Jn + k * A);
#pragma unroll
    for (int l = 0; l < A; ++l) acc.c[k][l] = fmaf(dt[k] * jr[l], ut[l], acc.c[k][l]);
  }
}

// Branch counts contribution (F81 closed form, natural basis).
template <int A>
__device__ __forceinline__ void branch_f81(Acc<A> &acc, const float (&D)[A], const float (&U)[A],
                                           float s, const float *__restrict__ pi, float4 abgt) {
  float piU = 0.f, dsum = 0.f;
#pragma unroll
  for (int a = 0; a < A; ++a) {
    piU = fmaf(pi[a], U[a], piU);
    dsum += D[a];
  }
  dsum *= s;
  const float as = abgt.x * s;
  const float bh = abgt.y * piU * s;
  const float bg = abgt.y * dsum;
#pragma unroll
  for (int i = 0; i < A; ++i) {
    const float ai = as * D[i];
#pragma unroll
    for (int j = 0; j < A; ++j) acc.c[i][j] = fmaf(ai, U[j], acc.c[i][j]);
    acc.h[i] = fmaf(bh, D[i], acc.h[i]);
    acc.g[i] = fmaf(bg, U[i], acc.g[i]);
  }
  acc.z = fmaf(abgt.z * dsum, piU, acc.z);
}

template <int A>
__global__ void __launch_bounds__(128) k_small(const KParams P) {
  extern __shared__ __align__(16) float sm[];
  for (int t = 0; t < P.ntab; ++t) {
    const SmemTable tb = P.stab[t];
    for (int i = threadIdx.x; i < tb.n; i += blockDim.x) sm[tb.sofs + i] = P.tab[tb.gofs + i];
  }
  const int4 *steps = P.steps;
  const int4 *slots = P.slots;
  if (P.smem_steps >= 0) {
    int4 *ss = reinterpret_cast<int4 *>(sm + P.smem_steps);
    int4 *sl = reinterpret_cast<int4 *>(sm + P.smem_slots);
    for (int i = threadIdx.x; i < P.nInt; i += blockDim.x) {
      ss[i] = P.steps[i];
      sl[i] = P.slots[i];
    }
    steps = ss;
    slots = sl;
  }
  __syncthreads();

  const float *MT = sm + P.stab[0].sofs;   // host places MT first
  const float *small = sm + P.stab[1].sofs;  // Vu, Vd, Ut, pi, S, V (FP32)
  const float *Vu = small;
  const float *Vd = Vu + A * A;
  const float *Ut = Vd + A * A;
  const float *pi = Ut + (A + 1) * A;
  const float *S32 = pi + A;
  const float *V32 = S32 + A * A;
  const float *MN = (P.ntab > 2) ? sm + P.stab[2].sofs : nullptr;
  const float *Jt = (P.ntab > 3) ? sm + P.stab[3].sofs : nullptr;  // J (eigen) or F81 coefs or ME (grad)

  const int C = P.C;
  const int nthr = gridDim.x * blockDim.x;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const bool counts = (P.mode & (kModeCounts | kModeGrad)) != 0;
  const bool f81 = (P.mode & kModeF81) != 0;
  const bool grad = (P.mode & kModeGrad) != 0;
  const size_t sstride = (size_t)nthr;

  // In gradient mode the eigenbasis accumulator is not reset per column: the
  // cotangent g_c is folded into the branch weight, so acc ends up holding
  // sum_c g_c C_c for this thread's columns.
  Acc<A> acc;
#pragma unroll
  for (int k = 0; k < A; ++k) {
#pragma unroll
    for (int l = 0; l < A; ++l) acc.c[k][l] = 0.f;
    acc.h[k] = 0.f;
    acc.g[k] = 0.f;
  }
  acc.z = 0.f;

  // Warp-uniform column loop: the 32 lanes of a warp always iterate together
  // (lanes past the end recompute the last column and store nothing), so the
  // warp-level reductions of the gradient mode see converged warps.
  const int lane = threadIdx.x & 31;
  for (int c0 = tid - lane; c0 < C; c0 += nthr) {
    const bool valid = c0 + lane < C;
    const int col = valid ? c0 + lane : C - 1;
    const int32_t *alnc = P.aln + col;
    // ------------------------------------------------------------ inside
    float ur[A];
    int eRoot = 0, hRoot = 0, iRoot = 0;
    if (P.root_is_leaf) {
      const int tok = __ldg(alnc);
      const int code = tok_code(tok, A);
#pragma unroll
      for (int a = 0; a < A; ++a) ur[a] = 1.f;
      apply_obs<A>(ur, code);
    }
    for (int i = 0; i < P.nInt; ++i) {
      const int4 st = steps[i];
      const int4 sl = slots[i];
      float cl[A], cr[A];
      int el, er, hl, hr, il, ir;
      if (st.w & kLeafL) {
        const int tok = __ldg(alnc + (size_t)st.y * C);
        ldv<A>(cl, MT + (st.y * (A + 1) + tok_code(tok, A)) * A);
        el = 0; hl = il = tok_ungapped(tok, A);
      } else {
        const size_t o = (size_t)sl.y * sstride + tid;
        ldv<A>(cl, P.scrV + o * A);
        const int w = P.scrW[o * 2];
        el = w >> 2; hl = (w >> 1) & 1; il = w & 1;
      }
      if (st.w & kLeafR) {
        const int tok = __ldg(alnc + (size_t)st.z * C);
        ldv<A>(cr, MT + (st.z * (A + 1) + tok_code(tok, A)) * A);
        er = 0; hr = ir = tok_ungapped(tok, A);
      } else {
        const size_t o = (size_t)sl.z * sstride + tid;
        ldv<A>(cr, P.scrV + o * A);
        const int w = P.scrW[o * 2];
        er = w >> 2; hr = (w >> 1) & 1; ir = w & 1;
      }
      (void)il; (void)ir;
      const int tokp = __ldg(alnc + (size_t)st.x * C);
      float u[A];
#pragma unroll
      for (int a = 0; a < A; ++a) u[a] = cl[a] * cr[a];
      apply_obs<A>(u, tok_code(tokp, A));
      const int eU = el + er + rescale<A>(u);
      const int h = hl | hr, init = hl & hr;
      if (st.w & kRoot) {
#pragma unroll
        for (int a = 0; a < A; ++a) ur[a] = u[a];
        eRoot = eU; hRoot = h; iRoot = init;
      } else {
        const float *mt = MT + st.x * (A + 1) * A;
        float cc[A];
#pragma unroll
        for (int b = 0; b < A; ++b) cc[b] = 0.f;
#pragma unroll
        for (int j = 0; j < A; ++j) {
          float mrow[A];
          ldv<A>(mrow, mt + j * A);
#pragma unroll
          for (int b = 0; b < A; ++b) cc[b] = fmaf(mrow[b], u[j], cc[b]);
        }
        const size_t o = (size_t)sl.x * sstride + tid;
        stv<A>(P.scrV + o * A, cc);
        P.scrW[o * 2] = (eU << 2) | (h << 1) | init;
      }
    }
    (void)hRoot;
    float Pp = 0.f;
#pragma unroll
    for (int a = 0; a < A; ++a) Pp = fmaf(pi[a], ur[a], Pp);
    const double ll = (double)eRoot * kLn2 + (double)logf(Pp);
    if ((P.mode & kModeLogLike) && valid) P.logL[col] = (float)ll;
    const float invP = 1.0f / Pp;
    if ((P.mode & kModeRootProb) && valid) {
#pragma unroll
      for (int a = 0; a < A; ++a) P.rootp[(size_t)a * C + col] = pi[a] * ur[a] * invP;
    }
    if (!counts || P.nInt == 0) {
      if (counts && !grad && valid) {
#pragma unroll
        for (int i = 0; i < A * A; ++i) P.counts[(size_t)i * C + col] = 0.f;
      }
      continue;
    }
    // ------------------------------------------------------------ outside
    if (!grad) {
#pragma unroll
      for (int k = 0; k < A; ++k) {
#pragma unroll
        for (int l = 0; l < A; ++l) acc.c[k][l] = 0.f;
        acc.h[k] = 0.f;
        acc.g[k] = 0.f;
      }
      acc.z = 0.f;
    }
    const float gc = grad ? (valid ? (P.g ? P.g[col] : 1.f) : 0.f) : 1.f;

    // Branch contribution for child n (natural-basis D and U, exponents summed).
    auto branch = [&](int n, const float (&D)[A], const float (&U)[A], int leafcode, int eDU,
                      int active) {
      const float s = active ? gc * invP * pow2i(eDU - eRoot) : 0.f;
      if (f81) {
        const float4 abgt = *reinterpret_cast<const float4 *>(Jt + n * 4);
        branch_f81<A>(acc, D, U, s, pi, abgt);
        return;
      }
      float ut[A];
      if (leafcode >= 0) {
        ldv<A>(ut, Ut + leafcode * A);
      } else {
#pragma unroll
        for (int l = 0; l < A; ++l) {
          float v = 0.f;
#pragma unroll
          for (int b = 0; b < A; ++b) v = fmaf(U[b], Vu[b * A + l], v);
          ut[l] = v;
        }
      }
      if (grad) {
        // distance gradient: s * sum_k D~_k mu_k e^{mu_k t} U~_k (subby/jax/vjp.py:92-112)
        float dt[A];
#pragma unroll
        for (int k = 0; k < A; ++k) {
          float v = 0.f;
#pragma unroll
          for (int a = 0; a < A; ++a) v = fmaf(D[a], Vd[a * A + k], v);
          dt[k] = v * s;
        }
        const float *ME = sm + P.stab[4].sofs + n * A;
        float gt = 0.f;
#pragma unroll
        for (int k = 0; k < A; ++k) gt = fmaf(dt[k] * ME[k], ut[k], gt);
        // warp-reduce then one double atomic per warp into the block partial
        for (int o = 16; o > 0; o >>= 1) gt += __shfl_xor_sync(0xffffffffu, gt, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(&P.grad_t[(size_t)blockIdx.x * P.R + n], (double)gt);
        const float *Jn = Jt + (size_t)n * A * A;
#pragma unroll
        for (int k = 0; k < A; ++k) {
          float jr[A];
          ldv<A>(jr, Jn + k * A);
#pragma unroll
          for (int l = 0; l < A; ++l) acc.c[k][l] = fmaf(dt[k] * jr[l], ut[l], acc.c[k][l]);
        }
        return;
      }
      branch_eigen<A>(acc, D, ut, s, Vd, Jt + (size_t)n * A * A);
    };

    for (int i = P.nInt - 1; i >= 0; --i) {
      const int4 st = steps[i];
      const int4 sl = slots[i];
      float cl[A], cr[A];
      int el, er, hl, hr, il, ir, codel = -1, coder = -1;
      if (st.w & kLeafL) {
        const int tok = __ldg(alnc + (size_t)st.y * C);
        codel = tok_code(tok, A);
        ldv<A>(cl, MT + (st.y * (A + 1) + codel) * A);
        el = 0; hl = il = tok_ungapped(tok, A);
      } else {
        const size_t o = (size_t)sl.y * sstride + tid;
        ldv<A>(cl, P.scrV + o * A);
        const int w = P.scrW[o * 2];
        el = w >> 2; hl = (w >> 1) & 1; il = w & 1;
      }
      if (st.w & kLeafR) {
        const int tok = __ldg(alnc + (size_t)st.z * C);
        coder = tok_code(tok, A);
        ldv<A>(cr, MT + (st.z * (A + 1) + coder) * A);
        er = 0; hr = ir = tok_ungapped(tok, A);
      } else {
        const size_t o = (size_t)sl.z * sstride + tid;
        ldv<A>(cr, P.scrV + o * A);
        const int w = P.scrW[o * 2];
        er = w >> 2; hr = (w >> 1) & 1; ir = w & 1;
      }
      const int codep = tok_code(__ldg(alnc + (size_t)st.x * C), A);
      float O[A];
      int eO, stp;
      if (st.w & kRoot) {
#pragma unroll
        for (int a = 0; a < A; ++a) O[a] = pi[a];
        apply_obs<A>(O, codep);
        eO = 0;
        stp = iRoot;
      } else {
        const size_t o = (size_t)sl.x * sstride + tid;
        float D[A];
        ldv<A>(D, P.scrV + o * A);
        const int wd = P.scrW[o * 2 + 1];
        const int wu = P.scrW[o * 2];
        const int eD = wd >> 2;
        stp = (wd >> 1) & 1;
        const int actp = wd & 1;
        const int eUp = wu >> 2;
        // U_p recomputed from the children contributions (same exponent as the inside pass)
        float U[A];
#pragma unroll
        for (int a = 0; a < A; ++a) U[a] = cl[a] * cr[a];
        apply_obs<A>(U, codep);
        const float us = pow2i(el + er - eUp);
#pragma unroll
        for (int a = 0; a < A; ++a) U[a] *= us;
        branch(st.x, D, U, -1, eD + eUp, actp);
        // O_p = (D_p^T M_p) o L(x_p)
        const float *mn = MN + st.x * A * A;
#pragma unroll
        for (int a = 0; a < A; ++a) O[a] = 0.f;
#pragma unroll
        for (int ii = 0; ii < A; ++ii) {
          float mrow[A];
          ldv<A>(mrow, mn + ii * A);
#pragma unroll
          for (int a = 0; a < A; ++a) O[a] = fmaf(D[ii], mrow[a], O[a]);
        }
        apply_obs<A>(O, codep);
        eO = eD + rescale<A>(O);
      }
      float Dl[A], Dr[A];
#pragma unroll
      for (int a = 0; a < A; ++a) {
        Dl[a] = O[a] * cr[a];
        Dr[a] = O[a] * cl[a];
      }
      const int eDl = eO + er + rescale<A>(Dl);
      const int eDr = eO + el + rescale<A>(Dr);
      const int stl = il | (stp & hl);
      const int str = ir | (stp & hr);
      int actl = 1, actr = 1;
      if (P.mask_mode == kMaskAuto) {
        actl = stl & stp;
        actr = str & stp;
      } else if (P.mask_mode == kMaskGiven) {
        actl = P.mask[(size_t)st.y * C + col] != 0;
        actr = P.mask[(size_t)st.z * C + col] != 0;
      }
      if (st.w & kLeafL) {
        float U[A];
#pragma unroll
        for (int a = 0; a < A; ++a) U[a] = 1.f;
        apply_obs<A>(U, codel);
        branch(st.y, Dl, U, codel, eDl, actl);
      } else {
        const size_t o = (size_t)sl.y * sstride + tid;
        stv<A>(P.scrV + o * A, Dl);
        P.scrW[o * 2 + 1] = (eDl << 2) | (stl << 1) | actl;
      }
      if (st.w & kLeafR) {
        float U[A];
#pragma unroll
        for (int a = 0; a < A; ++a) U[a] = 1.f;
        apply_obs<A>(U, coder);
        branch(st.z, Dr, U, coder, eDr, actr);
      } else {
        const size_t o = (size_t)sl.z * sstride + tid;
        stv<A>(P.scrV + o * A, Dr);
        P.scrW[o * 2 + 1] = (eDr << 2) | (str << 1) | actr;
      }
    }
    if (grad) continue;
    // ------------------------------------------------------------ epilogue
    if (!valid) continue;
    float *out = P.counts + col;
    if (f81) {
      const float mu = P.f81_mu;
#pragma unroll
      for (int i = 0; i < A; ++i)
#pragma unroll
        for (int j = 0; j < A; ++j) {
          const float I = acc.c[i][j] + acc.h[i] + pi[i] * acc.g[j] + pi[i] * acc.z;
          out[(size_t)(i * A + j) * C] = (i == j) ? I : mu * pi[j] * I;
        }
    } else if (P.mode & kModeBT64) {
      const double *V = P.tab64;
      const double *S = P.tab64 + A * A;
      double T[A][A];
#pragma unroll
      for (int k = 0; k < A; ++k)
#pragma unroll
        for (int j = 0; j < A; ++j) {
          double v = 0.0;
#pragma unroll
          for (int l = 0; l < A; ++l) v = fma((double)acc.c[k][l], __ldg(V + j * A + l), v);
          T[k][j] = v;
        }
#pragma unroll
      for (int i = 0; i < A; ++i)
#pragma unroll
        for (int j = 0; j < A; ++j) {
          double v = 0.0;
#pragma unroll
          for (int k = 0; k < A; ++k) v = fma(__ldg(V + i * A + k), T[k][j], v);
          out[(size_t)(i * A + j) * C] = (float)((i == j) ? v : __ldg(S + i * A + j) * v);
        }
    } else {
      float T[A][A];
#pragma unroll
      for (int k = 0; k < A; ++k)
#pragma unroll
        for (int j = 0; j < A; ++j) {
          float v = 0.f;
#pragma unroll
          for (int l = 0; l < A; ++l) v = fmaf(acc.c[k][l], V32[j * A + l], v);
          T[k][j] = v;
        }
#pragma unroll
      for (int i = 0; i < A; ++i)
#pragma unroll
        for (int j = 0; j < A; ++j) {
          float v = 0.f;
#pragma unroll
          for (int k = 0; k < A; ++k) v = fmaf(V32[i * A + k], T[k][j], v);
          out[(size_t)(i * A + j) * C] = (i == j) ? v : S32[i * A + j] * v;
        }
    }
  }
  if (grad) {
    // block-reduce sum_c g_c C_c into this block's partial (FP64 atomics in global)
#pragma unroll
    for (int k = 0; k < A; ++k)
#pragma unroll
      for (int l = 0; l < A; ++l) {
        float v = acc.c[k][l];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0)
          atomicAdd(&P.grad_C[((size_t)blockIdx.x * A + k) * A + l], (double)v);
      }
  }
}

template <int A>
int launch_t(const KParams &p, int grid, int block, size_t smem, cudaStream_t s) {
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k_small<A>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return (int)e;
  }
  k_small<A><<<grid, block, smem, s>>>(p);
  return (int)cudaGetLastError();
}

}  // namespace

bool small_supported(int A) { return A >= 2 && A <= 8; }
int small_block() { return 128; }

int launch_small(const KParams &p, int A, int grid, int block, size_t smem, cudaStream_t s) {
  switch (A) {
    case 2: return launch_t<2>(p, grid, block, smem, s);
    case 3: return launch_t<3>(p, grid, block, smem, s);
    case 4: return launch_t<4>(p, grid, block, smem, s);
    case 5: return launch_t<5>(p, grid, block, smem, s);
    case 6: return launch_t<6>(p, grid, block, smem, s);
    case 7: return launch_t<7>(p, grid, block, smem, s);
    case 8: return launch_t<8>(p, grid, block, smem, s);
    default: return -1;
  }
}

}  // namespace subby
