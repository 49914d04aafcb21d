// Warp-per-column kernels for larger alphabets (A = 16, 20, 32, 64).
//
// Same algorithm as k_small.cu (inside pass, LogLike/root posterior, outside
// pass fused with eigenbasis or F81 accumulation, Steiner mask bits,
// back-transform; subby/oracle/oracle.py:747-1256, 1372-1435), but one warp
// owns one column and each lane owns NPL = ceil(A/32) states of every vector.
// Matrix-vector products broadcast the input vector through a per-warp
// shared-memory line and read the (A x A) table rows coalesced from
// L1/L2-resident global memory.  The eigenbasis accumulator C_kl lives in
// registers with lane k owning row k.  Power-of-two rescaling as in
// k_small.cu.
#include "common.cuh"

namespace subby {
namespace {

constexpr double kLn2w = 0.69314718055994530942;

__device__ __forceinline__ int wtok_code(int tok, int A) { return (tok >= 0 && tok < A) ? tok : A; }
__device__ __forceinline__ int wtok_ungapped(int tok, int A) { return (tok >= 0 && tok <= A) ? 1 : 0; }
__device__ __forceinline__ float wpow2i(int k) {
  k = max(-127, min(127, k));
  return __int_as_float((k + 127) << 23);
}

template <int A>
struct WV {
  static constexpr int NPL = (A + 31) / 32;
  float x[NPL];
};

template <int A>
__device__ __forceinline__ void wload(WV<A> &v, const float *p, int lane) {
#pragma unroll
  for (int m = 0; m < WV<A>::NPL; ++m) {
    const int a = lane + 32 * m;
    v.x[m] = (a < A) ? p[a] : 0.f;
  }
}
template <int A>
__device__ __forceinline__ void wstore(float *p, const WV<A> &v, int lane) {
#pragma unroll
  for (int m = 0; m < WV<A>::NPL; ++m) {
    const int a = lane + 32 * m;
    if (a < A) p[a] = v.x[m];
  }
}
template <int A>
__device__ __forceinline__ void wobs(WV<A> &v, int code, int lane) {
  if (code < A) {
#pragma unroll
    for (int m = 0; m < WV<A>::NPL; ++m) v.x[m] = (lane + 32 * m == code) ? v.x[m] : 0.f;
  }
}
__device__ __forceinline__ float wmax(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ float wsum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
template <int A>
__device__ __forceinline__ int wrescale(WV<A> &v) {
  float m = v.x[0];
#pragma unroll
  for (int i = 1; i < WV<A>::NPL; ++i) m = fmaxf(m, v.x[i]);
  m = wmax(m);
  if (!(m > 0.f) || !(m < 3.0e38f)) return 0;
  int e = ((__float_as_int(m) >> 23) & 0xff) - 127;
  if (e == -127) {
    int ee;
    frexpf(m, &ee);
    e = ee - 1;
#pragma unroll
    for (int i = 0; i < WV<A>::NPL; ++i) v.x[i] = ldexpf(v.x[i], -e);
    return e;
  }
  const float s = __int_as_float((127 - e) << 23);
#pragma unroll
  for (int i = 0; i < WV<A>::NPL; ++i) v.x[i] *= s;
  return e;
}
// y_a = sum_j in_j T[j*A + a]; `in` is broadcast through the warp line `buf`.
template <int A>
__device__ __forceinline__ void wmatvec(WV<A> &y, const WV<A> &in, const float *__restrict__ T,
                                        float *buf, int lane) {
  __syncwarp();
  wstore<A>(buf, in, lane);
  __syncwarp();
#pragma unroll
  for (int m = 0; m < WV<A>::NPL; ++m) y.x[m] = 0.f;
#pragma unroll 4
  for (int j = 0; j < A; ++j) {
    const float w = buf[j];
#pragma unroll
    for (int m = 0; m < WV<A>::NPL; ++m) {
      const int a = lane + 32 * m;
      if (a < A) y.x[m] = fmaf(w, __ldg(T + j * A + a), y.x[m]);
    }
  }
}

template <int A>
__global__ void __launch_bounds__(128) k_warp(const KParams P) {
  constexpr int NPL = WV<A>::NPL;
  constexpr int LINE = (A + 3) & ~3;
  constexpr int TSTR = A + 1;
  extern __shared__ __align__(16) float smw[];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int wpb = blockDim.x >> 5;
  const int nw = gridDim.x * wpb;
  const int wid = blockIdx.x * wpb + warp;
  float *buf = smw + warp * (LINE + A * TSTR);
  float *tbuf = buf + LINE;

  const float *MT = P.tab + P.off.MT;
  const float *MN = P.tab + P.off.MN;
  const float *JT = P.tab + P.off.JT;
  const float *F8 = P.tab + P.off.F81;
  const float *Vu = P.tab + P.off.Vu;
  const float *Vd = P.tab + P.off.Vd;
  const float *Ut = P.tab + P.off.Ut;
  const float *pi = P.tab + P.off.pi;
  const float *V32 = P.tab + P.off.V;
  const float *S32 = P.tab + P.off.S;
  const float *ME = P.tab + P.off.ME;

  const int C = P.C;
  const bool counts = (P.mode & (kModeCounts | kModeGrad)) != 0;
  const bool f81 = (P.mode & kModeF81) != 0;
  const bool grad = (P.mode & kModeGrad) != 0;
  const size_t sstride = (size_t)nw;

  WV<A> piv;
  wload<A>(piv, pi, lane);

  float acc[NPL][A];   // eigen C rows (k = lane + 32m) or F81 G rows
  float hacc[NPL], gacc[NPL], zacc = 0.f;
#pragma unroll
  for (int m = 0; m < NPL; ++m) {
#pragma unroll
    for (int l = 0; l < A; ++l) acc[m][l] = 0.f;
    hacc[m] = 0.f;
    gacc[m] = 0.f;
  }

  for (int col = wid; col < C; col += nw) {
    const int32_t *alnc = P.aln + col;
    WV<A> ur;
    int eRoot = 0, iRoot = 0;
    if (P.root_is_leaf) {
#pragma unroll
      for (int m = 0; m < NPL; ++m) ur.x[m] = 1.f;
      wobs<A>(ur, wtok_code(__ldg(alnc), A), lane);
    }
    // ------------------------------------------------------------ inside
    for (int i = 0; i < P.nInt; ++i) {
      const int4 st = P.steps[i];
      const int4 sl = P.slots[i];
      WV<A> cl, cr;
      int el, er, hl, hr;
      if (st.w & kLeafL) {
        const int tok = __ldg(alnc + (size_t)st.y * C);
        wload<A>(cl, MT + ((size_t)st.y * (A + 1) + wtok_code(tok, A)) * A, lane);
        el = 0; hl = wtok_ungapped(tok, A);
      } else {
        const size_t o = (size_t)sl.y * sstride + wid;
        wload<A>(cl, P.scrV + o * A, lane);
        const int w = P.scrW[o * 2];
        el = w >> 2; hl = (w >> 1) & 1;
      }
      if (st.w & kLeafR) {
        const int tok = __ldg(alnc + (size_t)st.z * C);
        wload<A>(cr, MT + ((size_t)st.z * (A + 1) + wtok_code(tok, A)) * A, lane);
        er = 0; hr = wtok_ungapped(tok, A);
      } else {
        const size_t o = (size_t)sl.z * sstride + wid;
        wload<A>(cr, P.scrV + o * A, lane);
        const int w = P.scrW[o * 2];
        er = w >> 2; hr = (w >> 1) & 1;
      }
      WV<A> u;
#pragma unroll
      for (int m = 0; m < NPL; ++m) u.x[m] = cl.x[m] * cr.x[m];
      wobs<A>(u, wtok_code(__ldg(alnc + (size_t)st.x * C), A), lane);
      const int eU = el + er + wrescale<A>(u);
      const int h = hl | hr, init = hl & hr;
      if (st.w & kRoot) {
        ur = u;
        eRoot = eU;
        iRoot = init;
      } else {
        WV<A> cc;
        wmatvec<A>(cc, u, MT + (size_t)st.x * (A + 1) * A, buf, lane);
        const size_t o = (size_t)sl.x * sstride + wid;
        wstore<A>(P.scrV + o * A, cc, lane);
        if (lane == 0) P.scrW[o * 2] = (eU << 2) | (h << 1) | init;
      }
    }
    float pp = 0.f;
#pragma unroll
    for (int m = 0; m < NPL; ++m) pp = fmaf(piv.x[m], ur.x[m], pp);
    const float Pp = wsum(pp);
    if ((P.mode & kModeLogLike) && lane == 0)
      P.logL[col] = (float)((double)eRoot * kLn2w + (double)logf(Pp));
    const float invP = 1.0f / Pp;
    if (P.mode & kModeRootProb) {
#pragma unroll
      for (int m = 0; m < NPL; ++m) {
        const int a = lane + 32 * m;
        if (a < A) P.rootp[(size_t)a * C + col] = piv.x[m] * ur.x[m] * invP;
      }
    }
    if (!counts) continue;
    if (P.nInt == 0) {
      if (!grad) {
        for (int i = lane; i < A * A; i += 32) P.counts[(size_t)i * C + col] = 0.f;
      }
      continue;
    }
    // ------------------------------------------------------------ outside
    if (!grad) {
#pragma unroll
      for (int m = 0; m < NPL; ++m) {
#pragma unroll
        for (int l = 0; l < A; ++l) acc[m][l] = 0.f;
        hacc[m] = 0.f;
        gacc[m] = 0.f;
      }
      zacc = 0.f;
    }
    const float gc = grad ? (P.g ? P.g[col] : 1.f) : 1.f;

    auto branch = [&](int n, const WV<A> &D, const WV<A> &U, int leafcode, int eDU, int active) {
      const float s = active ? gc * invP * wpow2i(eDU - eRoot) : 0.f;
      if (f81) {
        const float4 abgt = *reinterpret_cast<const float4 *>(F8 + n * 4);
        float pu = 0.f, ds = 0.f;
#pragma unroll
        for (int m = 0; m < NPL; ++m) {
          pu = fmaf(piv.x[m], U.x[m], pu);
          ds += D.x[m];
        }
        const float piU = wsum(pu);
        const float dsum = wsum(ds) * s;
        const float as = abgt.x * s, bh = abgt.y * piU * s, bg = abgt.y * dsum;
        __syncwarp();
        wstore<A>(buf, U, lane);
        __syncwarp();
#pragma unroll
        for (int m = 0; m < NPL; ++m) {
          const float ai = as * D.x[m];
#pragma unroll
          for (int j = 0; j < A; ++j) acc[m][j] = fmaf(ai, buf[j], acc[m][j]);
          hacc[m] = fmaf(bh, D.x[m], hacc[m]);
          gacc[m] = fmaf(bg, U.x[m], gacc[m]);
        }
        zacc = fmaf(abgt.z * dsum, piU, zacc);
        return;
      }
      WV<A> ut, dt;
      if (leafcode >= 0) {
        wload<A>(ut, Ut + leafcode * A, lane);
      } else {
        wmatvec<A>(ut, U, Vu, buf, lane);
      }
      wmatvec<A>(dt, D, Vd, buf, lane);
#pragma unroll
      for (int m = 0; m < NPL; ++m) dt.x[m] *= s;
      if (grad) {
        float gt = 0.f;
#pragma unroll
        for (int m = 0; m < NPL; ++m) {
          const int k = lane + 32 * m;
          if (k < A) gt = fmaf(dt.x[m] * __ldg(ME + (size_t)n * A + k), ut.x[m], gt);
        }
        gt = wsum(gt);
        if (lane == 0) atomicAdd(&P.grad_t[(size_t)blockIdx.x * P.R + n], (double)gt);
      }
      __syncwarp();
      wstore<A>(buf, ut, lane);
      __syncwarp();
      const float *Jn = JT + (size_t)n * A * A;
#pragma unroll
      for (int l = 0; l < A; ++l) {
        const float w = buf[l];
#pragma unroll
        for (int m = 0; m < NPL; ++m) {
          const int k = lane + 32 * m;
          if (k < A) acc[m][l] = fmaf(dt.x[m] * w, __ldg(Jn + l * A + k), acc[m][l]);
        }
      }
    };

    for (int i = P.nInt - 1; i >= 0; --i) {
      const int4 st = P.steps[i];
      const int4 sl = P.slots[i];
      WV<A> cl, cr;
      int el, er, hl, hr, il, ir, codel = -1, coder = -1;
      if (st.w & kLeafL) {
        const int tok = __ldg(alnc + (size_t)st.y * C);
        codel = wtok_code(tok, A);
        wload<A>(cl, MT + ((size_t)st.y * (A + 1) + codel) * A, lane);
        el = 0; hl = il = wtok_ungapped(tok, A);
      } else {
        const size_t o = (size_t)sl.y * sstride + wid;
        wload<A>(cl, P.scrV + o * A, lane);
        const int w = P.scrW[o * 2];
        el = w >> 2; hl = (w >> 1) & 1; il = w & 1;
      }
      if (st.w & kLeafR) {
        const int tok = __ldg(alnc + (size_t)st.z * C);
        coder = wtok_code(tok, A);
        wload<A>(cr, MT + ((size_t)st.z * (A + 1) + coder) * A, lane);
        er = 0; hr = ir = wtok_ungapped(tok, A);
      } else {
        const size_t o = (size_t)sl.z * sstride + wid;
        wload<A>(cr, P.scrV + o * A, lane);
        const int w = P.scrW[o * 2];
        er = w >> 2; hr = (w >> 1) & 1; ir = w & 1;
      }
      const int codep = wtok_code(__ldg(alnc + (size_t)st.x * C), A);
      WV<A> O;
      int eO, stp;
      if (st.w & kRoot) {
        O = piv;
        wobs<A>(O, codep, lane);
        eO = 0;
        stp = iRoot;
      } else {
        const size_t o = (size_t)sl.x * sstride + wid;
        WV<A> D;
        wload<A>(D, P.scrV + o * A, lane);
        const int wd = P.scrW[o * 2 + 1];
        const int wu = P.scrW[o * 2];
        const int eD = wd >> 2;
        stp = (wd >> 1) & 1;
        const int actp = wd & 1;
        const int eUp = wu >> 2;
        WV<A> U;
#pragma unroll
        for (int m = 0; m < NPL; ++m) U.x[m] = cl.x[m] * cr.x[m];
        wobs<A>(U, codep, lane);
        const float us = wpow2i(el + er - eUp);
#pragma unroll
        for (int m = 0; m < NPL; ++m) U.x[m] *= us;
        branch(st.x, D, U, -1, eD + eUp, actp);
        wmatvec<A>(O, D, MN + (size_t)st.x * A * A, buf, lane);
        wobs<A>(O, codep, lane);
        eO = eD + wrescale<A>(O);
      }
      WV<A> Dl, Dr;
#pragma unroll
      for (int m = 0; m < NPL; ++m) {
        Dl.x[m] = O.x[m] * cr.x[m];
        Dr.x[m] = O.x[m] * cl.x[m];
      }
      const int eDl = eO + er + wrescale<A>(Dl);
      const int eDr = eO + el + wrescale<A>(Dr);
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
        WV<A> U;
#pragma unroll
        for (int m = 0; m < NPL; ++m) U.x[m] = 1.f;
        wobs<A>(U, codel, lane);
        branch(st.y, Dl, U, codel, eDl, actl);
      } else {
        const size_t o = (size_t)sl.y * sstride + wid;
        wstore<A>(P.scrV + o * A, Dl, lane);
        if (lane == 0) P.scrW[o * 2 + 1] = (eDl << 2) | (stl << 1) | actl;
      }
      if (st.w & kLeafR) {
        WV<A> U;
#pragma unroll
        for (int m = 0; m < NPL; ++m) U.x[m] = 1.f;
        wobs<A>(U, coder, lane);
        branch(st.z, Dr, U, coder, eDr, actr);
      } else {
        const size_t o = (size_t)sl.z * sstride + wid;
        wstore<A>(P.scrV + o * A, Dr, lane);
        if (lane == 0) P.scrW[o * 2 + 1] = (eDr << 2) | (str << 1) | actr;
      }
    }
    if (grad) continue;
    // ------------------------------------------------------------ epilogue
    if (f81) {
      const float mu = P.f81_mu;
      __syncwarp();
#pragma unroll
      for (int m = 0; m < NPL; ++m) {
        const int a = lane + 32 * m;
        if (a < A) buf[a] = gacc[m];
      }
      __syncwarp();
#pragma unroll
      for (int m = 0; m < NPL; ++m) {
        const int i = lane + 32 * m;
        if (i >= A) continue;
        const float pii = piv.x[m];
#pragma unroll 4
        for (int j = 0; j < A; ++j) {
          const float I = acc[m][j] + hacc[m] + pii * buf[j] + pii * zacc;
          P.counts[(size_t)(i * A + j) * C + col] = (i == j) ? I : mu * __ldg(pi + j) * I;
        }
      }
      continue;
    }
    // back-transform: VCV = V C V^T (FP32), counts = diag VCV, S o VCV off-diagonal
    __syncwarp();
#pragma unroll
    for (int m = 0; m < NPL; ++m) {
      const int k = lane + 32 * m;
      if (k < A) {
#pragma unroll
        for (int l = 0; l < A; ++l) tbuf[k * TSTR + l] = acc[m][l];
      }
    }
    __syncwarp();
    // T_kj = sum_l C_kl V_jl  (rows k owned by this lane), written back over C
    float trow[NPL][A];
#pragma unroll
    for (int m = 0; m < NPL; ++m) {
      const int k = lane + 32 * m;
#pragma unroll
      for (int j = 0; j < A; ++j) trow[m][j] = 0.f;
      if (k < A) {
        for (int l = 0; l < A; ++l) {
          const float c = tbuf[k * TSTR + l];
#pragma unroll
          for (int j = 0; j < A; ++j) trow[m][j] = fmaf(c, __ldg(V32 + j * A + l), trow[m][j]);
        }
      }
    }
    __syncwarp();
#pragma unroll
    for (int m = 0; m < NPL; ++m) {
      const int k = lane + 32 * m;
      if (k < A) {
#pragma unroll
        for (int j = 0; j < A; ++j) tbuf[k * TSTR + j] = trow[m][j];
      }
    }
    __syncwarp();
#pragma unroll
    for (int m = 0; m < NPL; ++m) {
      const int i = lane + 32 * m;
      if (i >= A) continue;
      float vrow[A];
#pragma unroll
      for (int j = 0; j < A; ++j) vrow[j] = 0.f;
      for (int k = 0; k < A; ++k) {
        const float vik = __ldg(V32 + i * A + k);
#pragma unroll
        for (int j = 0; j < A; ++j) vrow[j] = fmaf(vik, tbuf[k * TSTR + j], vrow[j]);
      }
#pragma unroll
      for (int j = 0; j < A; ++j)
        P.counts[(size_t)(i * A + j) * C + col] = (i == j) ? vrow[j] : __ldg(S32 + i * A + j) * vrow[j];
    }
  }
  if (grad) {
#pragma unroll
    for (int m = 0; m < NPL; ++m) {
      const int k = lane + 32 * m;
      if (k >= A) continue;
#pragma unroll
      for (int l = 0; l < A; ++l)
        atomicAdd(&P.grad_C[((size_t)blockIdx.x * A + k) * A + l], (double)acc[m][l]);
    }
  }
}

template <int A>
int wlaunch_t(const KParams &p, int grid, int block, size_t smem, cudaStream_t s) {
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k_warp<A>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return (int)e;
  }
  k_warp<A><<<grid, block, smem, s>>>(p);
  return (int)cudaGetLastError();
}

}  // namespace

bool warp_supported(int A) { return A == 16 || A == 20 || A == 32 || A == 64; }
int warp_block() { return 128; }
size_t warp_smem_per_warp(int A) {
  const int line = (A + 3) & ~3;
  return (size_t)(line + A * (A + 1)) * sizeof(float);
}

int launch_warp(const KParams &p, int A, int grid, int block, size_t smem, cudaStream_t s) {
  switch (A) {
    case 16: return wlaunch_t<16>(p, grid, block, smem, s);
    case 20: return wlaunch_t<20>(p, grid, block, smem, s);
    case 32: return wlaunch_t<32>(p, grid, block, smem, s);
    case 64: return wlaunch_t<64>(p, grid, block, smem, s);
    default: return -1;
  }
}

}  // namespace subby
