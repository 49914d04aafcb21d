// Large-alphabet path (A = 16, 20, 32, 64): tree walk + staged accumulation.
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
// Kernel 2, k_acc<A, F81>: per group of G columns, accumulates
// C_kl += D~_k J_kl U~_l over all branches (oracle.py:1010-1044) — or the
// F81 rank-3 terms — with 4 x 4 (k, l) register blocks, J rows and staged
// vectors double-buffered through shared memory, then back-transforms
// V C V^T (oracle.py:1087-1137) through shared memory and writes counts.
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

template <int A>
struct Walk {
  static constexpr int H = Geo<A>::H;
  static constexpr int S = Geo<A>::S;
  int c, h, warp;
  float *xch;     // shared exchange buffer: [2][32 states][128 cols] floats
  int *xmax;      // shared [2][128] ints (exponent-field exchange)

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
  // y_b = sum_j T[j][b] x_j over all A inputs j (T rows contiguous, stride A)
  __device__ __forceinline__ void matvec(BV<A> &y, const BV<A> &x, const float *__restrict__ T) const {
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

template <int A, int MODE>  // MODE: 0 inside only, 1 eigen staging, 2 F81 staging
__global__ void __launch_bounds__(128 * Geo<A>::H, 1) k_walk(const KParams P, float *__restrict__ stage_a,
                                                              float *__restrict__ stage_b, int c_base,
                                                              int c_count) {
  constexpr int S = Geo<A>::S;
  __shared__ __align__(16) float s_xch[Geo<A>::H == 2 ? 2 * 32 * kTile : 4];
  __shared__ int s_xmax[2 * kTile];
  Walk<A> wk;
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
  const int4 *prog = P.prog;
  const int C = P.C;
  const size_t tile_slots = (size_t)P.nslots * kTile;
  float *svec = P.scrV + (size_t)blockIdx.x * tile_slots * A;  // [slot][c][A]
  int *sword = P.scrW + (size_t)blockIdx.x * tile_slots;       // [slot][c]
  BV<A> piv;
  wk.ld(piv, pig + 32 * h);

  const int ntiles = (c_count + kTile - 1) / kTile;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int cc0 = tile * kTile + cl;              // column within the chunk
    const bool valid = cc0 < c_count;
    const int col = c_base + (valid ? cc0 : c_count - 1);
    const int32_t *alnc = P.aln + col;
    auto tok = [&](int n) { return __ldg(alnc + (size_t)n * C); };
    auto slotv = [&](int s) { return svec + ((size_t)s * kTile + cl) * A + 32 * h; };
    auto slotw = [&](int s) -> int & { return sword[(size_t)s * kTile + cl]; };
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
      wk.matvec(o.cc, u, MT + (size_t)n * (A + 1) * A);
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
        if (s1.y == -2) derive(nl, u, k0, k1, cd, s1.x, s1, s3.x, s3.y);
        else basic(nl, s1.x, s1.y);
        if (s2.y == -2) derive(nr, u, k0, k1, cd, s2.x, s2, s3.z, s3.w);
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
        wk.matvec(cc, u, MT + (size_t)s0.x * (A + 1) * A);
        wk.st(slotv(s0.y), cc);
        if (h == 0) slotw(s0.y) = (eU << 2) | (hh << 1) | init;
      }
    }
    // P = pi . U_root (combined over the pair)
    float pp = 0.f;
#pragma unroll
    for (int q = 0; q < S; ++q) pp = fmaf(piv.v[q], ur.v[q], pp);
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
      for (int q = 0; q < S; ++q) P.rootp[(size_t)(32 * h + q) * C + col] = piv.v[q] * ur.v[q] * invP;
    }
    if (MODE == 0 || P.nsteps == 0) continue;

    // ---------------------------------------------------------------- outside
    // stage the two vectors of the branch above node n for column cc0
    auto emit = [&](int n, const BV<A> &D, const BV<A> &U, int leafcode, int eDU, int active) {
      float s = invP * __int_as_float((max(-127, min(127, eDU - eRoot)) + 127) << 23);
      s = active ? s : 0.f;
      float *pa = stage_a + ((size_t)(n - 1) * c_count + (valid ? cc0 : c_count - 1)) * A + 32 * h;
      float *pb = stage_b + ((size_t)(n - 1) * c_count + (valid ? cc0 : c_count - 1)) * A + 32 * h;
      if (MODE == 2) {
        BV<A> Ds;
#pragma unroll
        for (int q = 0; q < S; ++q) Ds.v[q] = D.v[q] * s;
        if (valid) {
          wk.st(pa, Ds);
          wk.st(pb, U);
        }
        return;
      }
      BV<A> Ds, dt, ut;
#pragma unroll
      for (int q = 0; q < S; ++q) Ds.v[q] = D.v[q] * s;
      wk.matvec(dt, Ds, Vd);
      if (leafcode >= 0) wk.ld(ut, Ut + leafcode * A + 32 * h);
      else wk.matvec(ut, U, Vu);
      if (valid) {
        wk.st(pa, dt);
        wk.st(pb, ut);
      }
    };
    auto act_of = [&](int n, int stn, int stpar) -> int {
      if (P.mask_mode == kMaskAuto) return stn & stpar;
      if (P.mask_mode == kMaskGiven) return P.mask[(size_t)n * C + col] != 0;
      return 1;
    };
    for (int i = P.nsteps - 1; i >= 0; --i) {
      const int4 s0 = prog[4 * i], s1 = prog[4 * i + 1], s2 = prog[4 * i + 2], s3 = prog[4 * i + 3];
      BN<A> nl, nr, k[4];
      BV<A> du[2];
      int dcode[2] = {-1, -1};
      if (s1.y == -2) derive(nl, du[0], k[0], k[1], dcode[0], s1.x, s1, s3.x, s3.y);
      else basic(nl, s1.x, s1.y);
      if (s2.y == -2) derive(nr, du[1], k[2], k[3], dcode[1], s2.x, s2, s3.z, s3.w);
      else basic(nr, s2.x, s2.y);
      const int codep = btcode(tok(s0.x), A);
      BV<A> O;
      int eO, stp;
      if (s0.z) {
        O = piv;
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
        emit(s0.x, D, U, -1, eD + eUp, actp);
        wk.matvec(O, D, MN + (size_t)s0.x * A * A);
        wk.obs(O, codep);
        eO = eD + wk.rescale(O);
      }
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
          BV<A> U;
          wk.fill(U, 1.f);
          wk.obs(U, me.code);
          emit(sc.x, Dc, U, me.code, eDc, actc);
        } else if (sc.y >= 0) {
          __syncwarp();
          wk.st(slotv(sc.y), Dc);
          if (h == 0) slotw(sc.y) = (eDc << 2) | (stc << 1) | actc;
        } else {
          emit(sc.x, Dc, du[side], -1, eDc + me.e, actc);
          BV<A> Oc;
          wk.matvec(Oc, Dc, MN + (size_t)sc.x * A * A);
          wk.obs(Oc, dcode[side]);
          const int eOc = eDc + wk.rescale(Oc);
          const int gks[2] = {side ? s3.z : s3.x, side ? s3.w : s3.y};
          const int gn[2] = {sc.z, sc.w};
#pragma unroll
          for (int gs = 0; gs < 2; ++gs) {
            const BN<A> &g = k[2 * side + gs];
            const BN<A> &gsib = k[2 * side + 1 - gs];
            BV<A> Dg;
#pragma unroll
            for (int q = 0; q < S; ++q) Dg.v[q] = Oc.v[q] * gsib.cc.v[q];
            const int eDg = eOc + gsib.e;
            const int stg = g.init | (stc & g.hh);
            const int actg = act_of(gn[gs], stg, stc);
            if (gks[gs] == -1) {
              BV<A> U;
              wk.fill(U, 1.f);
              wk.obs(U, g.code);
              emit(gn[gs], Dg, U, g.code, eDg, actg);
            } else {
              wk.st(slotv(gks[gs]), Dg);
              if (h == 0) slotw(gks[gs]) = (eDg << 2) | (stg << 1) | actg;
            }
          }
        }
      }
    }
  }
}

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

template <int A, bool F81>
__global__ void __launch_bounds__(256, 1) k_acc(const KParams P, const float *__restrict__ stage_a,
                                                 const float *__restrict__ stage_b, int c_base, int c_count) {
  using Gm = AccGeo<A>;
  constexpr int G = Gm::G;
  extern __shared__ __align__(16) float sm[];
  // double-buffered stage: J_n (A*A) + a (G*A) + b (G*A); later reused for C / T
  float *buf[2] = {sm, sm + A * A + 2 * G * A};
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

  for (int gi = blockIdx.x; gi < ngroups; gi += gridDim.x) {
    const int g0 = gi * G;                       // first column (chunk-relative)
    const int gcols = min(G, c_count - g0);
    float acc[16][8];
    float hv[4][8], gv[4][8], zv[8];
#pragma unroll
    for (int a = 0; a < 16; ++a)
#pragma unroll
      for (int q = 0; q < 8; ++q) acc[a][q] = 0.f;
    if (F81) {
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int q = 0; q < 8; ++q) hv[a][q] = gv[a][q] = 0.f;
#pragma unroll
      for (int q = 0; q < 8; ++q) zv[q] = 0.f;
    }
    auto load = [&](int n, float *dst) {
      // J_n (eigen) and the staged vectors of branch n for this group's columns
      if (!F81)
        for (int i = t; i < A * A / 4; i += blockDim.x)
          reinterpret_cast<float4 *>(dst)[i] = __ldg(reinterpret_cast<const float4 *>(J + (size_t)(n + 1) * A * A) + i);
      const size_t off = ((size_t)n * c_count + g0) * A;
      float *da = dst + A * A, *db = dst + A * A + G * A;
      for (int i = t; i < G * A / 4; i += blockDim.x) {
        const bool in = i * 4 < gcols * A;
        reinterpret_cast<float4 *>(da)[i] = in ? __ldg(reinterpret_cast<const float4 *>(stage_a + off) + i)
                                              : make_float4(0.f, 0.f, 0.f, 0.f);
        reinterpret_cast<float4 *>(db)[i] = in ? __ldg(reinterpret_cast<const float4 *>(stage_b + off) + i)
                                              : make_float4(0.f, 0.f, 0.f, 0.f);
      }
    };
    load(0, buf[0]);
    __syncthreads();
    float *scal = sm + 2 * (A * A + 2 * G * A);  // F81: piU, Dsum per column
    for (int n = 0; n < nbr; ++n) {
      float *cur = buf[n & 1];
      if (n + 1 < nbr) load(n + 1, buf[(n + 1) & 1]);
      if (F81) {
        if (t < G) {
          const float *Ds = cur + A * A + t * A, *U = cur + A * A + G * A + t * A;
          float piU = 0.f, dsum = 0.f;
          for (int a = 0; a < A; ++a) {
            piU = fmaf(__ldg(pig + a), U[a], piU);
            dsum += Ds[a];
          }
          scal[2 * t] = piU;
          scal[2 * t + 1] = dsum;
        }
        __syncthreads();
      }
      if (active) {
        const float *da = cur + A * A, *db = cur + A * A + G * A;
        if (!F81) {
          float jb[4][4];
#pragma unroll
          for (int a = 0; a < 4; ++a) {
            const float4 r = *reinterpret_cast<const float4 *>(cur + (k0 + a) * A + l0);
            jb[a][0] = r.x, jb[a][1] = r.y, jb[a][2] = r.z, jb[a][3] = r.w;
          }
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            const int cc = grp * 8 + q;
            const float4 d = *reinterpret_cast<const float4 *>(da + cc * A + k0);
            const float4 u = *reinterpret_cast<const float4 *>(db + cc * A + l0);
            const float dk[4] = {d.x, d.y, d.z, d.w}, ul[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
              for (int b = 0; b < 4; ++b) acc[a * 4 + b][q] = fmaf(dk[a] * jb[a][b], ul[b], acc[a * 4 + b][q]);
          }
        } else {
          const float4 abg = __ldg(reinterpret_cast<const float4 *>(F8) + n + 1);
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            const int cc = grp * 8 + q;
            const float *Ds = da + cc * A, *U = db + cc * A;
            const float piU = scal[2 * cc], dsum = scal[2 * cc + 1];
            const float4 d = *reinterpret_cast<const float4 *>(Ds + k0);
            const float4 u = *reinterpret_cast<const float4 *>(U + l0);
            const float dk[4] = {d.x, d.y, d.z, d.w}, ul[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
            for (int a = 0; a < 4; ++a) {
#pragma unroll
              for (int b = 0; b < 4; ++b) acc[a * 4 + b][q] = fmaf(abg.x * dk[a], ul[b], acc[a * 4 + b][q]);
              hv[a][q] = fmaf(abg.y * piU, dk[a], hv[a][q]);
              gv[a][q] = fmaf(abg.y * dsum, ul[a], gv[a][q]);
            }
            zv[q] = fmaf(abg.z * dsum, piU, zv[q]);
          }
        }
      }
      __syncthreads();
    }
    // ------------------------------------------------------------- epilogue
    float *out = P.counts;
    if (F81) {
      // h_i lives with l0 == 0 blocks' rows? Every block owns h for its k rows
      // and g for its l columns; all blocks computed both, use them directly.
      if (active) {
        const float mu = P.f81_mu;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int cc = grp * 8 + q;
          if (cc >= gcols) continue;
          const int col = c_base + g0 + cc;
#pragma unroll
          for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b) {
              const int i = k0 + a, j = l0 + b;
              const float pi_i = __ldg(pig + i);
              // h (row i) and g (column j): recomputed per block from its own
              // accumulators — hv[a] holds h_i, gv[b] holds g_j
              const float I = acc[a * 4 + b][q] + hv[a][q] + pi_i * (gv[b][q] + zv[q]);
              out[(size_t)(i * A + j) * C + col] = (i == j) ? I : mu * __ldg(pig + j) * I;
            }
        }
      }
      __syncthreads();
      continue;
    }
    // back-transform: C -> T = C V^T -> VCV = V T, through shared memory [c][k][l]
    float *Cs = sm;  // G * A * A floats
    const float *V = P.tab + P.off.V;
    const float *Sm = P.tab + P.off.S;
    if (active) {
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int cc = grp * 8 + q;
#pragma unroll
        for (int a = 0; a < 4; ++a)
          *reinterpret_cast<float4 *>(Cs + ((size_t)cc * A + k0 + a) * A + l0) =
              make_float4(acc[a * 4][q], acc[a * 4 + 1][q], acc[a * 4 + 2][q], acc[a * 4 + 3][q]);
      }
    }
    __syncthreads();
    // T[c][k][j] = sum_l C[c][k][l] V[j][l]   (block (k0.., j0 = l0..))
    if (active) {
#pragma unroll
      for (int a = 0; a < 16; ++a)
#pragma unroll
        for (int q = 0; q < 8; ++q) acc[a][q] = 0.f;
      for (int l = 0; l < A; l += 4) {
        float vj[4][4];
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          const float4 r = __ldg(reinterpret_cast<const float4 *>(V + (l0 + b) * A + l));
          vj[b][0] = r.x, vj[b][1] = r.y, vj[b][2] = r.z, vj[b][3] = r.w;
        }
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int cc = grp * 8 + q;
#pragma unroll
          for (int a = 0; a < 4; ++a) {
            const float4 cr = *reinterpret_cast<const float4 *>(Cs + ((size_t)cc * A + k0 + a) * A + l);
            const float cv[4] = {cr.x, cr.y, cr.z, cr.w};
#pragma unroll
            for (int b = 0; b < 4; ++b)
#pragma unroll
              for (int m = 0; m < 4; ++m) acc[a * 4 + b][q] = fmaf(cv[m], vj[b][m], acc[a * 4 + b][q]);
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
              make_float4(acc[a * 4][q], acc[a * 4 + 1][q], acc[a * 4 + 2][q], acc[a * 4 + 3][q]);
      }
    }
    __syncthreads();
    // VCV[c][i][j] = sum_k V[i][k] T[c][k][j]   (block (i0 = k0.., j0 = l0..))
    if (active) {
#pragma unroll
      for (int a = 0; a < 16; ++a)
#pragma unroll
        for (int q = 0; q < 8; ++q) acc[a][q] = 0.f;
      for (int k = 0; k < A; ++k) {
        float vi[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) vi[a] = __ldg(V + (k0 + a) * A + k);
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int cc = grp * 8 + q;
          const float4 tr = *reinterpret_cast<const float4 *>(Cs + ((size_t)cc * A + k) * A + l0);
          const float tv[4] = {tr.x, tr.y, tr.z, tr.w};
#pragma unroll
          for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b) acc[a * 4 + b][q] = fmaf(vi[a], tv[b], acc[a * 4 + b][q]);
        }
      }
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int cc = grp * 8 + q;
        if (cc >= gcols) continue;
        const int col = c_base + g0 + cc;
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int b = 0; b < 4; ++b) {
            const int i = k0 + a, j = l0 + b;
            const float v = acc[a * 4 + b][q];
            out[(size_t)(i * A + j) * C + col] = (i == j) ? v : __ldg(Sm + i * A + j) * v;
          }
      }
    }
    __syncthreads();
  }
}

template <int A>
int walk_launch(const KParams &p, int mode, float *sa, float *sb, int c_base, int c_count, int grid,
                cudaStream_t s) {
  const int threads = 128 * Geo<A>::H;
  if (mode == 0) k_walk<A, 0><<<grid, threads, 0, s>>>(p, sa, sb, c_base, c_count);
  else if (mode == 1) k_walk<A, 1><<<grid, threads, 0, s>>>(p, sa, sb, c_base, c_count);
  else k_walk<A, 2><<<grid, threads, 0, s>>>(p, sa, sb, c_base, c_count);
  return (int)cudaGetLastError();
}

template <int A>
int acc_launch(const KParams &p, bool f81, const float *sa, const float *sb, int c_base, int c_count, int grid,
               cudaStream_t s) {
  using Gm = AccGeo<A>;
  const size_t stage = (size_t)(A * A + 2 * Gm::G * A) * 2 * sizeof(float);
  const size_t cbuf = (size_t)Gm::G * A * A * sizeof(float);
  const size_t smem = (stage + 2 * Gm::G * sizeof(float)) > cbuf ? (stage + 2 * Gm::G * sizeof(float)) : cbuf;
  cudaError_t e;
  if (f81) {
    e = cudaFuncSetAttribute(k_acc<A, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return (int)e;
    k_acc<A, true><<<grid, 256, smem, s>>>(p, sa, sb, c_base, c_count);
  } else {
    e = cudaFuncSetAttribute(k_acc<A, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return (int)e;
    k_acc<A, false><<<grid, 256, smem, s>>>(p, sa, sb, c_base, c_count);
  }
  return (int)cudaGetLastError();
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

int launch_walk(const KParams &p, int A, int mode, float *sa, float *sb, int c_base, int c_count, int grid,
                cudaStream_t s) {
  switch (A) {
    case 16: return walk_launch<16>(p, mode, sa, sb, c_base, c_count, grid, s);
    case 20: return walk_launch<20>(p, mode, sa, sb, c_base, c_count, grid, s);
    case 32: return walk_launch<32>(p, mode, sa, sb, c_base, c_count, grid, s);
    case 64: return walk_launch<64>(p, mode, sa, sb, c_base, c_count, grid, s);
    default: return -1;
  }
}

int launch_acc(const KParams &p, int A, bool f81, const float *sa, const float *sb, int c_base, int c_count,
               int grid, cudaStream_t s) {
  switch (A) {
    case 16: return acc_launch<16>(p, f81, sa, sb, c_base, c_count, grid, s);
    case 20: return acc_launch<20>(p, f81, sa, sb, c_base, c_count, grid, s);
    case 32: return acc_launch<32>(p, f81, sa, sb, c_base, c_count, grid, s);
    case 64: return acc_launch<64>(p, f81, sa, sb, c_base, c_count, grid, s);
    default: return -1;
  }
}

}  // namespace subby
