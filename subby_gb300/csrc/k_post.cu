// Node and branch posteriors (InsideOutside.node_posterior / branch_posterior,
// subby/jax/__init__.py:868-1040; subby/oracle/oracle.py:1755-1905) from the
// raw per-branch staging of the large-alphabet walk (k_walk MODE 2):
//   stage_a[n-1][c][a] = D_n(c, a) s_n(c),  stage_b[n-1][c][b] = U_n(c, b),
// s_n = 2^(e_D + e_U - e_root) / P(column), D_n the outside vector of branch n
// indexed by the parent's state, U_n the inside vector of node n.
//
//   node n > 0 : post_n(j) = (sum_i D_n(i) M_n[i][j]) U_n(j) / Z
//   branch n   : joint_n(i, j) = D_n(i) M_n[i][j] U_n(j) / Z
//   Z = sum_j (D_n^T M_n)(j) U_n(j)   (1 up to rounding: the scale s_n makes
//   the joint a probability; the explicit division follows the reference).
// The root's posterior (pi . U_root normalised) is the walk's RootProb.
//
// Work item: (branch n, tile of 128 columns); one thread per column, M_n in
// shared memory (broadcast reads), the column's D_n in registers.  Output
// stores are coalesced across the tile's columns.  The kernel is bound by the
// output writes (A or A^2 floats per branch and column) plus the staging reads
// (2 A floats).
#include "common.cuh"

namespace subby {

namespace {

constexpr int kPostTile = 128;

template <int A, bool NODE, bool BRANCH>
__global__ void __launch_bounds__(kPostTile) k_post(const KParams P, const float *__restrict__ sa,
                                                    const float *__restrict__ sb, int c_base, int c_count, int n_lo,
                                                    int n_hi, int row_off, float *__restrict__ node_out,
                                                    float *__restrict__ br_out) {
  constexpr int JB = (A % 16 == 0) ? 16 : 4;  // outputs per pass of the matvec
  extern __shared__ __align__(16) float s_post[];
  float *Ms = s_post;          // A x A: M_n[i][j]
  float *ys = s_post + A * A;  // NODE: [j][128 columns] unnormalised posterior
  const int t = threadIdx.x;
  const int ntiles = (c_count + kPostTile - 1) / kPostTile;
  const long long items = (long long)(n_hi - n_lo) * ntiles;
  const float *MN = P.tab + P.off.MN;
  const int C = P.C;
  for (long long it = blockIdx.x; it < items; it += gridDim.x) {
    const int n = n_lo + (int)(it / ntiles);
    const int tile = (int)(it % ntiles);
    __syncthreads();  // the previous item's reads of Ms / ys are done
    const float4 *Mg = reinterpret_cast<const float4 *>(MN + (size_t)n * A * A);
    for (int e = t; e < A * A / 4; e += kPostTile) reinterpret_cast<float4 *>(Ms)[e] = __ldg(Mg + e);
    __syncthreads();
    const int cc = tile * kPostTile + t;
    const bool valid = cc < c_count;
    const size_t srow = ((size_t)(n - 1) * c_count + (valid ? cc : c_count - 1)) * A;
    const float *pa = sa + srow;
    const float *pb = sb + srow;
    float d[A];
#pragma unroll
    for (int q = 0; q < A / 4; ++q) {
      const float4 v = __ldg(reinterpret_cast<const float4 *>(pa) + q);
      d[4 * q] = v.x, d[4 * q + 1] = v.y, d[4 * q + 2] = v.z, d[4 * q + 3] = v.w;
    }
    float Z = 0.f;
#pragma unroll 1
    for (int jb = 0; jb < A; jb += JB) {
      float acc[JB];
#pragma unroll
      for (int jj = 0; jj < JB; ++jj) acc[jj] = 0.f;
#pragma unroll
      for (int i = 0; i < A; ++i) {
        const float4 *mr = reinterpret_cast<const float4 *>(Ms + i * A + jb);
#pragma unroll
        for (int q = 0; q < JB / 4; ++q) {
          const float4 m = mr[q];
          acc[4 * q] = fmaf(d[i], m.x, acc[4 * q]);
          acc[4 * q + 1] = fmaf(d[i], m.y, acc[4 * q + 1]);
          acc[4 * q + 2] = fmaf(d[i], m.z, acc[4 * q + 2]);
          acc[4 * q + 3] = fmaf(d[i], m.w, acc[4 * q + 3]);
        }
      }
#pragma unroll
      for (int q = 0; q < JB / 4; ++q) {
        const float4 u = __ldg(reinterpret_cast<const float4 *>(pb + jb) + q);
        // rounded products (no contraction into the sum), so that every
        // variant of the kernel forms the same Z
        const float y0 = __fmul_rn(acc[4 * q], u.x), y1 = __fmul_rn(acc[4 * q + 1], u.y),
                    y2 = __fmul_rn(acc[4 * q + 2], u.z), y3 = __fmul_rn(acc[4 * q + 3], u.w);
        Z += (y0 + y1) + (y2 + y3);
        if constexpr (NODE) {
          ys[(jb + 4 * q) * kPostTile + t] = y0;
          ys[(jb + 4 * q + 1) * kPostTile + t] = y1;
          ys[(jb + 4 * q + 2) * kPostTile + t] = y2;
          ys[(jb + 4 * q + 3) * kPostTile + t] = y3;
        }
      }
    }
    // the reference divides only where the total is positive
    const float inv = Z > 0.f ? 1.0f / Z : 1.0f;
    if (!valid) continue;
    const size_t col = (size_t)c_base + cc;
    const size_t row = (size_t)(n - row_off);
    if constexpr (NODE) {
      float *o = node_out + row * A * C + col;
#pragma unroll 4
      for (int j = 0; j < A; ++j) o[(size_t)j * C] = ys[j * kPostTile + t] * inv;
    }
    if constexpr (BRANCH) {
      float *o = br_out + row * A * A * C + col;
#pragma unroll 1
      for (int j = 0; j < A; ++j) {
        const float u = __ldg(pb + j) * inv;
#pragma unroll
        for (int i = 0; i < A; ++i) o[((size_t)i * A + j) * C] = d[i] * Ms[i * A + j] * u;
      }
    }
  }
}

template <int A, bool NODE, bool BRANCH>
int post_launch1(const KParams &p, const float *sa, const float *sb, int c_base, int c_count, int n_lo, int n_hi,
                 int row_off, float *node_out, float *br_out, int grid, cudaStream_t s) {
  const size_t smem = (size_t)(A * A + (NODE ? A * kPostTile : 0)) * sizeof(float);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k_post<A, NODE, BRANCH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return (int)e;
  }
  k_post<A, NODE, BRANCH><<<grid, kPostTile, smem, s>>>(p, sa, sb, c_base, c_count, n_lo, n_hi, row_off, node_out,
                                                        br_out);
  return (int)cudaGetLastError();
}

template <int A>
int post_launch(const KParams &p, const float *sa, const float *sb, int c_base, int c_count, int n_lo, int n_hi,
                int row_off, float *node_out, float *br_out, int grid, cudaStream_t s) {
  if (node_out && br_out)
    return post_launch1<A, true, true>(p, sa, sb, c_base, c_count, n_lo, n_hi, row_off, node_out, br_out, grid, s);
  if (node_out)
    return post_launch1<A, true, false>(p, sa, sb, c_base, c_count, n_lo, n_hi, row_off, node_out, br_out, grid, s);
  return post_launch1<A, false, true>(p, sa, sb, c_base, c_count, n_lo, n_hi, row_off, node_out, br_out, grid, s);
}

}  // namespace

bool post_supported(int A) { return A == 4 || A == 8 || big_supported(A); }

int post_tile() { return kPostTile; }

int launch_post(const KParams &p, int A, const float *sa, const float *sb, int c_base, int c_count, int n_lo,
                int n_hi, int row_off, float *node_out, float *br_out, int grid, cudaStream_t s) {
  switch (A) {
    case 4: return post_launch<4>(p, sa, sb, c_base, c_count, n_lo, n_hi, row_off, node_out, br_out, grid, s);
    case 8: return post_launch<8>(p, sa, sb, c_base, c_count, n_lo, n_hi, row_off, node_out, br_out, grid, s);
    case 16: return post_launch<16>(p, sa, sb, c_base, c_count, n_lo, n_hi, row_off, node_out, br_out, grid, s);
    case 20: return post_launch<20>(p, sa, sb, c_base, c_count, n_lo, n_hi, row_off, node_out, br_out, grid, s);
    case 32: return post_launch<32>(p, sa, sb, c_base, c_count, n_lo, n_hi, row_off, node_out, br_out, grid, s);
    case 64: return post_launch<64>(p, sa, sb, c_base, c_count, n_lo, n_hi, row_off, node_out, br_out, grid, s);
    default: return -1;
  }
}

}  // namespace subby
