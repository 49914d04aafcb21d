// Branch posteriors (InsideOutside.branch_posterior, subby/jax/__init__.py:
// 948-1040; subby/oracle/oracle.py:1833-1905) from the raw per-branch staging
// of the walk (k_walk mode 3, k_walkpost.cu):
//   stage_a[n-1][c][a] = D_n(c, a) s_n(c),  stage_b[n-1][c][b] = U_n(c, b),
// s_n = 2^(e_D + e_U - e_root) / P(column), D_n the outside vector of branch n
// indexed by the parent's state, U_n the inside vector of node n.
//
//   joint_n(i, j) = D_n(i) M_n[i][j] U_n(j) / Z,
//   Z = sum_j (D_n^T M_n)(j) U_n(j)   (1 up to rounding: the scale s_n makes
//   the joint a probability; the explicit division follows the reference).
//
// Work item: (branch n, tile of 128 columns); one thread per column, M_n in
// shared memory (broadcast reads), the column's D_n in registers.  Output
// stores are coalesced across the tile's columns.  The kernel is bound by the
// output writes (A^2 floats per branch and column).
#include "common.cuh"

namespace subby {

namespace {

constexpr int kPostTile = 128;

template <int A>
__global__ void __launch_bounds__(kPostTile) k_post(const KParams P, const float *__restrict__ sa,
                                                    const float *__restrict__ sb, int c_base, int c_count, int n_lo,
                                                    int n_hi, int row_off, float *__restrict__ br_out) {
  constexpr int JB = (A % 16 == 0) ? 16 : 4;  // outputs per pass of the matvec
  extern __shared__ __align__(16) float s_post[];
  float *Ms = s_post;  // A x A: M_n[i][j]
  const int t = threadIdx.x;
  const int ntiles = (c_count + kPostTile - 1) / kPostTile;
  const long long items = (long long)(n_hi - n_lo) * ntiles;
  const float *MN = P.tab + P.off.MN;
  const int C = P.C;
  for (long long it = blockIdx.x; it < items; it += gridDim.x) {
    const int n = n_lo + (int)(it / ntiles);
    const int tile = (int)(it % ntiles);
    __syncthreads();  // the previous item's reads of Ms are done
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
        Z += (acc[4 * q] * u.x + acc[4 * q + 1] * u.y) + (acc[4 * q + 2] * u.z + acc[4 * q + 3] * u.w);
      }
    }
    // the reference divides only where the total is positive
    const float inv = Z > 0.f ? 1.0f / Z : 1.0f;
    if (!valid) continue;
    const size_t col = (size_t)c_base + cc;
    const size_t row = (size_t)(n - row_off);
    float *o = br_out + row * A * A * C + col;
#pragma unroll 1
    for (int j = 0; j < A; ++j) {
      const float u = __ldg(pb + j) * inv;
#pragma unroll
      for (int i = 0; i < A; ++i) __stcs(o + ((size_t)i * A + j) * C, d[i] * Ms[i * A + j] * u);  // streamed: written once, never re-read here
    }
  }
}

template <int A>
int post_launch(const KParams &p, const float *sa, const float *sb, int c_base, int c_count, int n_lo, int n_hi,
                int row_off, float *br_out, int grid, cudaStream_t s) {
  k_post<A><<<grid, kPostTile, (size_t)A * A * sizeof(float), s>>>(p, sa, sb, c_base, c_count, n_lo, n_hi, row_off,
                                                                  br_out);
  return (int)cudaGetLastError();
}

}  // namespace

bool post_supported(int A) { return A == 4 || A == 8 || big_supported(A); }

int post_tile() { return kPostTile; }

int launch_post(const KParams &p, int A, const float *sa, const float *sb, int c_base, int c_count, int n_lo,
                int n_hi, int row_off, float *br_out, int grid, cudaStream_t s) {
  switch (A) {
    case 4: return post_launch<4>(p, sa, sb, c_base, c_count, n_lo, n_hi, row_off, br_out, grid, s);
    case 8: return post_launch<8>(p, sa, sb, c_base, c_count, n_lo, n_hi, row_off, br_out, grid, s);
    case 16: return post_launch<16>(p, sa, sb, c_base, c_count, n_lo, n_hi, row_off, br_out, grid, s);
    case 20: return post_launch<20>(p, sa, sb, c_base, c_count, n_lo, n_hi, row_off, br_out, grid, s);
    case 32: return post_launch<32>(p, sa, sb, c_base, c_count, n_lo, n_hi, row_off, br_out, grid, s);
    case 64: return post_launch<64>(p, sa, sb, c_base, c_count, n_lo, n_hi, row_off, br_out, grid, s);
    default: return -1;
  }
}

}  // namespace subby
