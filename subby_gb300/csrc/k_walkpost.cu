// The walk of the posteriors (InsideOutside.node_posterior / branch_posterior,
// subby/jax/__init__.py:868-1040): k_walk in mode 3 writes the node
// posteriors of every branch's child from the D_n and U_n it holds, and
// stages D_n s_n, U_n for the branch-posterior kernel (k_post.cu) when asked;
// mode 0 (inside only) gives the root's.  Own translation unit, so that these
// instantiations compile beside the count path's.
#include "walk.cuh"

namespace subby {

namespace {

template <int A, bool TC>
int walk_post1(const KParams &p, int mode, float *sa, float *sb, int c_base, int c_count, int grid, cudaStream_t s) {
  const bool f = !TC && p.f81_model != 0;
  constexpr bool kF = !TC;
  if (mode == 0)
    return f ? walk_launch1<A, 0, TC, kF>(p, sa, sb, c_base, c_count, grid, s)
             : walk_launch1<A, 0, TC, false>(p, sa, sb, c_base, c_count, grid, s);
  return f ? walk_launch1<A, 3, TC, kF>(p, sa, sb, c_base, c_count, grid, s)
           : walk_launch1<A, 3, TC, false>(p, sa, sb, c_base, c_count, grid, s);
}

template <int A>
int walk_post(const KParams &p, int mode, bool tc, float *sa, float *sb, int c_base, int c_count, int grid,
              cudaStream_t s) {
  if constexpr (A == 64) {
    // the closed-form F81 walk has no matrix products for the tensor cores
    if (tc && !p.f81_model) return walk_post1<A, true>(p, mode, sa, sb, c_base, c_count, grid, s);
  }
  return walk_post1<A, false>(p, mode, sa, sb, c_base, c_count, grid, s);
}

}  // namespace

int launch_walk_post(const KParams &p, int A, int mode, bool tc, float *sa, float *sb, int c_base, int c_count,
                     int grid, cudaStream_t s) {
  switch (A) {
    case 4: return walk_post<4>(p, mode, tc, sa, sb, c_base, c_count, grid, s);
    case 8: return walk_post<8>(p, mode, tc, sa, sb, c_base, c_count, grid, s);
    case 16: return walk_post<16>(p, mode, tc, sa, sb, c_base, c_count, grid, s);
    case 20: return walk_post<20>(p, mode, tc, sa, sb, c_base, c_count, grid, s);
    case 32: return walk_post<32>(p, mode, tc, sa, sb, c_base, c_count, grid, s);
    case 64: return walk_post<64>(p, mode, tc, sa, sb, c_base, c_count, grid, s);
    default: return -1;
  }
}

}  // namespace subby
