// Character -> token mapping of the front-end parsers (subby/formats.py:
// 228-625 tokenise sequence characters: alphabet index, A+1 for '-' / '.'):
// a 256-entry table in shared memory applied to a device byte buffer, 16
// bytes per thread per step (one 16-byte load, four 16-byte stores); bytes
// the table maps to -1 record their smallest index in *first_bad.
// HBM-bound: 1 byte read + 4 bytes written per cell.
#include <cuda_runtime.h>

#include <algorithm>

#include "common.cuh"
#include "subby_gb300.h"

namespace subby {
namespace {

__global__ void k_tokenize(const uint8_t *__restrict__ in, long long n, const int32_t *__restrict__ lut,
                           int32_t *__restrict__ out, unsigned long long *first_bad) {
  __shared__ int32_t s_lut[256];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) s_lut[i] = lut[i];
  __syncthreads();
  const long long nvec = n / 16;
  unsigned long long bad = ~0ull;
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nvec;
       v += (long long)gridDim.x * blockDim.x) {
    const uint4 w = reinterpret_cast<const uint4 *>(in)[v];
    const uint32_t words[4] = {w.x, w.y, w.z, w.w};
    int32_t t[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      t[q] = s_lut[(words[q >> 2] >> (8 * (q & 3))) & 0xffu];
      if (t[q] < 0) bad = min(bad, (unsigned long long)(v * 16 + q));
    }
    int4 *o = reinterpret_cast<int4 *>(out + v * 16);
#pragma unroll
    for (int q = 0; q < 4; ++q) o[q] = make_int4(t[4 * q], t[4 * q + 1], t[4 * q + 2], t[4 * q + 3]);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    for (long long i = nvec * 16; i < n; ++i) {
      const int32_t t = s_lut[in[i]];
      out[i] = t;
      if (t < 0) bad = min(bad, (unsigned long long)i);
    }
  }
  if (bad != ~0ull) atomicMin(first_bad, bad);
}

}  // namespace
}  // namespace subby

extern "C" int subby_tokenize(const uint8_t *chars, int64_t n, const int32_t *lut, int32_t *out,
                              int64_t *first_bad, void *stream_) {
  if (!lut || !first_bad || n < 0) return SUBBY_ERR_ARG;
  if (n == 0) return SUBBY_OK;  // empty device buffers may be null
  if (!chars || !out) return SUBBY_ERR_ARG;
  if ((reinterpret_cast<uintptr_t>(chars) & 15) || (reinterpret_cast<uintptr_t>(out) & 15)) return SUBBY_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream_;
  int dev = 0, nsm = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int block = 256;
  const long long nvec = std::max<long long>(1, n / 16);
  const int grid = (int)std::min<long long>((nvec + block - 1) / block, (long long)nsm * 8);
  subby::k_tokenize<<<grid, block, 0, s>>>(chars, n, lut, out, reinterpret_cast<unsigned long long *>(first_bad));
  return cudaGetLastError() == cudaSuccess ? SUBBY_OK : SUBBY_ERR_CUDA;
}

// Token rows of a job's alignment gathered from where the caller holds them
// (pinned host memory, read by the SMs over the host link, or device memory)
// into a contiguous (R, C) device array: dst[r][c] = src[map(r) * pitch + c],
// map(r) = rowmap[r] (device array) or r.  A serving loop hands each job's
// alignment over as a window of a larger host buffer this way, without a
// host-side copy into a staging buffer.  Rows whose source and destination
// are 16-byte aligned (and C a multiple of 4) move as 16-byte vectors.
namespace subby {
namespace {

__global__ void k_gather_rows(const int32_t *__restrict__ src, long long pitch, const int32_t *__restrict__ rowmap,
                              int C, int32_t *__restrict__ dst) {
  const int r = blockIdx.y;
  const long long sr = rowmap ? (long long)rowmap[r] : (long long)r;
  const int32_t *s = src + sr * pitch;
  int32_t *d = dst + (long long)r * C;
  const bool vec = ((reinterpret_cast<uintptr_t>(s) | reinterpret_cast<uintptr_t>(d)) & 15) == 0 && (C & 3) == 0;
  if (vec) {
    const int nv = C >> 2;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x)
      reinterpret_cast<int4 *>(d)[v] = reinterpret_cast<const int4 *>(s)[v];
  } else {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < C; c += gridDim.x * blockDim.x) d[c] = s[c];
  }
}

}  // namespace
}  // namespace subby

extern "C" int subby_gather_rows(const int32_t *src, int64_t pitch, const int32_t *rowmap, int R, int C,
                                 int32_t *dst, void *stream_) {
  if (R < 0 || C < 0 || pitch < C) return SUBBY_ERR_ARG;
  if (R == 0 || C == 0) return SUBBY_OK;
  if (!src || !dst) return SUBBY_ERR_ARG;
  if (R > 65535) return SUBBY_ERR_UNSUPPORTED;
  const int block = 256;
  const int per_thread = 4;  // 16-byte vectors per thread per row
  const int gx = std::max(1, std::min(1024, (C / 4 + block * per_thread - 1) / (block * per_thread)));
  subby::k_gather_rows<<<dim3(gx, R), block, 0, (cudaStream_t)stream_>>>(src, pitch, rowmap, C, dst);
  return cudaGetLastError() == cudaSuccess ? SUBBY_OK : SUBBY_ERR_CUDA;
}

// Row-strided copy run by the SMs (device memory to pinned host memory in
// the serving engine): dst[r * dpitch + i] = src[r * spitch + i] for byte i
// < width.  Unlike a copy-engine transfer, whose queue is served in order,
// its CTAs are scheduled like any kernel's, so the result copies of short
// jobs (on high-priority streams) are not held behind multi-gigabyte copies
// of long ones.  Rows whose addresses and width are 16-byte aligned move as
// 16-byte vectors, others as 4-byte words (all uses copy float32 arrays).
namespace subby {
namespace {

__global__ void k_copy_rows(char *__restrict__ dst, size_t dpitch, const char *__restrict__ src, size_t spitch,
                            size_t width) {
  char *d = dst + (size_t)blockIdx.y * dpitch;
  const char *s = src + (size_t)blockIdx.y * spitch;
  const size_t step = (size_t)gridDim.x * blockDim.x;
  if (((reinterpret_cast<uintptr_t>(d) | reinterpret_cast<uintptr_t>(s) | width) & 15) == 0) {
    const size_t nv = width >> 4;
    for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += step)
      reinterpret_cast<int4 *>(d)[v] = reinterpret_cast<const int4 *>(s)[v];
  } else {
    const size_t nw = width >> 2;
    for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < nw; v += step)
      reinterpret_cast<int *>(d)[v] = reinterpret_cast<const int *>(s)[v];
  }
}

}  // namespace

int launch_copy_rows(void *dst, size_t dpitch, const void *src, size_t spitch, size_t width, int rows,
                     cudaStream_t s) {
  if (rows <= 0 || width == 0) return 0;
  if ((width & 3) || rows > 65535) return (int)cudaErrorInvalidValue;
  const int block = 256;
  const size_t per_cta = (size_t)block * 16 * 4;  // four 16-byte vectors per thread
  const int gx = (int)std::max<size_t>(1, std::min<size_t>(1024, (width + per_cta - 1) / per_cta));
  k_copy_rows<<<dim3(gx, rows), block, 0, s>>>(static_cast<char *>(dst), dpitch, static_cast<const char *>(src),
                                               spitch, width);
  return (int)cudaGetLastError();
}

}  // namespace subby
