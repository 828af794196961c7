// Post-processing of finished maps: mp_sqom's speckle filter (code/src/mp_sqom56.f90:1531-1570).
//
// The reference walks the flattened map once (x fastest) with wrap-around neighbours,
// replacing a value v_i below min(v_{i-1}, v_{i+1}) / s_trig by that minimum and a value above
// s_trig * max(v_{i-1}, v_{i+1}) by that maximum, where v_{i-1} is the already filtered
// predecessor and v_{i+1} the unfiltered successor (the filtered first value for the last
// one); for plane maps it repeats the walk over the transposed map.  Each step depends on the
// step before it, so the GPU form is speculative: one CTA splits the line into a chunk per
// thread, filters every chunk from its unfiltered left neighbour, and refilters a chunk
// whenever the value entering it from the left changes, until nothing changes.  Chunk 0
// enters from the unfiltered last value, as the reference's first step does, so it is right
// after one pass and chunk k after at most k + 1; the last element's right neighbour is the
// filtered first value.  The result is bit-identical to the sequential walk (FP32, the
// reference's division and multiplication, no contraction).
#include <cuda_runtime.h>

#include <algorithm>

#include "mpsq.h"
#include "mpsq_internal.h"

namespace mpsq {
namespace {

constexpr int kSpeckleThreads = 1024;

// One step of the reference's walk (two tests in its order; the second sees the first's result).
__device__ __forceinline__ float speckle_step(float v, float left, float right, float s_trig) {
  const float lo = fminf(left, right), hi = fmaxf(left, right);
  if (v < __fdiv_rn(lo, s_trig)) v = lo;
  if (v > __fmul_rn(s_trig, hi)) v = hi;
  return v;
}

__global__ void __launch_bounds__(kSpeckleThreads)
    speckle_line_kernel(const float* __restrict__ in, float* __restrict__ out, int64_t n,
                        float s_trig) {
  __shared__ float last_out[kSpeckleThreads];
  __shared__ float first_out;
  const int t = threadIdx.x;
  const int64_t chunk = (n + kSpeckleThreads - 1) / kSpeckleThreads;
  const int64_t lo = (int64_t)t * chunk;
  const int64_t hi = min(n, lo + chunk);
  const bool live = lo < hi;
  const bool owns_last = live && hi == n;
  // the value entering this chunk from the left, and (last chunk) the first value's filtered form
  float left = live ? in[lo == 0 ? n - 1 : lo - 1] : 0.0f;
  float right_end = in[0];
  bool dirty = live;
  for (int pass = 0; pass <= kSpeckleThreads + 1; ++pass) {  // terminates by pass n_chunks + 1
    if (dirty) {
      float prev = left;
      for (int64_t i = lo; i < hi; ++i) {
        const float right = i + 1 < n ? in[i + 1] : right_end;
        prev = speckle_step(in[i], prev, right, s_trig);
        out[i] = prev;
      }
      last_out[t] = prev;
      if (t == 0) first_out = out[0];
    }
    __syncthreads();
    bool changed = false;
    if (live && t > 0 && __float_as_int(last_out[t - 1]) != __float_as_int(left)) {
      left = last_out[t - 1];
      changed = true;
    }
    if (owns_last && __float_as_int(first_out) != __float_as_int(right_end)) {
      right_end = first_out;
      changed = true;
    }
    dirty = changed;
    if (!__syncthreads_or(changed)) break;
  }
}

// out[c][r] = in[r][c] * scale for an (rows x cols) row-major input.
__global__ void transpose_scale_kernel(const float* __restrict__ in, float* __restrict__ out,
                                       int64_t rows, int64_t cols, float scale) {
  __shared__ float tile[32][33];
  const int64_t c0 = (int64_t)blockIdx.x * 32, r0 = (int64_t)blockIdx.y * 32;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int64_t r = r0 + k, c = c0 + threadIdx.x;
    if (r < rows && c < cols) tile[k][threadIdx.x] = in[r * cols + c];
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int64_t c = c0 + k, r = r0 + threadIdx.x;
    if (r < rows && c < cols) out[c * rows + r] = __fmul_rn(tile[threadIdx.x][k], scale);
  }
}

__global__ void scale_copy_kernel(const float* __restrict__ in, float* __restrict__ out,
                                  int64_t n, float scale) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = __fmul_rn(in[i], scale);
}

}  // namespace
}  // namespace mpsq

using namespace mpsq;

extern "C" int mpsq_speckle_filter(float* map, int64_t n_fast, int64_t n_slow, float s_trig,
                                   int32_t perpendicular, float post_scale, int32_t host,
                                   void* stream) {
  if (!map) return fail(MPSQ_ERR_ARG, "speckle_filter: null map");
  if (n_fast < 1 || n_slow < 1) return fail(MPSQ_ERR_ARG, "speckle_filter: empty map");
  if (!(s_trig > 0.0f)) return fail(MPSQ_ERR_ARG, "speckle_filter: s_trig must be > 0 (0 is off)");
  const int64_t n = n_fast * n_slow;
  if (n > ((int64_t)1 << 31)) return fail(MPSQ_ERR_ARG, "speckle_filter: map too large");
  cudaStream_t s = (cudaStream_t)stream;
  if (perpendicular && std::max(n_fast, n_slow) > (int64_t)65535 * 32)
    return fail(MPSQ_ERR_ARG, "speckle_filter: map side too long for the transposes");
  float *a = nullptr, *b = nullptr;
  auto cleanup = [&]() {
    cudaFree(a);
    cudaFree(b);
  };
  cudaError_t e = cudaMalloc(&a, n * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&b, n * sizeof(float));
  if (e != cudaSuccess) {
    cleanup();
    return fail(MPSQ_ERR_ALLOC, "speckle_filter: %s", cudaGetErrorString(e));
  }
  e = cudaMemcpyAsync(a, map, n * sizeof(float), host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, s);
  if (e != cudaSuccess) {
    cleanup();
    return fail(MPSQ_ERR_CUDA, "speckle_filter: %s", cudaGetErrorString(e));
  }
  float* result = b;
  if (n > 1) {  // a one-value map compares its value with itself and never changes
    speckle_line_kernel<<<1, kSpeckleThreads, 0, s>>>(a, b, n, s_trig);
    count_launch();
    if (perpendicular) {
      const dim3 tb(32, 8);
      transpose_scale_kernel<<<dim3((unsigned)((n_fast + 31) / 32), (unsigned)((n_slow + 31) / 32)), tb, 0, s>>>(
          b, a, n_slow, n_fast, 1.0f);
      speckle_line_kernel<<<1, kSpeckleThreads, 0, s>>>(a, b, n, s_trig);
      transpose_scale_kernel<<<dim3((unsigned)((n_slow + 31) / 32), (unsigned)((n_fast + 31) / 32)), tb, 0, s>>>(
          b, a, n_fast, n_slow, post_scale);
      count_launch(3);
      result = a;
    } else {
      scale_copy_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(b, a, n, post_scale);
      count_launch();
      result = a;
    }
  } else {
    scale_copy_kernel<<<1, 32, 0, s>>>(a, b, n, post_scale);
    count_launch();
  }
  e = cudaGetLastError();
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(map, result, n * sizeof(float), host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cleanup();
  if (e != cudaSuccess) return fail(MPSQ_ERR_CUDA, "speckle_filter: %s", cudaGetErrorString(e));
  return MPSQ_OK;
}
