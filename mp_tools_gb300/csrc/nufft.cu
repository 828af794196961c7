// Type-1 NUFFT engine for sm_103a: bin (with halo copies) -> owner-computes tile spreading in
// shared memory -> cuFFT on the fine grid -> deconvolution / mode extraction.
//
// Replaces the work FINUFFT does inside the finufft2d1 call of MP_TOOLS
// (code/src/mp_sqom56.f90:1148, code/src/mp_sql56.f90:1129).  The arithmetic follows the
// published method (Barnett, Magland, af Klinteberg 2019): exponential-of-semicircle kernel,
// upsampling factor 2, division by the kernel's Fourier transform.  The GPU organisation is
// this library's own: every fine-grid cell is written exactly once by the CTA that owns its
// tile (no global atomics, no zero fill), points are duplicated into each tile their support
// touches, and the whole grid leaves the SM through coalesced stores.
#include <cuda_runtime.h>
#include <cufft.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <type_traits>
#include <string>
#include <vector>

#include "mpsq_internal.h"

namespace mpsq {

// ------------------------------------------------------------------------------ errors
std::atomic<int64_t> g_launches{0};
static thread_local char t_err[1024] = "";

int fail(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(t_err, sizeof(t_err), fmt, ap);
  va_end(ap);
  return code;
}

// ------------------------------------------------------------------------- ES kernel
EsKernel es_params(double eps, int precision) {
  double lo = precision == MPSQ_FP64 ? 1e-14 : 1e-7;
  if (!(eps >= lo)) eps = lo;   // also catches NaN
  if (eps > 1e-1) eps = 1e-1;
  int w = (int)std::ceil(std::log10(1.0 / eps)) + 1;
  w = std::max(2, std::min(16, w));
  // FP32 transforms stop at eps = 1e-7 (w = 8): below that the FP32 rounding of spreading and
  // FFT, not the kernel's truncation, sets the error.
  EsKernel k;
  k.w = w;
  k.beta = 2.30 * w;
  return k;
}

// Gauss-Legendre nodes/weights on [-1,1] by Newton iteration on P_n.
static void gauss_legendre(int n, std::vector<double>& x, std::vector<double>& wt) {
  x.resize(n);
  wt.resize(n);
  for (int i = 0; i < n; ++i) {
    double z = std::cos(M_PI * (i + 0.75) / (n + 0.5));
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= n; ++k) {
        double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      double dp = n * (z * p1 - p0) / (z * z - 1.0);
      double dz = p1 / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-16) break;
    }
    double p0 = 1.0, p1 = z;
    for (int k = 2; k <= n; ++k) {
      double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
      p0 = p1;
      p1 = p2;
    }
    double dp = n * (z * p1 - p0) / (z * z - 1.0);
    x[i] = z;
    wt[i] = 2.0 / ((1.0 - z * z) * dp * dp);
  }
}

void es_correction(const EsKernel& es, int64_t nf, int64_t m, double* out) {
  // phihat(k) = int_{-w/2}^{w/2} phi(2u/w) cos(2 pi k u / nf) du, u in fine-grid cells.
  const int nq = 4 * es.w + 40;
  std::vector<double> x, wt;
  gauss_legendre(nq, x, wt);
  const double half = 0.5 * es.w;
  std::vector<double> u(nq), f(nq);
  for (int q = 0; q < nq; ++q) {
    u[q] = half * x[q];
    double z = x[q];
    f[q] = half * wt[q] * std::exp(es.beta * (std::sqrt(std::max(0.0, 1.0 - z * z)) - 1.0));
  }
  for (int64_t i = 0; i < m; ++i) {
    int64_t k = i - m / 2;
    double s = 0.0;
    for (int q = 0; q < nq; ++q) s += f[q] * std::cos(2.0 * M_PI * (double)k * u[q] / (double)nf);
    out[i] = 1.0 / s;
  }
}

static bool smooth235(int64_t n) {
  for (int p : {2, 3, 5})
    while (n % p == 0) n /= p;
  return n == 1;
}

int64_t fine_size(int64_t m, int w, int tile) {
  int64_t n = std::max<int64_t>({2 * m, 2 * (int64_t)w, (int64_t)tile});
  n = ((n + tile - 1) / tile) * tile;
  while (!smooth235(n)) n += tile;
  return n;
}

int make_geom(int dim, const int64_t* m, int w, GridGeom* g) {
  if (dim != 2 && dim != 3) return fail(MPSQ_ERR_ARG, "dim must be 2 or 3 (got %d)", dim);
  GridGeom r;
  r.dim = dim;
  int tile = dim == 3 ? kTile3 : kTile2;
  for (int a = 0; a < 3; ++a) {
    if (a < dim) {
      if (m[a] < 1) return fail(MPSQ_ERR_ARG, "n_modes[%d] = %lld < 1", a, (long long)m[a]);
      if (m[a] > (1 << 15)) return fail(MPSQ_ERR_ARG, "n_modes[%d] = %lld too large", a, (long long)m[a]);
      r.m[a] = m[a];
      r.nf[a] = fine_size(m[a], w, tile);
      r.tile[a] = tile;
      r.ntile[a] = (int)(r.nf[a] / tile);
    } else {
      r.m[a] = 1;
      r.nf[a] = 1;
      r.tile[a] = 1;
      r.ntile[a] = 1;
    }
  }
  r.n_tiles = (int64_t)r.ntile[0] * r.ntile[1] * r.ntile[2];
  r.n_fine = r.nf[0] * r.nf[1] * r.nf[2];
  r.n_modes = r.m[0] * r.m[1] * r.m[2];
  *g = r;
  return MPSQ_OK;
}

int check_dev_error(const int* dev_flag, cudaStream_t s) {
  int h = 0;
  MPSQ_CUDA_TRY(cudaMemcpyAsync(&h, dev_flag, sizeof(int), cudaMemcpyDeviceToHost, s));
  MPSQ_CUDA_TRY(cudaStreamSynchronize(s));
  if (h & kErrRecOverflow) return fail(MPSQ_ERR_DEVICE, "binning: record capacity exceeded");
  if (h & kErrBadIndex) return fail(MPSQ_ERR_DEVICE, "kernel bound check failed (flag %d)", h);
  return MPSQ_OK;
}

// --------------------------------------------------------------------------- device code
// Plan API binning: coordinates in radians (FINUFFT convention).
template <typename T>
__global__ void bin_plan_kernel(int64_t nj, const T* __restrict__ x, const T* __restrict__ y,
                                const T* __restrict__ z, SpreadArgs a, int scatter,
                                int* cursor, const int* __restrict__ starts,
                                typename RecOf<T>::type* recs, int* idx_out, int64_t cap,
                                int* err) {
  int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nj) return;
  double g[3] = {0.0, 0.0, 0.0};
  g[0] = fold_grid((double)x[j] * a.gscale[0], (double)a.nf[0], a.ginv[0]);
  g[1] = fold_grid((double)y[j] * a.gscale[1], (double)a.nf[1], a.ginv[1]);
  if (a.dim == 3) g[2] = fold_grid((double)z[j] * a.gscale[2], (double)a.nf[2], a.ginv[2]);
  typename Cplx<T>::type zero;
  zero.x = 0;
  zero.y = 0;
  emit_records<T>(a, g, 0, 0, scatter != 0, cursor, starts, recs, nullptr, zero, idx_out, (int)j,
                  cap, err);
}

// Exclusive scan of n counts into starts[0..n], one CTA of kScanThreads threads: the counts
// pass through shared memory in spans of kScanThreads * kScanPer (coalesced loads and
// stores), each thread scanning kScanPer consecutive entries of a span, with a running carry.
constexpr int kScanThreads = 1024;
constexpr int kScanPer = 8;
__global__ void __launch_bounds__(kScanThreads)
    scan_kernel(const int* __restrict__ counts, int* __restrict__ starts, int64_t n) {
  __shared__ int buf[kScanThreads * kScanPer];
  __shared__ long long warp_sums[kScanThreads / 32];
  const int tid = threadIdx.x;
  const int lane = tid & 31, wid = tid >> 5;
  constexpr int span = kScanThreads * kScanPer;
  long long carry = 0;
  for (int64_t base = 0; base < n; base += span) {
    for (int i = tid; i < span; i += kScanThreads) {
      const int64_t g = base + i;
      buf[i] = g < n ? counts[g] : 0;
    }
    __syncthreads();
    int v[kScanPer];
    long long sum = 0;
#pragma unroll
    for (int k = 0; k < kScanPer; ++k) {
      v[k] = buf[tid * kScanPer + k];
      sum += v[k];
    }
    long long incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const long long t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    if (lane == 31) warp_sums[wid] = incl;
    __syncthreads();
    if (wid == 0) {
      long long w = warp_sums[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const long long t = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += t;
      }
      warp_sums[lane] = w;
    }
    __syncthreads();
    long long excl = carry + incl - sum + (wid > 0 ? warp_sums[wid - 1] : 0);
#pragma unroll
    for (int k = 0; k < kScanPer; ++k) {
      buf[tid * kScanPer + k] = (int)excl;
      excl += v[k];
    }
    carry += warp_sums[kScanThreads / 32 - 1];
    __syncthreads();
    for (int i = tid; i < span; i += kScanThreads) {
      const int64_t g = base + i;
      if (g < n) starts[g] = buf[i];
    }
    __syncthreads();   // buf and warp_sums are rewritten by the next span
  }
  if (tid == 0) starts[n] = (int)carry;
}

template <typename T>
__device__ __forceinline__ T es_eval(T z, T beta);
template <>
__device__ __forceinline__ float es_eval<float>(float z, float beta) {
  return expf(beta * (sqrtf(fmaxf(1.0f - z * z, 0.0f)) - 1.0f));
}
template <>
__device__ __forceinline__ double es_eval<double>(double z, double beta) {
  return exp(beta * (sqrt(fmax(1.0 - z * z, 0.0)) - 1.0));
}

// One CTA owns one tile of one fine grid: accumulates every point record binned to the tile
// in shared memory, then writes the whole tile (zeros included) with coalesced stores.
template <typename T, int DIM, int NT>
__global__ void __launch_bounds__(NT)
    spread_tile_kernel(SpreadArgs a, const typename RecOf<T>::type* __restrict__ recs,
                       const int* __restrict__ idx, const typename Cplx<T>::type* __restrict__ cv,
                       int64_t c_stride, const int* __restrict__ starts, int real_pair,
                       typename Cplx<T>::type* __restrict__ fine) {
  using C = typename Cplx<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int TX = a.tile[0], TY = a.tile[1], TZ = a.tile[2];
  const int cells = TX * TY * TZ;
  const int w = a.w;
  T* acc_re = reinterpret_cast<T*>(smem_raw);
  T* acc_im = acc_re + cells;
  T* ker = acc_im + cells;  // [DIM*w][NT]
  const int tid = threadIdx.x;
  const int64_t key = blockIdx.x;
  const int trans = blockIdx.y;
  const int64_t keygrid = key / a.n_tiles;
  const int64_t tile = key - keygrid * a.n_tiles;
  const int tx = (int)(tile % a.ntile[0]);
  const int ty = (int)((tile / a.ntile[0]) % a.ntile[1]);
  const int tz = (int)(tile / ((int64_t)a.ntile[0] * a.ntile[1]));

  for (int c = tid; c < cells; c += NT) {
    acc_re[c] = (T)0;
    acc_im[c] = (T)0;
  }
  __syncthreads();

  const T beta = (T)a.beta;
  const T two_over_w = (T)(2.0 / w);
  const int r0 = starts[key], r1 = starts[key + 1];
  for (int r = r0 + tid; r < r1; r += NT) {
    const auto rec = recs[r];
    C c;  // a null strength array means unit strengths
    if (cv) {
      c = idx ? cv[(int64_t)trans * c_stride + idx[r]] : cv[r];
    } else {
      c.x = (T)1;
      c.y = (T)0;
    }
    const int lx = (rec.packed & 0xff) - 64;
    const int ly = ((rec.packed >> 8) & 0xff) - 64;
    const int lz = ((rec.packed >> 16) & 0xff) - 64;
    const int comp = (rec.packed >> 24) & 1;
    T* kx = ker + (0 * w) * NT + tid;
    T* ky = ker + (1 * w) * NT + tid;
    T* kz = ker + (2 * w) * NT + tid;
    for (int i = 0; i < w; ++i) {
      kx[i * NT] = es_eval<T>((rec.dx + (T)i) * two_over_w, beta);
      ky[i * NT] = es_eval<T>((rec.dy + (T)i) * two_over_w, beta);
      if (DIM == 3) kz[i * NT] = es_eval<T>((rec.dz + (T)i) * two_over_w, beta);
    }
    const int ax0 = max(0, -lx), ax1 = min(w, TX - lx);
    const int ay0 = max(0, -ly), ay1 = min(w, TY - ly);
    const int az0 = DIM == 3 ? max(0, -lz) : 0;
    const int az1 = DIM == 3 ? min(w, TZ - lz) : 1;
    for (int iz = az0; iz < az1; ++iz) {
      const T vz = DIM == 3 ? kz[iz * NT] : (T)1;
      const int zoff = DIM == 3 ? (lz + iz) * TY : 0;
      for (int iy = ay0; iy < ay1; ++iy) {
        const T vzy = vz * ky[iy * NT];
        const int row = (zoff + ly + iy) * TX + lx;
        if (real_pair) {
          T* dst = comp ? acc_im : acc_re;
          const T s = vzy * c.x;
          for (int ix = ax0; ix < ax1; ++ix) atomicAdd(&dst[row + ix], s * kx[ix * NT]);
        } else {
          const T sr = vzy * c.x, si = vzy * c.y;
          for (int ix = ax0; ix < ax1; ++ix) {
            const T k = kx[ix * NT];
            atomicAdd(&acc_re[row + ix], sr * k);
            atomicAdd(&acc_im[row + ix], si * k);
          }
        }
      }
    }
  }
  __syncthreads();

  C* out = fine + (keygrid + trans) * a.n_fine;
  const int64_t nf0 = a.nf[0], nf1 = a.nf[1];
  const int64_t x0 = (int64_t)tx * TX, y0 = (int64_t)ty * TY, z0 = (int64_t)tz * TZ;
  for (int c = tid; c < cells; c += NT) {
    const int x = c % TX;
    const int y = (c / TX) % TY;
    const int z = c / (TX * TY);
    C v;
    v.x = acc_re[c];
    v.y = acc_im[c];
    out[((z0 + z) * nf1 + (y0 + y)) * nf0 + (x0 + x)] = v;
  }
}

// One CTA owns one tile; each warp takes one record at a time.  The warp's lanes evaluate the
// record's DIM x w kernel values together (one exponential per lane), then cover its support
// with rows of w cells along x (32 / w rows per pass), so that the shared-memory atomics of one
// instruction all go to distinct cells.  Points that coincide — the atoms of a crystal column
// projected onto a Q plane, the case of mp_sqom's (hk0) maps — then no longer make the 32 lanes
// of a warp add to the same cell at once, which the thread-per-record form above serialises.
template <typename T, int DIM, int NT>
__global__ void __launch_bounds__(NT)
    spread_tile_warp_kernel(SpreadArgs a, const typename RecOf<T>::type* __restrict__ recs,
                            const int* __restrict__ idx,
                            const typename Cplx<T>::type* __restrict__ cv, int64_t c_stride,
                            const int* __restrict__ starts, int real_pair,
                            typename Cplx<T>::type* __restrict__ fine) {
  using C = typename Cplx<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int TX = a.tile[0], TY = a.tile[1], TZ = a.tile[2];
  const int cells = TX * TY * TZ;
  const int w = a.w;
  T* acc_re = reinterpret_cast<T*>(smem_raw);
  T* acc_im = acc_re + cells;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  T* ker = acc_im + cells + warp * 48;    // [axis][16]: this warp's record's kernel values
  const int64_t key = blockIdx.x;
  const int trans = blockIdx.y;
  const int64_t keygrid = key / a.n_tiles;
  const int64_t tile = key - keygrid * a.n_tiles;
  const int tx = (int)(tile % a.ntile[0]);
  const int ty = (int)((tile / a.ntile[0]) % a.ntile[1]);
  const int tz = (int)(tile / ((int64_t)a.ntile[0] * a.ntile[1]));
  for (int c = tid; c < cells; c += NT) {
    acc_re[c] = (T)0;
    acc_im[c] = (T)0;
  }
  __syncthreads();
  const T beta = (T)a.beta;
  const T two_over_w = (T)(2.0 / w);
  const int rows = 32 / w;                 // support rows per pass (w <= 16)
  const int li = lane % w, lj = lane / w;  // lanes with lj >= rows stay idle
  const int r0 = starts[key], r1 = starts[key + 1];
  for (int r = r0 + warp; r < r1; r += NT / 32) {
    const auto rec = recs[r];              // one address for the whole warp
    C c;
    if (cv) {
      c = idx ? cv[(int64_t)trans * c_stride + idx[r]] : cv[r];
    } else {
      c.x = (T)1;
      c.y = (T)0;
    }
    for (int l = lane; l < DIM * w; l += 32) {   // DIM w <= 48 values
      const int ax = l / w, i = l - ax * w;
      const T d = ax == 0 ? rec.dx : (ax == 1 ? rec.dy : rec.dz);
      ker[ax * 16 + i] = es_eval<T>((d + (T)i) * two_over_w, beta);
    }
    __syncwarp();
    const int lx = (rec.packed & 0xff) - 64;
    const int ly = ((rec.packed >> 8) & 0xff) - 64;
    const int lz = ((rec.packed >> 16) & 0xff) - 64;
    const int comp = (rec.packed >> 24) & 1;
    const int x = lx + li;
    const bool xin = lj < rows && x >= 0 && x < TX;
    const T kx = ker[li];
    const int nzs = DIM == 3 ? w : 1;
    for (int kz = 0; kz < nzs; ++kz) {
      const int z = DIM == 3 ? lz + kz : 0;
      if (DIM == 3 && (z < 0 || z >= TZ)) continue;        // warp-uniform
      const T vz = DIM == 3 ? ker[32 + kz] : (T)1;
      for (int j0 = 0; j0 < w; j0 += rows) {
        const int j = j0 + lj, y = ly + j;
        if (xin && j < w && y >= 0 && y < TY) {
          const T v = kx * ker[16 + j] * vz;
          const int cell = (z * TY + y) * TX + x;
          if (real_pair) {
            atomicAdd(&(comp ? acc_im : acc_re)[cell], v * c.x);
          } else {
            atomicAdd(&acc_re[cell], v * c.x);
            atomicAdd(&acc_im[cell], v * c.y);
          }
        }
      }
    }
    __syncwarp();                          // ker is rewritten by the warp's next record
  }
  __syncthreads();
  C* out = fine + (keygrid + trans) * a.n_fine;
  const int64_t nf0 = a.nf[0], nf1 = a.nf[1];
  const int64_t x0 = (int64_t)tx * TX, y0 = (int64_t)ty * TY, z0 = (int64_t)tz * TZ;
  for (int c = tid; c < cells; c += NT) {
    const int x = c % TX;
    const int y = (c / TX) % TY;
    const int z = c / (TX * TY);
    C v;
    v.x = acc_re[c];
    v.y = acc_im[c];
    out[((z0 + z) * nf1 + (y0 + y)) * nf0 + (x0 + x)] = v;
  }
}

// FP32, 3D, 16^3 tiles, compile-time kernel width W, no atomics: thread (x, y) of the CTA owns
// the 16-cell z-column (x, y, 0..15) of the tile in registers.  Records are staged in shared
// memory in chunks with their x and y kernel values and their z kernel row already shifted
// into tile coordinates (zeros outside the support); every thread then walks the chunk, and a
// thread inside a record's x-y footprint adds 16 FMAs v * kz_row[z].  Warps whose two y-rows
// miss the footprint skip the record (warp-uniform branch).  The tile is written once with
// coalesced stores.
template <int W>
__global__ void __launch_bounds__(256)
    spread3_f32_w_kernel(SpreadArgs a, const RecF* __restrict__ recs, const int* __restrict__ idx,
                         const float2* __restrict__ cv, int64_t c_stride,
                         const int* __restrict__ starts, int real_pair,
                         float2* __restrict__ fine) {
  constexpr int TL = 16, NT = 256, CH = 256;
  __shared__ __align__(16) float s_kx[CH][8];
  __shared__ __align__(16) float s_ky[CH][8];
  __shared__ __align__(16) float s_kz[CH][TL];
  __shared__ __align__(16) int4 s_meta[CH];     // lx, ly, comp, -
  __shared__ __align__(16) float2 s_str[CH];
  const int tid = threadIdx.x;
  const int x = tid & (TL - 1), y = tid >> 4;
  const int wy0 = (tid >> 5) * 2;  // the two y-rows of this warp: wy0, wy0 + 1
  const int64_t key = blockIdx.x;
  const int trans = blockIdx.y;
  const int keygrid = (int)(key / a.n_tiles);
  const int tile = (int)(key - (int64_t)keygrid * a.n_tiles);
  const int tx = tile % a.ntile[0];
  const int ty = (tile / a.ntile[0]) % a.ntile[1];
  const int tz = tile / (a.ntile[0] * a.ntile[1]);
  float acc_re[TL], acc_im[TL];
#pragma unroll
  for (int z = 0; z < TL; ++z) {
    acc_re[z] = 0.0f;
    acc_im[z] = 0.0f;
  }
  const float beta = (float)a.beta;
  const float s2w = 2.0f / (float)W;
  const int r0 = starts[key], r1 = starts[key + 1];
  for (int c0 = r0; c0 < r1; c0 += CH) {
    const int n = min(CH, r1 - c0);
    if (tid < n) {  // stage one record per thread
      const int r = c0 + tid;
      const RecF rec = recs[r];
      const float2 c = !cv ? make_float2(1.0f, 0.0f) : idx ? cv[(int64_t)trans * c_stride + idx[r]] : cv[r];
      const int lx = (rec.packed & 0xff) - 64;
      const int ly = ((rec.packed >> 8) & 0xff) - 64;
      const int lz = ((rec.packed >> 16) & 0xff) - 64;
      const int comp = (rec.packed >> 24) & 1;
      float kz[W];
#pragma unroll
      for (int i = 0; i < W; ++i) {
        s_kx[tid][i] = es_eval<float>((rec.dx + (float)i) * s2w, beta);
        s_ky[tid][i] = es_eval<float>((rec.dy + (float)i) * s2w, beta);
        kz[i] = es_eval<float>((rec.dz + (float)i) * s2w, beta);
      }
#pragma unroll
      for (int z = 0; z < TL; ++z) {
        float v = 0.0f;
#pragma unroll
        for (int i = 0; i < W; ++i) v = (z - lz == i) ? kz[i] : v;
        s_kz[tid][z] = v;
      }
      s_meta[tid] = make_int4(lx, ly, comp, 0);
      s_str[tid] = c;
    }
    __syncthreads();
    for (int i = 0; i < n; ++i) {
      const int4 m = s_meta[i];
      if (wy0 + 1 < m.y || wy0 >= m.y + W) continue;  // warp-uniform: footprint misses our rows
      const int dx = x - m.x, dy = y - m.y;
      const bool act = (unsigned)dx < (unsigned)W && (unsigned)dy < (unsigned)W;
      const float v = act ? s_kx[i][act ? dx : 0] * s_ky[i][act ? dy : 0] : 0.0f;
      const float2 c = s_str[i];
      const float4* kzr = reinterpret_cast<const float4*>(s_kz[i]);
      if (real_pair) {
        const float vv = v * c.x;
        if (m.z == 0) {
#pragma unroll
          for (int q = 0; q < TL / 4; ++q) {
            const float4 k4 = kzr[q];
            acc_re[4 * q + 0] = fmaf(vv, k4.x, acc_re[4 * q + 0]);
            acc_re[4 * q + 1] = fmaf(vv, k4.y, acc_re[4 * q + 1]);
            acc_re[4 * q + 2] = fmaf(vv, k4.z, acc_re[4 * q + 2]);
            acc_re[4 * q + 3] = fmaf(vv, k4.w, acc_re[4 * q + 3]);
          }
        } else {
#pragma unroll
          for (int q = 0; q < TL / 4; ++q) {
            const float4 k4 = kzr[q];
            acc_im[4 * q + 0] = fmaf(vv, k4.x, acc_im[4 * q + 0]);
            acc_im[4 * q + 1] = fmaf(vv, k4.y, acc_im[4 * q + 1]);
            acc_im[4 * q + 2] = fmaf(vv, k4.z, acc_im[4 * q + 2]);
            acc_im[4 * q + 3] = fmaf(vv, k4.w, acc_im[4 * q + 3]);
          }
        }
      } else {
        const float vr = v * c.x, vi = v * c.y;
#pragma unroll
        for (int q = 0; q < TL / 4; ++q) {
          const float4 k4 = kzr[q];
          acc_re[4 * q + 0] = fmaf(vr, k4.x, acc_re[4 * q + 0]);
          acc_re[4 * q + 1] = fmaf(vr, k4.y, acc_re[4 * q + 1]);
          acc_re[4 * q + 2] = fmaf(vr, k4.z, acc_re[4 * q + 2]);
          acc_re[4 * q + 3] = fmaf(vr, k4.w, acc_re[4 * q + 3]);
          acc_im[4 * q + 0] = fmaf(vi, k4.x, acc_im[4 * q + 0]);
          acc_im[4 * q + 1] = fmaf(vi, k4.y, acc_im[4 * q + 1]);
          acc_im[4 * q + 2] = fmaf(vi, k4.z, acc_im[4 * q + 2]);
          acc_im[4 * q + 3] = fmaf(vi, k4.w, acc_im[4 * q + 3]);
        }
      }
    }
    __syncthreads();
  }
  float2* out = fine + (int64_t)(keygrid + trans) * a.n_fine;
  const int64_t nf0 = a.nf[0], nf1 = a.nf[1];
  const int64_t base = ((int64_t)tz * TL * nf1 + (int64_t)ty * TL + y) * nf0 + (int64_t)tx * TL + x;
#pragma unroll
  for (int z = 0; z < TL; ++z) out[base + (int64_t)z * nf1 * nf0] = make_float2(acc_re[z], acc_im[z]);
}

// Plan API deconvolution: fk[t][mode] = fine[t][k mod nf] / phihat(k), FINUFFT mode order.
template <typename T>
__global__ void deconv_plan_kernel(SpreadArgs a, int64_t m0, int64_t m1, int64_t m2,
                                   const typename Cplx<T>::type* __restrict__ fine,
                                   const T* __restrict__ c0, const T* __restrict__ c1,
                                   const T* __restrict__ c2, typename Cplx<T>::type* __restrict__ fk,
                                   int ntrans) {
  const int64_t nm = m0 * m1 * m2;
  const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= nm * ntrans) return;
  const int64_t t = id / nm;
  const int64_t q = id - t * nm;
  const int64_t i = q % m0, j = (q / m0) % m1, l = q / (m0 * m1);
  const int64_t kx = i - m0 / 2, ky = j - m1 / 2, kz = l - m2 / 2;
  const int64_t sx = (kx + a.nf[0]) % a.nf[0];
  const int64_t sy = (ky + a.nf[1]) % a.nf[1];
  const int64_t sz = (kz + a.nf[2]) % a.nf[2];
  const T f = c0[i] * c1[j] * c2[l];
  auto v = fine[t * a.n_fine + (sz * a.nf[1] + sy) * a.nf[0] + sx];
  v.x *= f;
  v.y *= f;
  fk[id] = v;
}

// In-place radix-2 FFT (length n = 2^logn <= 1024) along `qt` adjacent columns of a row-major
// array with row stride `ld` (elements): column c of the CTA's tile is data[r*ld + col0 + c],
// r = 0..n-1.  qt = 1 with ld = 1 and col0 = row*n transforms a contiguous row instead.
// sign -1: exp(-2 pi i k t/n).  Used where no FFT library plan may be created.
__global__ void fft_radix2_kernel(double2* __restrict__ data, int n, int logn, int64_t ld,
                                  int64_t col_stride_blocks, int qt, int sign) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* xs = reinterpret_cast<double2*>(smem_raw);  // [n][qt]
  double2* tw = xs + (size_t)n * qt;                   // [n/2]
  const int tid = threadIdx.x, NT = blockDim.x;
  const int64_t base = (int64_t)blockIdx.x * col_stride_blocks;
  for (int i = tid; i < n / 2; i += NT) {
    double s_, c_;
    sincospi((double)sign * 2.0 * (double)i / n, &s_, &c_);
    tw[i] = make_double2(c_, s_);
  }
  for (int e = tid; e < n * qt; e += NT) {
    const int r = e / qt, c = e % qt;
    const int rr = (int)(__brev((unsigned)r) >> (32 - logn));
    xs[rr * qt + c] = data[base + (int64_t)r * ld + c];
  }
  __syncthreads();
  for (int s = 0; s < logn; ++s) {
    const int half = 1 << s, stride = n >> (s + 1);
    for (int e = tid; e < (n / 2) * qt; e += NT) {
      const int c = e % qt, b = e / qt;
      const int pos = b & (half - 1);
      const int i = ((b >> s) << (s + 1)) + pos, j = i + half;
      const double2 w = tw[pos * stride];
      const double2 u = xs[i * qt + c], v0 = xs[j * qt + c];
      const double2 v = make_double2(v0.x * w.x - v0.y * w.y, v0.x * w.y + v0.y * w.x);
      xs[i * qt + c] = make_double2(u.x + v.x, u.y + v.y);
      xs[j * qt + c] = make_double2(u.x - v.x, u.y - v.y);
    }
    __syncthreads();
  }
  for (int e = tid; e < n * qt; e += NT) {
    const int r = e / qt, c = e % qt;
    data[base + (int64_t)r * ld + c] = xs[r * qt + c];
  }
}

// ------------------------------------------------------------------------- host helpers
template <typename T>
int launch_scan(const int* counts, int* starts, int64_t n, cudaStream_t s) {
  scan_kernel<<<1, kScanThreads, 0, s>>>(counts, starts, n);
  MPSQ_LAUNCH_CHECK();
  return MPSQ_OK;
}
template int launch_scan<float>(const int*, int*, int64_t, cudaStream_t);
template int launch_scan<double>(const int*, int*, int64_t, cudaStream_t);

template <typename T>
static size_t spread_smem(const SpreadArgs& a, int nt) {
  const size_t cells = (size_t)a.tile[0] * a.tile[1] * a.tile[2];
  return (2 * cells + (size_t)a.dim * a.w * nt) * sizeof(T);
}

template <typename T, int DIM, int NT>
static int launch_spread_impl(const SpreadArgs& a, const typename RecOf<T>::type* recs,
                              const int* idx, const typename Cplx<T>::type* cv, int64_t c_stride,
                              const int* starts, int nkeys, int ntrans, bool real_pair,
                              typename Cplx<T>::type* fine, cudaStream_t s,
                              bool tensor_core = true, bool repro = false) {
  if constexpr (std::is_same<T, float>::value && DIM == 3) {
    if (a.tile[0] == 16 && a.tile[1] == 16 && a.tile[2] == 16 && a.w >= 3 && a.w <= 8) {
      if (real_pair && tensor_core && spread_pair_mma_enabled())
        return launch_spread_pair_mma(a, recs, idx, cv, c_stride, starts, nkeys, ntrans, fine, s,
                                      0, 0, 0, repro);
      dim3 grid((unsigned)nkeys, (unsigned)ntrans);
      const int rp = real_pair ? 1 : 0;
      switch (a.w) {
        case 3: spread3_f32_w_kernel<3><<<grid, 256, 0, s>>>(a, recs, idx, cv, c_stride, starts, rp, fine); break;
        case 4: spread3_f32_w_kernel<4><<<grid, 256, 0, s>>>(a, recs, idx, cv, c_stride, starts, rp, fine); break;
        case 5: spread3_f32_w_kernel<5><<<grid, 256, 0, s>>>(a, recs, idx, cv, c_stride, starts, rp, fine); break;
        case 6: spread3_f32_w_kernel<6><<<grid, 256, 0, s>>>(a, recs, idx, cv, c_stride, starts, rp, fine); break;
        case 7: spread3_f32_w_kernel<7><<<grid, 256, 0, s>>>(a, recs, idx, cv, c_stride, starts, rp, fine); break;
        default: spread3_f32_w_kernel<8><<<grid, 256, 0, s>>>(a, recs, idx, cv, c_stride, starts, rp, fine); break;
      }
      MPSQ_LAUNCH_CHECK();
      return MPSQ_OK;
    }
  }
  dim3 grid((unsigned)nkeys, (unsigned)ntrans);
  if (a.w <= 16 && (DIM == 2 || sizeof(T) == 8)) {
    // warp per record: 2D grids (crystal columns coincide on a Q plane) and FP64 volumes
    constexpr int NTW = 256;
    const size_t smem = (2 * (size_t)a.tile[0] * a.tile[1] * a.tile[2] + (NTW / 32) * 48) * sizeof(T);
    static std::once_flag once_w;
    static cudaError_t attr_w = cudaSuccess;
    std::call_once(once_w, [&] {
      attr_w = cudaFuncSetAttribute(spread_tile_warp_kernel<T, DIM, NTW>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    });
    if (attr_w != cudaSuccess)
      return fail(MPSQ_ERR_CUDA, "spread smem attribute: %s", cudaGetErrorString(attr_w));
    if (smem > 200 * 1024) return fail(MPSQ_ERR_ARG, "spread tile needs %zu B shared memory", smem);
    spread_tile_warp_kernel<T, DIM, NTW><<<grid, NTW, smem, s>>>(a, recs, idx, cv, c_stride,
                                                                starts, real_pair ? 1 : 0, fine);
    MPSQ_LAUNCH_CHECK();
    return MPSQ_OK;
  }
  size_t smem = spread_smem<T>(a, NT);
  static std::once_flag once;
  static cudaError_t attr_err = cudaSuccess;
  std::call_once(once, [&] {
    attr_err = cudaFuncSetAttribute(spread_tile_kernel<T, DIM, NT>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  });
  if (attr_err != cudaSuccess)
    return fail(MPSQ_ERR_CUDA, "spread smem attribute: %s", cudaGetErrorString(attr_err));
  if (smem > 200 * 1024) return fail(MPSQ_ERR_ARG, "spread tile needs %zu B shared memory", smem);
  spread_tile_kernel<T, DIM, NT><<<grid, NT, smem, s>>>(a, recs, idx, cv, c_stride, starts,
                                                        real_pair ? 1 : 0, fine);
  MPSQ_LAUNCH_CHECK();
  return MPSQ_OK;
}

// Spread records binned under keys [0, ngrid*n_tiles) into `ngrid` grids (job pipeline:
// strengths per record, no gather; str == nullptr: every strength is 1).
template <typename T>
int launch_spread(const SpreadArgs& a, const typename RecOf<T>::type* recs,
                  const typename Cplx<T>::type* str, const int* starts, bool real_pair,
                  typename Cplx<T>::type* fine, cudaStream_t s, bool tensor_core, bool repro) {
  constexpr int NT = sizeof(T) == 4 ? 256 : 128;
  int nkeys = (int)(a.n_tiles * a.ngrid);
  if (a.dim == 3)
    return launch_spread_impl<T, 3, NT>(a, recs, nullptr, str, 0, starts, nkeys, 1, real_pair,
                                        fine, s, tensor_core, repro);
  return launch_spread_impl<T, 2, NT>(a, recs, nullptr, str, 0, starts, nkeys, 1, real_pair,
                                      fine, s, tensor_core, repro);
}
template int launch_spread<float>(const SpreadArgs&, const RecF*, const float2*, const int*, bool,
                                  float2*, cudaStream_t, bool, bool);
template int launch_spread<double>(const SpreadArgs&, const RecD*, const double2*, const int*,
                                   bool, double2*, cudaStream_t, bool, bool);

int make_fft_plan(const GridGeom& g, int ngrid, int precision, cudaStream_t s, cufftHandle* h) {
  long long n[3];
  int rank = g.dim;
  if (rank == 3) {
    n[0] = g.nf[2];
    n[1] = g.nf[1];
    n[2] = g.nf[0];
  } else {
    n[0] = g.nf[1];
    n[1] = g.nf[0];
  }
  cufftHandle p;
  MPSQ_CUFFT_TRY(cufftCreate(&p));
  size_t ws = 0;
  cufftResult r = cufftMakePlanMany64(p, rank, n, nullptr, 1, (long long)g.n_fine, nullptr, 1,
                                      (long long)g.n_fine,
                                      precision == MPSQ_FP64 ? CUFFT_Z2Z : CUFFT_C2C, ngrid, &ws);
  if (r != CUFFT_SUCCESS) {
    cufftDestroy(p);
    return fail(MPSQ_ERR_CUFFT, "cufftMakePlanMany(%d x %lld^%d) status %d", ngrid,
                (long long)g.nf[0], rank, (int)r);
  }
  r = cufftSetStream(p, s);
  if (r != CUFFT_SUCCESS) {
    cufftDestroy(p);
    return fail(MPSQ_ERR_CUFFT, "cufftSetStream status %d", (int)r);
  }
  *h = p;
  return MPSQ_OK;
}

int exec_fft(cufftHandle h, int precision, void* data, int direction) {
  if (precision == MPSQ_FP64) {
    MPSQ_CUFFT_TRY(cufftExecZ2Z(h, (cufftDoubleComplex*)data, (cufftDoubleComplex*)data, direction));
  } else {
    MPSQ_CUFFT_TRY(cufftExecC2C(h, (cufftComplex*)data, (cufftComplex*)data, direction));
  }
  return MPSQ_OK;
}

}  // namespace mpsq

// =============================================================================== plan API
using namespace mpsq;

struct mpsq_nufft_plan {
  int dim = 3, iflag = -1, ntrans = 1, precision = MPSQ_FP64;
  double eps = 1e-6;
  cudaStream_t stream = nullptr;
  EsKernel es{};
  GridGeom g{};
  SpreadArgs sa{};
  void* fine = nullptr;
  int* counts = nullptr;
  int* starts = nullptr;
  void* recs = nullptr;
  int* idx = nullptr;
  int64_t cap = 0;
  int64_t nj = -1;
  void* corr[3] = {nullptr, nullptr, nullptr};
  cufftHandle fft = 0;
  bool have_fft = false;
  int* err = nullptr;
};

static void plan_free(mpsq_nufft_plan* p) {
  if (!p) return;
  if (p->have_fft) cufftDestroy(p->fft);
  cudaFree(p->fine);
  cudaFree(p->counts);
  cudaFree(p->starts);
  cudaFree(p->recs);
  cudaFree(p->idx);
  for (int a = 0; a < 3; ++a) cudaFree(p->corr[a]);
  cudaFree(p->err);
  delete p;
}

extern "C" int mpsq_nufft_makeplan(int dim, const int64_t* n_modes, int iflag, int ntrans,
                                   double eps, int precision, void* stream,
                                   mpsq_nufft_plan** plan) {
  if (!plan || !n_modes) return fail(MPSQ_ERR_ARG, "makeplan: null pointer");
  *plan = nullptr;
  if (precision != MPSQ_FP32 && precision != MPSQ_FP64)
    return fail(MPSQ_ERR_ARG, "makeplan: precision must be MPSQ_FP32 or MPSQ_FP64");
  if (ntrans < 1) return fail(MPSQ_ERR_ARG, "makeplan: ntrans must be >= 1");
  auto* p = new mpsq_nufft_plan();
  p->dim = dim;
  p->iflag = iflag;
  p->ntrans = ntrans;
  p->precision = precision;
  p->eps = eps;
  p->stream = (cudaStream_t)stream;
  p->es = es_params(eps, precision);
  int rc = make_geom(dim, n_modes, p->es.w, &p->g);
  if (rc) {
    delete p;
    return rc;
  }
  SpreadArgs& a = p->sa;
  a.dim = dim;
  a.w = p->es.w;
  a.beta = p->es.beta;
  for (int k = 0; k < 3; ++k) {
    a.nf[k] = p->g.nf[k];
    a.tile[k] = p->g.tile[k];
    a.ntile[k] = p->g.ntile[k];
  }
  a.n_tiles = p->g.n_tiles;
  a.n_fine = p->g.n_fine;
  a.ngrid = 1;
  finish_spread_args(a);
  const size_t csz = precision == MPSQ_FP64 ? sizeof(double2) : sizeof(float2);
  const size_t rsz = precision == MPSQ_FP64 ? sizeof(RecD) : sizeof(RecF);
  (void)rsz;
  cudaError_t e;
  e = cudaMalloc(&p->fine, csz * p->g.n_fine * ntrans);
  if (e == cudaSuccess) e = cudaMalloc(&p->counts, sizeof(int) * (p->g.n_tiles + 1));
  if (e == cudaSuccess) e = cudaMalloc(&p->starts, sizeof(int) * (p->g.n_tiles + 1));
  if (e == cudaSuccess) e = cudaMalloc(&p->err, sizeof(int));
  const size_t esz = precision == MPSQ_FP64 ? sizeof(double) : sizeof(float);
  for (int k = 0; k < 3 && e == cudaSuccess; ++k) {
    std::vector<double> c(p->g.m[k]);
    if (k < dim)
      es_correction(p->es, p->g.nf[k], p->g.m[k], c.data());
    else
      c.assign(1, 1.0);
    e = cudaMalloc(&p->corr[k], esz * c.size());
    if (e != cudaSuccess) break;
    if (precision == MPSQ_FP64) {
      e = cudaMemcpy(p->corr[k], c.data(), esz * c.size(), cudaMemcpyHostToDevice);
    } else {
      std::vector<float> cf(c.begin(), c.end());
      e = cudaMemcpy(p->corr[k], cf.data(), esz * c.size(), cudaMemcpyHostToDevice);
    }
  }
  if (e == cudaSuccess) e = cudaMemset(p->err, 0, sizeof(int));
  if (e != cudaSuccess) {
    plan_free(p);
    return fail(e == cudaErrorMemoryAllocation ? MPSQ_ERR_ALLOC : MPSQ_ERR_CUDA,
                "makeplan: %s", cudaGetErrorString(e));
  }
  rc = make_fft_plan(p->g, ntrans, precision, p->stream, &p->fft);
  if (rc) {
    plan_free(p);
    return rc;
  }
  p->have_fft = true;
  *plan = p;
  return MPSQ_OK;
}

template <typename T>
static int plan_setpts_t(mpsq_nufft_plan* p, int64_t nj, const void* x, const void* y,
                         const void* z) {
  const int64_t per = p->dim == 3 ? 8 : 4;
  const int64_t need = std::max<int64_t>(1, nj * per);
  if (need > (int64_t)INT32_MAX) return fail(MPSQ_ERR_ARG, "setpts: too many points (%lld)", (long long)nj);
  if (need > p->cap) {
    cudaFree(p->recs);
    cudaFree(p->idx);
    p->recs = nullptr;
    p->idx = nullptr;
    p->cap = 0;
    MPSQ_CUDA_TRY(cudaMalloc(&p->recs, sizeof(typename RecOf<T>::type) * need));
    MPSQ_CUDA_TRY(cudaMalloc(&p->idx, sizeof(int) * need));
    p->cap = need;
  }
  cudaStream_t s = p->stream;
  const int64_t nkeys = p->g.n_tiles;
  MPSQ_CUDA_TRY(cudaMemsetAsync(p->counts, 0, sizeof(int) * (nkeys + 1), s));
  const int bt = 256;
  const unsigned nb = (unsigned)std::max<int64_t>(1, (nj + bt - 1) / bt);
  auto* recs = (typename RecOf<T>::type*)p->recs;
  if (nj > 0) {
    bin_plan_kernel<T><<<nb, bt, 0, s>>>(nj, (const T*)x, (const T*)y, (const T*)z, p->sa, 0,
                                         p->counts, p->starts, recs, p->idx, p->cap, p->err);
    MPSQ_LAUNCH_CHECK();
  }
  int rc = launch_scan<T>(p->counts, p->starts, nkeys, s);
  if (rc) return rc;
  MPSQ_CUDA_TRY(cudaMemsetAsync(p->counts, 0, sizeof(int) * (nkeys + 1), s));
  if (nj > 0) {
    bin_plan_kernel<T><<<nb, bt, 0, s>>>(nj, (const T*)x, (const T*)y, (const T*)z, p->sa, 1,
                                         p->counts, p->starts, recs, p->idx, p->cap, p->err);
    MPSQ_LAUNCH_CHECK();
  }
  p->nj = nj;
  return MPSQ_OK;
}

extern "C" int mpsq_nufft_setpts(mpsq_nufft_plan* p, int64_t nj, const void* x, const void* y,
                                 const void* z) {
  if (!p) return fail(MPSQ_ERR_ARG, "setpts: null plan");
  if (nj < 0) return fail(MPSQ_ERR_ARG, "setpts: nj < 0");
  if (nj > 0 && (!x || !y || (p->dim == 3 && !z))) return fail(MPSQ_ERR_ARG, "setpts: null coordinates");
  return p->precision == MPSQ_FP64 ? plan_setpts_t<double>(p, nj, x, y, z)
                                   : plan_setpts_t<float>(p, nj, x, y, z);
}

template <typename T>
static int plan_execute_t(mpsq_nufft_plan* p, const void* c, void* fk) {
  using C = typename Cplx<T>::type;
  cudaStream_t s = p->stream;
  SpreadArgs a = p->sa;
  constexpr int NT = sizeof(T) == 4 ? 256 : 128;
  int rc;
  const int nkeys = (int)p->g.n_tiles;
  const auto* recs = (const typename RecOf<T>::type*)p->recs;
  if (p->dim == 3)
    rc = launch_spread_impl<T, 3, NT>(a, recs, p->idx, (const C*)c, p->nj, p->starts, nkeys,
                                      p->ntrans, false, (C*)p->fine, s);
  else
    rc = launch_spread_impl<T, 2, NT>(a, recs, p->idx, (const C*)c, p->nj, p->starts, nkeys,
                                      p->ntrans, false, (C*)p->fine, s);
  if (rc) return rc;
  rc = exec_fft(p->fft, p->precision, p->fine, p->iflag >= 0 ? CUFFT_INVERSE : CUFFT_FORWARD);
  if (rc) return rc;
  const int64_t total = p->g.n_modes * p->ntrans;
  const int bt = 256;
  deconv_plan_kernel<T><<<(unsigned)((total + bt - 1) / bt), bt, 0, s>>>(
      a, p->g.m[0], p->g.m[1], p->g.m[2], (const C*)p->fine, (const T*)p->corr[0],
      (const T*)p->corr[1], (const T*)p->corr[2], (C*)fk, p->ntrans);
  MPSQ_LAUNCH_CHECK();
  return MPSQ_OK;
}

extern "C" int mpsq_nufft_execute(mpsq_nufft_plan* p, const void* c, void* fk) {
  if (!p) return fail(MPSQ_ERR_ARG, "execute: null plan");
  if (p->nj < 0) return fail(MPSQ_ERR_STATE, "execute: setpts not called");
  if (!fk || (p->nj > 0 && !c)) return fail(MPSQ_ERR_ARG, "execute: null array");
  return p->precision == MPSQ_FP64 ? plan_execute_t<double>(p, c, fk)
                                   : plan_execute_t<float>(p, c, fk);
}

extern "C" int mpsq_nufft_destroy(mpsq_nufft_plan* p) {
  plan_free(p);
  return MPSQ_OK;
}

extern "C" int mpsq_nufft_info(const mpsq_nufft_plan* p, int* width, int64_t* fine_grid) {
  if (!p) return fail(MPSQ_ERR_ARG, "info: null plan");
  if (width) *width = p->es.w;
  if (fine_grid)
    for (int k = 0; k < 3; ++k) fine_grid[k] = p->g.nf[k];
  return MPSQ_OK;
}

namespace mpsq {
const int* plan_error_flag(const mpsq_nufft_plan* p) { return p ? p->err : nullptr; }
int dev_error_status(int flag) {
  if (flag & kErrRecOverflow) return fail(MPSQ_ERR_DEVICE, "binning: record capacity exceeded");
  if (flag & kErrBadIndex) return fail(MPSQ_ERR_DEVICE, "kernel bound check failed (flag %d)", flag);
  return MPSQ_OK;
}
}  // namespace mpsq

extern "C" int mpsq_nufft_check_error(mpsq_nufft_plan* p) {
  if (!p) return fail(MPSQ_ERR_ARG, "null plan");
  return check_dev_error(p->err, p->stream);
}

extern "C" const char* mpsq_last_error(void) { return mpsq::t_err; }
extern "C" const char* mpsq_version(void) { return "mpsq 0.1 (sm_103a)"; }
extern "C" int64_t mpsq_launch_count(void) { return mpsq::g_launches.load(); }

// ====================================================== allocation-free 2D type-1 entry point
// For callers that may not allocate device memory during a call (hosts whose device memory is
// handed out by their own pool under a fixed budget, or plug-in hosts that forbid allocation
// inside a call): all scratch of this transform — fine grid, bin counts and offsets, point
// records, correction factors, error flag — lives in one file-scope device array that every
// GPU loading this library holds until the process exits.  Nothing is copied from host memory;
// the call ends by reading the error flag back and synchronising the stream.
namespace {

constexpr int64_t kNoallocMaxPoints = 65536;   // nonuniform points per call
constexpr int64_t kNoallocMaxModes = 256;      // modes per dimension
constexpr int64_t kNoallocMaxFine = 512;       // fine grid per dimension (power of two)
constexpr int kNoallocTile = 32;
constexpr size_t kNoallocScratchBytes = size_t(16) << 20;  // 16 MiB

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

std::mutex g_noalloc_mu;
constexpr int kNoallocMaxDevices = 64;
unsigned char* g_noalloc_base[kNoallocMaxDevices] = {};  // device address, per device ordinal

constexpr size_t al256(size_t b) { return (b + 255) & ~size_t(255); }

constexpr size_t noalloc_bytes(int64_t nf0, int64_t nf1, int64_t nj, int64_t ms, int64_t mt) {
  return al256(sizeof(double2) * nf0 * nf1)                                    // fine grid
         + 2 * al256(sizeof(int) * ((nf0 / kNoallocTile) * (nf1 / kNoallocTile) + 1))  // counts, starts
         + al256(sizeof(mpsq::RecD) * 4 * (nj > 0 ? nj : 1))                    // records
         + al256(sizeof(int) * 4 * (nj > 0 ? nj : 1))                           // source index
         + al256(sizeof(double) * ms) + al256(sizeof(double) * mt) + al256(sizeof(double))
         + al256(sizeof(int));                                                  // error flag
}
static_assert(noalloc_bytes(kNoallocMaxFine, kNoallocMaxFine, kNoallocMaxPoints, kNoallocMaxModes,
                            kNoallocMaxModes) <= kNoallocScratchBytes,
              "scratch array too small for the stated maximum sizes");

int64_t pow2_at_least(int64_t n) {
  int64_t p = 1;
  while (p < n) p <<= 1;
  return p;
}

constexpr int kNoallocMaxQuad = 4 * 16 + 40;   // Gauss-Legendre order for the widest kernel

// Deconvolution factors 1/phihat(k) of both axes, computed on the device into the scratch (the
// quadrature of es_correction: Gauss-Legendre nodes by Newton iteration on P_n, then
// phihat(k) = int_{-w/2}^{w/2} phi(2u/w) cos(2 pi k u / nf) du), so that a call copies nothing
// from host memory.  One CTA; corr2 (the unused third axis) is set to 1.
__global__ void noalloc_corr_kernel(int w, double beta, int64_t nf0, int64_t ms, int64_t nf1,
                                    int64_t mt, double* __restrict__ corr0,
                                    double* __restrict__ corr1, double* __restrict__ corr2) {
  __shared__ double su[kNoallocMaxQuad], sf[kNoallocMaxQuad];
  const int nq = 4 * w + 40;
  const double half = 0.5 * w;
  for (int i = threadIdx.x; i < nq; i += blockDim.x) {
    double z = cospi((i + 0.75) / (nq + 0.5));
    double dp = 1.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= nq; ++k) {
        const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      dp = nq * (z * p1 - p0) / (z * z - 1.0);
      const double dz = p1 / dp;
      z -= dz;
      if (fabs(dz) < 1e-16) break;
    }
    double p0 = 1.0, p1 = z;
    for (int k = 2; k <= nq; ++k) {
      const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
      p0 = p1;
      p1 = p2;
    }
    dp = nq * (z * p1 - p0) / (z * z - 1.0);
    const double wt = 2.0 / ((1.0 - z * z) * dp * dp);
    su[i] = half * z;
    sf[i] = half * wt * exp(beta * (sqrt(fmax(0.0, 1.0 - z * z)) - 1.0));
  }
  __syncthreads();
  for (int64_t i = threadIdx.x; i < ms + mt; i += blockDim.x) {
    const bool first = i < ms;
    const int64_t m = first ? ms : mt, nf = first ? nf0 : nf1;
    const int64_t ii = first ? i : i - ms;
    const double k = (double)(ii - m / 2);
    double s = 0.0;
    for (int q = 0; q < nq; ++q) s += sf[q] * cospi(2.0 * k * su[q] / (double)nf);
    (first ? corr0 : corr1)[ii] = 1.0 / s;
  }
  if (threadIdx.x == 0) *corr2 = 1.0;
}

}  // namespace

// Same transform as finufft2d1 (FP64, FINUFFT mode order) on DEVICE pointers, synchronous on
// `stream`.  The first call on a device looks up the scratch array's device address (set-up,
// done once per device with that device current), so that first call should come before any
// stream capture.  Calls overlapping on the GPU (other host threads, other streams) race on
// the shared scratch and must be serialised by the caller.
extern "C" int mpsq_nufft2d1_noalloc(int64_t nj, const double* x, const double* y,
                                     const double* c, int iflag, double eps, int64_t ms,
                                     int64_t mt, double* fk, void* stream) {
  using namespace mpsq;
  if (nj < 0 || nj > kNoallocMaxPoints)
    return fail(MPSQ_ERR_ARG, "nufft2d1_noalloc: nj = %lld outside 0..%lld (static scratch limit)",
                (long long)nj, (long long)kNoallocMaxPoints);
  if (ms < 1 || mt < 1 || ms > kNoallocMaxModes || mt > kNoallocMaxModes)
    return fail(MPSQ_ERR_ARG, "nufft2d1_noalloc: modes %lld x %lld outside 1..%lld per dimension",
                (long long)ms, (long long)mt, (long long)kNoallocMaxModes);
  if (!fk || (nj > 0 && (!x || !y || !c)))
    return fail(MPSQ_ERR_ARG, "nufft2d1_noalloc: null device pointer");
  cudaStream_t s = (cudaStream_t)stream;
  int dev = 0;
  MPSQ_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kNoallocMaxDevices)
    return fail(MPSQ_ERR_ARG, "nufft2d1_noalloc: device ordinal %d not supported", dev);
  unsigned char* base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_base[dev]) {
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p)
        return fail(MPSQ_ERR_CUDA, "nufft2d1_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
      g_noalloc_base[dev] = (unsigned char*)p;
    }
    base = g_noalloc_base[dev];
  }
  const EsKernel es = es_params(eps, MPSQ_FP64);
  const int64_t nf0 = std::max<int64_t>(kNoallocTile, pow2_at_least(std::max<int64_t>(2 * ms, 2 * es.w)));
  const int64_t nf1 = std::max<int64_t>(kNoallocTile, pow2_at_least(std::max<int64_t>(2 * mt, 2 * es.w)));
  if (nf0 > kNoallocMaxFine || nf1 > kNoallocMaxFine ||
      noalloc_bytes(nf0, nf1, nj, ms, mt) > kNoallocScratchBytes)
    return fail(MPSQ_ERR_ARG, "nufft2d1_noalloc: problem exceeds the static scratch");
  SpreadArgs a{};
  a.dim = 2;
  a.w = es.w;
  a.beta = es.beta;
  a.nf[0] = nf0;
  a.nf[1] = nf1;
  a.nf[2] = 1;
  a.tile[0] = a.tile[1] = kNoallocTile;
  a.tile[2] = 1;
  a.ntile[0] = (int)(nf0 / kNoallocTile);
  a.ntile[1] = (int)(nf1 / kNoallocTile);
  a.ntile[2] = 1;
  a.n_tiles = (int64_t)a.ntile[0] * a.ntile[1];
  a.n_fine = nf0 * nf1;
  a.ngrid = 1;
  finish_spread_args(a);
  const int64_t cap = 4 * std::max<int64_t>(nj, 1);
  // carve the scratch array
  unsigned char* q = base;
  auto take = [&](size_t bytes) {
    unsigned char* r = q;
    q += al256(bytes);
    return r;
  };
  double2* fine = (double2*)take(sizeof(double2) * a.n_fine);
  int* counts = (int*)take(sizeof(int) * (a.n_tiles + 1));
  int* starts = (int*)take(sizeof(int) * (a.n_tiles + 1));
  RecD* recs = (RecD*)take(sizeof(RecD) * cap);
  int* idx = (int*)take(sizeof(int) * cap);
  double* corr0 = (double*)take(sizeof(double) * ms);
  double* corr1 = (double*)take(sizeof(double) * mt);
  double* corr2 = (double*)take(sizeof(double));
  int* err = (int*)take(sizeof(int));
  // deconvolution factors, computed on the device (no copy from host memory)
  if (es.w > 16) return fail(MPSQ_ERR_ARG, "nufft2d1_noalloc: kernel width %d above 16", es.w);
  noalloc_corr_kernel<<<1, 128, 0, s>>>(es.w, es.beta, nf0, ms, nf1, mt, corr0, corr1, corr2);
  MPSQ_LAUNCH_CHECK();
  // the previous call's contents stay in the array: clear what must start at zero
  MPSQ_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), s));
  MPSQ_CUDA_TRY(cudaMemsetAsync(counts, 0, sizeof(int) * (a.n_tiles + 1), s));
  const int bt = 256;
  const unsigned nb = (unsigned)std::max<int64_t>(1, (nj + bt - 1) / bt);
  if (nj > 0) {
    bin_plan_kernel<double><<<nb, bt, 0, s>>>(nj, x, y, nullptr, a, 0, counts, starts, recs, idx, cap, err);
    MPSQ_LAUNCH_CHECK();
  }
  int rc = launch_scan<double>(counts, starts, a.n_tiles, s);
  if (rc) return rc;
  MPSQ_CUDA_TRY(cudaMemsetAsync(counts, 0, sizeof(int) * (a.n_tiles + 1), s));
  if (nj > 0) {
    bin_plan_kernel<double><<<nb, bt, 0, s>>>(nj, x, y, nullptr, a, 1, counts, starts, recs, idx, cap, err);
    MPSQ_LAUNCH_CHECK();
  }
  rc = launch_spread_impl<double, 2, 128>(a, recs, idx, (const double2*)c, nj, starts,
                                          (int)a.n_tiles, 1, false, fine, s);
  if (rc) return rc;
  const int sign = iflag >= 0 ? 1 : -1;
  int l0 = 0, l1 = 0;
  while ((int64_t(1) << l0) < nf0) ++l0;
  while ((int64_t(1) << l1) < nf1) ++l1;
  // rows (length nf0, contiguous), then columns (length nf1, stride nf0), 4 columns per CTA
  fft_radix2_kernel<<<(unsigned)nf1, 256, sizeof(double2) * (nf0 + nf0 / 2), s>>>(fine, (int)nf0, l0, 1, nf0, 1, sign);
  MPSQ_LAUNCH_CHECK();
  fft_radix2_kernel<<<(unsigned)(nf0 / 4), 256, sizeof(double2) * (nf1 * 4 + nf1 / 2), s>>>(fine, (int)nf1, l1, nf0, 4, 4, sign);
  MPSQ_LAUNCH_CHECK();
  const int64_t nm = ms * mt;
  deconv_plan_kernel<double><<<(unsigned)((nm + 255) / 256), 256, 0, s>>>(
      a, ms, mt, 1, fine, corr0, corr1, corr2, (double2*)fk, 1);
  MPSQ_LAUNCH_CHECK();
  return check_dev_error(err, s);
}
