// Internal declarations shared by the CUDA translation units of libmpsq.
#pragma once

#include <cuda_runtime.h>
#include <cufft.h>

#include <atomic>
#include <cstdint>
#include <cstdio>

#include "../../include/mpsq.h"

namespace mpsq {

// ---------------------------------------------------------------- errors / bookkeeping
int fail(int code, const char* fmt, ...);          // records the message, returns code
extern std::atomic<int64_t> g_launches;            // kernels launched by this library
inline void count_launch(int n = 1) { g_launches.fetch_add(n, std::memory_order_relaxed); }

#define MPSQ_CUDA_TRY(expr)                                                              \
  do {                                                                                   \
    cudaError_t e_ = (expr);                                                             \
    if (e_ != cudaSuccess)                                                               \
      return ::mpsq::fail(MPSQ_ERR_CUDA, "%s: %s (%s:%d)", #expr, cudaGetErrorString(e_), \
                          __FILE__, __LINE__);                                           \
  } while (0)

#define MPSQ_CUFFT_TRY(expr)                                                             \
  do {                                                                                   \
    cufftResult r_ = (expr);                                                             \
    if (r_ != CUFFT_SUCCESS)                                                             \
      return ::mpsq::fail(MPSQ_ERR_CUFFT, "%s: cufft status %d (%s:%d)", #expr, (int)r_,  \
                          __FILE__, __LINE__);                                           \
  } while (0)

#define MPSQ_LAUNCH_CHECK()                                                              \
  do {                                                                                   \
    ::mpsq::count_launch();                                                              \
    cudaError_t e_ = cudaGetLastError();                                                 \
    if (e_ != cudaSuccess)                                                               \
      return ::mpsq::fail(MPSQ_ERR_CUDA, "kernel launch: %s (%s:%d)",                    \
                          cudaGetErrorString(e_), __FILE__, __LINE__);                   \
  } while (0)

// ------------------------------------------------------------- exponential of semicircle
// Kernel phi(z) = exp(beta (sqrt(1 - z^2) - 1)), |z| <= 1, spread over w fine-grid cells
// (Barnett, Magland, af Klinteberg, SIAM J. Sci. Comput. 41(5) C479 (2019), eq. 1.8 and
// the choice w = ceil(log10(1/eps)) + 1, beta = 2.30 w for upsampling 2).
struct EsKernel {
  int w;          // width in fine-grid cells
  double beta;
};
EsKernel es_params(double eps, int precision);
// 1/phihat(k) for k = -m/2 .. (m-1)/2 on a fine grid of nf cells (Gauss-Legendre quadrature
// of the kernel's Fourier integral).
void es_correction(const EsKernel& es, int64_t nf, int64_t m, double* out);
// Smallest fine size >= max(2m, 2w, tile) that is a multiple of tile with factors 2,3,5,7.
int64_t fine_size(int64_t m, int w, int tile);

// --------------------------------------------------------------------- spreading layout
constexpr int kMaxDim = 3;
constexpr int kTile3 = 16;     // 16^3 fine cells per tile in 3D
constexpr int kTile2 = 32;     // 32^2 fine cells per tile in 2D
constexpr int kSpreadThreads = 256;

struct GridGeom {
  int dim = 3;
  int64_t m[3] = {1, 1, 1};      // modes
  int64_t nf[3] = {1, 1, 1};     // fine grid
  int tile[3] = {1, 1, 1};
  int ntile[3] = {1, 1, 1};
  int64_t n_tiles = 1;           // tiles per grid
  int64_t n_fine = 1;            // cells per grid
  int64_t n_modes = 1;           // modes per transform
};
int make_geom(int dim, const int64_t* m, int w, GridGeom* g);

// Binned point record.  Start cell of the support inside the tile, packed 8 bits per
// dimension with offset 64 (bits 0-7 x, 8-15 y, 16-23 z); bit 24 selects the imaginary
// component for packed real species pairs.  d = start cell - grid coordinate (|d| <= w/2+1).
struct __align__(16) RecF {
  float dx, dy, dz;
  int packed;
};
struct __align__(16) RecD {
  double dx, dy, dz;
  int packed;
  int pad;
};
template <typename T> struct RecOf;
template <> struct RecOf<float> { using type = RecF; };
template <> struct RecOf<double> { using type = RecD; };

template <typename T> struct Cplx;
template <> struct Cplx<float> { using type = float2; };
template <> struct Cplx<double> { using type = double2; };

// Device-side description of a spread/deconvolution problem (passed by value).
struct SpreadArgs {
  int dim;
  int w;
  double beta;
  int64_t nf[3];
  int tile[3];
  int ntile[3];
  int64_t n_tiles;
  int64_t n_fine;
  int ngrid;
};

// ------------------------------------------------------------------ shared kernel helpers
// Launch helpers implemented in nufft.cu, used by the plan API and the job pipeline.
template <typename T>
int launch_scan(const int* counts, int* starts, int64_t n, cudaStream_t s);
template <typename T>
int launch_spread(const SpreadArgs& a, const typename RecOf<T>::type* recs,
                  const typename Cplx<T>::type* str, const int* starts, bool real_pair,
                  typename Cplx<T>::type* fine, cudaStream_t s);

// cuFFT plan cache key
int make_fft_plan(const GridGeom& g, int ngrid, int precision, cudaStream_t s, cufftHandle* h);
int exec_fft(cufftHandle h, int precision, void* data, int direction);

// Device error flag helpers (one int per plan / job).  Kernels set bits instead of faulting.
constexpr int kErrRecOverflow = 1;
constexpr int kErrBadIndex = 2;
int check_dev_error(const int* dev_flag, cudaStream_t s);

// View of a job's amplitude store for the time-axis kernels.
struct JobView {
  int precision;
  cudaStream_t s;
  void* cs;            // n_frames x n_q complex, Q fastest
  void* cs_species;    // n_frames x n_species x n_q complex or NULL
  int64_t n_q;
  int32_t n_frames;
  int32_t n_species;
};
}  // namespace mpsq
struct mpsq_job;
namespace mpsq {
JobView job_view(mpsq_job* j);

}  // namespace mpsq
