// Internal declarations shared by the CUDA translation units of libmpsq.
#pragma once

#include <cuda_runtime.h>
#include <cufft.h>
#include <nvtx3/nvToolsExt.h>

#include <atomic>
#include <cstdint>
#include <cstdio>

#include "../../include/mpsq.h"

namespace mpsq {
// Host-side NVTX range around the launches of one pipeline phase (sort/bin, spread, fft +
// deconvolution, time transform, reduction), so that a profiler can select a phase's kernels.
// Header-only NVTX: without an attached tool a push/pop costs a few nanoseconds.
struct PhaseRange {
  explicit PhaseRange(const char* name) { nvtxRangePushA(name); }
  ~PhaseRange() { nvtxRangePop(); }
  PhaseRange(const PhaseRange&) = delete;
  PhaseRange& operator=(const PhaseRange&) = delete;
};
}  // namespace mpsq

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
// Smallest fine size >= max(2m, 2w, tile) that is a multiple of tile with factors 2, 3, 5.
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
  double gscale[3];  // nf / (2 pi): radians -> fine-grid units
  double ginv[3];    // 1 / nf
  int tshift[3];     // log2(tile): tiles are powers of two
};

inline void finish_spread_args(SpreadArgs& a) {
  for (int k = 0; k < 3; ++k) {
    a.gscale[k] = (double)a.nf[k] * 0.15915494309189533576888376337251436;
    a.ginv[k] = 1.0 / (double)a.nf[k];
    int sh = 0;
    while ((1 << sh) < a.tile[k]) ++sh;
    a.tshift[k] = sh;
  }
}

// Fold a fine-grid coordinate into [0, nf); NaN / inf give 0 so every index stays in range.
__device__ __forceinline__ double fold_grid(double g, double nf, double inv_nf) {
  g -= nf * floor(g * inv_nf);
  if (g >= nf) g -= nf;
  if (g < 0.0) g += nf;
  if (!(g >= 0.0 && g < nf)) g = 0.0;
  return g;
}

// ---- exact phase reduction in FP32 arithmetic (Dekker product, Knuth sum)
struct F2 {
  float hi, lo;
};
__device__ __forceinline__ F2 two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}
// sum_b r_b (A_hi[b] + A_lo[b]) + (B_hi + B_lo) with ~45-bit accuracy: each product r*A_hi is
// split exactly with an FMA, the hi parts are summed exactly, the small parts in FP32.
__device__ __forceinline__ F2 affine_f2(const float r[3], const float* ahi, const float* alo,
                                        float bhi, float blo) {
  float hi = bhi, lo = blo;
#pragma unroll
  for (int b = 0; b < 3; ++b) {
    const float p = __fmul_rn(r[b], ahi[b]);
    const float pe = fmaf(r[b], ahi[b], -p);
    const F2 s = two_sum(hi, p);
    hi = s.hi;
    lo = __fadd_rn(lo, __fadd_rn(s.lo, fmaf(r[b], alo[b], pe)));
  }
  const F2 s = two_sum(hi, lo);
  return s;
}
// The same for one term: r (A_hi + A_lo) + (B_hi + B_lo), identical to affine_f2 with the
// other two coefficients zero (for finite r).
__device__ __forceinline__ F2 affine1_f2(float r, float ahi, float alo, float bhi, float blo) {
  const float p = __fmul_rn(r, ahi);
  const float pe = fmaf(r, ahi, -p);
  const F2 s = two_sum(bhi, p);
  const float lo = __fadd_rn(blo, __fadd_rn(s.lo, fmaf(r, alo, pe)));
  return two_sum(s.hi, lo);
}
// Folds g = hi + lo into [0, nf) and returns the first support cell s = ceil(g - w/2) and the
// offset d = s - g in [-w/2, -w/2 + 1), both exact up to the FP32 rounding of d.
__device__ __forceinline__ void split_cell_f2(F2 g, int nf, float inv_nf, int w, int* s, float* d) {
  const float fnf = (float)nf;
  const float n = floorf(__fmul_rn(g.hi, inv_nf));
  // remove the integer multiple of nf keeping the result as a hi+lo pair (the shifted value
  // can be larger than g.hi, so a plain FP32 subtraction would round)
  F2 t = two_sum(g.hi, -__fmul_rn(n, fnf));
  t = two_sum(t.hi, __fadd_rn(t.lo, g.lo));
  float gh = t.hi, gl = t.lo;
  if (!(gh == gh) || !(gl == gl) || fabsf(gh) > 4.0f * fnf) {  // NaN / inf input
    gh = 0.0f;
    gl = 0.0f;
  }
  if (__fadd_rn(gh, gl) < 0.0f) {
    t = two_sum(gh, fnf);
    gh = t.hi;
    gl = __fadd_rn(gl, t.lo);
  }
  if (__fadd_rn(gh, gl) >= fnf) {
    t = two_sum(gh, -fnf);
    gh = t.hi;
    gl = __fadd_rn(gl, t.lo);
  }
  const float hw = 0.5f * (float)w;
  float c = ceilf(__fsub_rn(gh, hw));
  float dd = __fsub_rn(__fsub_rn(c, gh), gl);  // c - gh is exact (integer minus nearby float)
  if (dd < -hw) {
    c += 1.0f;
    dd = __fadd_rn(dd, 1.0f);
  } else if (dd >= 1.0f - hw) {
    c -= 1.0f;
    dd = __fsub_rn(dd, 1.0f);
  }
  int si = (int)c;
  // keep the first cell in [-w/2 - 1, nf) whatever the input
  si = si < -w ? -w : (si >= nf ? nf - 1 : si);
  *s = si;
  *d = dd;
}

// Emits the halo copies of one point whose support starts at cell s[k] with offset d[k]:
// one record per tile its w-cell support touches (at most 2 per dimension, periodic, since
// every tile is at least w cells wide; unused dimensions have one tile of one cell).
// Pass 0 (scatter = false) counts records per (grid, tile) key into `cursor`; pass 1 writes
// them at starts[key] + slot, `cursor` having been zeroed between the passes.  The up to 8
// candidate tiles are handled in phases (keys, then all cursor atomics, then all stores) so
// that the atomics' round trips overlap instead of following one another.  Every lane that
// is still running in the warp must call it (the atomics are combined across the warp).
template <typename T>
__device__ __forceinline__ void emit_cells(const SpreadArgs& a, const int s_in[3], const T d_in[3],
                                           int keygrid, int comp, bool scatter, int* cursor,
                                           const int* __restrict__ starts,
                                           typename RecOf<T>::type* recs,
                                           typename Cplx<T>::type* str_out,
                                           typename Cplx<T>::type strength, int* idx_out,
                                           int src_index, int64_t cap, int* err) {
  int tlo[3], two[3], wrap_lo[3], wrap_hi[3], loc_lo[3];
  T d[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    if (k < a.dim) {
      const int s = s_in[k];        // first cell of the support
      const int e = s + a.w - 1;    // last cell
      d[k] = d_in[k];
      tlo[k] = s >> a.tshift[k];    // floor division: >= -1 since s >= -w and tile >= w
      two[k] = (e >> a.tshift[k]) != tlo[k];   // second tile tlo + 1 <= ntile since e < nf + tile
      const int nt = a.ntile[k];
      wrap_lo[k] = tlo[k] < 0 ? tlo[k] + nt : tlo[k];
      wrap_hi[k] = tlo[k] + 1 >= nt ? tlo[k] + 1 - nt : tlo[k] + 1;
      loc_lo[k] = s - (tlo[k] << a.tshift[k]);      // local start in the first tile
    } else {
      d[k] = (T)0;
      tlo[k] = two[k] = wrap_lo[k] = wrap_hi[k] = loc_lo[k] = 0;
    }
  }
  const int64_t gbase = (int64_t)keygrid * a.n_tiles;
  int key[8];   // < ngrid * n_tiles < 2^31
  int slot[8];
  int packed[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const int ix = c & 1, iy = (c >> 1) & 1, iz = c >> 2;
    if ((ix && !two[0]) || (iy && !two[1]) || (iz && !two[2])) continue;
    const int wx = ix ? wrap_hi[0] : wrap_lo[0];
    const int wy = iy ? wrap_hi[1] : wrap_lo[1];
    const int wz = iz ? wrap_hi[2] : wrap_lo[2];
    const int lx = loc_lo[0] - (ix << a.tshift[0]);
    const int ly = loc_lo[1] - (iy << a.tshift[1]);
    const int lz = loc_lo[2] - (iz << a.tshift[2]);
    key[c] = (int)(gbase + ((int64_t)wz * a.ntile[1] + wy) * a.ntile[0] + wx);
    packed[c] = (lx + 64) | ((ly + 64) << 8) | ((lz + 64) << 16) | (comp << 24);
  }
  // Cursor atomics combined per warp: the lanes that share a key take consecutive slots from
  // one atomic of their lowest lane (points in locality order share most keys).
  const unsigned live = __activemask();
  const int lane = threadIdx.x & 31;
  const unsigned below = (1u << lane) - 1u;
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const int ix = c & 1, iy = (c >> 1) & 1, iz = c >> 2;
    const bool has = !((ix && !two[0]) || (iy && !two[1]) || (iz && !two[2]));
    const unsigned act = __ballot_sync(live, has);
    if (has) {
      const unsigned peers = __match_any_sync(act, key[c]);
      const int leader = __ffs(peers) - 1;
      if (!scatter) {
        if (lane == leader) atomicAdd(&cursor[key[c]], __popc(peers));
      } else {
        int base = 0;
        if (lane == leader) base = atomicAdd(&cursor[key[c]], __popc(peers));
        slot[c] = __shfl_sync(peers, base, leader) + __popc(peers & below);
      }
    }
  }
  if (!scatter) return;
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const int ix = c & 1, iy = (c >> 1) & 1, iz = c >> 2;
    if ((ix && !two[0]) || (iy && !two[1]) || (iz && !two[2])) continue;
    const int64_t pos = (int64_t)starts[key[c]] + slot[c];   // key + 1 <= ngrid * n_tiles
    if (pos >= (int64_t)starts[key[c] + 1] || pos >= cap) {
      atomicOr(err, 1);
      continue;
    }
    typename RecOf<T>::type r;
    r.dx = d[0];
    r.dy = d[1];
    r.dz = d[2];
    r.packed = packed[c];
    recs[pos] = r;
    if (str_out) str_out[pos] = strength;
    if (idx_out) idx_out[pos] = src_index;
  }
}

// Same from a folded FP64 fine-grid coordinate g (the FP64 path and the plan API).
template <typename T>
__device__ __forceinline__ void emit_records(const SpreadArgs& a, const double g[3], int keygrid,
                                             int comp, bool scatter, int* cursor,
                                             const int* __restrict__ starts,
                                             typename RecOf<T>::type* recs,
                                             typename Cplx<T>::type* str_out,
                                             typename Cplx<T>::type strength, int* idx_out,
                                             int src_index, int64_t cap, int* err) {
  int s[3] = {0, 0, 0};
  T d[3] = {(T)0, (T)0, (T)0};
#pragma unroll
  for (int k = 0; k < 3; ++k)
    if (k < a.dim) {
      s[k] = (int)ceil(g[k] - 0.5 * a.w);
      d[k] = (T)((double)s[k] - g[k]);
    }
  emit_cells<T>(a, s, d, keygrid, comp, scatter, cursor, starts, recs, str_out, strength, idx_out,
                src_index, cap, err);
}

// ------------------------------------------------------------------ shared kernel helpers
// Launch helpers implemented in nufft.cu, used by the plan API and the job pipeline.
template <typename T>
int launch_scan(const int* counts, int* starts, int64_t n, cudaStream_t s);
template <typename T>
int launch_spread(const SpreadArgs& a, const typename RecOf<T>::type* recs,
                  const typename Cplx<T>::type* str, const int* starts, bool real_pair,
                  typename Cplx<T>::type* fine, cudaStream_t s, bool tensor_core = true,
                  bool repro = false);

// Tensor-core spreading of packed real species pairs (3D, 16^3 tiles, FP32 grid); strengths
// must be real with |s| <= 8.  Selected by default; MPSQ_SPREAD=fma in the environment keeps
// the CUDA-core kernel instead.
bool spread_pair_mma_enabled();
// Keys [key0, key0 + nkeys); a z-slab launch (gstride > 0) writes the tiles' cells at plane
// z - z0 of grids gstride elements apart (otherwise the full grids, n_fine apart).  repro:
// each tile's records are ordered by content before they are accumulated, so that the result
// does not depend on the order they were binned in.
int launch_spread_pair_mma(const SpreadArgs& a, const RecF* recs, const int* idx,
                           const float2* cv, int64_t c_stride, const int* starts, int nkeys,
                           int ntrans, float2* fine, cudaStream_t s, int64_t key0 = 0,
                           int z0 = 0, int64_t gstride = 0, bool repro = false);

// cuFFT plan cache key
int make_fft_plan(const GridGeom& g, int ngrid, int precision, cudaStream_t s, cufftHandle* h);
int exec_fft(cufftHandle h, int precision, void* data, int direction);

// Device error flag helpers (one int per plan / job).  Kernels set bits instead of faulting.
constexpr int kErrRecOverflow = 1;
constexpr int kErrBadIndex = 2;
int check_dev_error(const int* dev_flag, cudaStream_t s);
// The device error flag of a plan (for callers that copy it back with their own results) and
// the status a flag value stands for.
const int* plan_error_flag(const mpsq_nufft_plan* p);
int dev_error_status(int flag);

// View of a job's amplitude store for the time-axis kernels.
struct JobView {
  int precision;
  cudaStream_t s;
  void* cs;            // n_frames x n_q complex, Q fastest
  void* cs_species;    // n_frames x n_species x n_q complex or NULL
  int64_t n_q;         // modes per frame in the store (those of the current Q slab)
  bool slab;           // the store holds a Q slab, not the whole grid
  int32_t n_frames;
  int32_t n_species;
  int64_t m[3];        // modes per dimension
  int store_species;
};
}  // namespace mpsq
struct mpsq_job;
namespace mpsq {
JobView job_view(mpsq_job* j);

}  // namespace mpsq
