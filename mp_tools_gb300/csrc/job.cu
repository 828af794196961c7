// S(Q,omega) job pipeline: the frame loop of mp_sqom (code/src/mp_sqom56.f90:965-1165) on the
// GPU.  Per frame, one kernel selects atoms, computes their NUFFT phases and strengths and
// bins them (mp_sqom56.f90:1100-1143 fused into the binning), one kernel spreads all species
// grids, cuFFT transforms them, and one kernel deconvolves, separates packed species pairs,
// applies the species weights (:1338-1377, weight tables :901-936) and stores the weighted
// amplitude cs(t,Q) of the frame.
#include <cuda_runtime.h>
#include <cufft.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "fft_smem.cuh"
#include "mpsq_internal.h"

namespace mpsq {

// Parameters of the per-point preparation, passed by value.
struct PrepArgs {
  int dim;
  int n_species;
  int64_t species_offset[MPSQ_MAX_SPECIES + 1];
  int group_of[MPSQ_MAX_SPECIES];  // -1: species not transformed (mask 0)
  int comp_of[MPSQ_MAX_SPECIES];   // 0 real / 1 imaginary component in a packed pair
  int input_method;
  int phase_rounding;
  int use_range;
  int bulk_nsuper1;
  int n_row[3];
  double axis[3][3];
  float axis_f[3][3];
  double tpe[3];
  float tpe_f[3];
  double centre[3];
  float centre_f[3];
  double pos_min[3], pos_max[3];
  float pos_min_f[3], pos_max_f[3];
  float tol_f;
  int has_qc;
  double q_center[3];
  float tpq_f[3];  // 2 pi q_center in FP32 (reference rounding)
  int window;
  int pack;
  int64_t n_atoms_frame;
  // FP32 path: fine-grid coordinate g_k = sum_b A_kb r_b + B_k as hi+lo float pairs, and the
  // strength phase in turns q_center . r likewise
  float ahi[3][3], alo[3][3], bhi[3], blo[3];
  float qhi[3], qlo[3];
  float inv_nf[3];
  int nf[3];
  int diag;   // 1: A is diagonal (axis-aligned grid), g_k needs only r_k
};

// Parameters of the fused deconvolution / weighting.
struct WeightArgs {
  int ngroups;
  int pair[MPSQ_MAX_SPECIES];      // per group: 1 if it holds two species
  int sp_a[MPSQ_MAX_SPECIES];      // species in the real component (or the only one)
  int sp_b[MPSQ_MAX_SPECIES];      // species in the imaginary component
  int weight_mode;
  double b_coh[MPSQ_MAX_SPECIES];  // evaluated in the job's precision
  double xff[MPSQ_MAX_SPECIES][9];
  double kappa;                     // |Q|^2 -> exponent scale of the form factor
  double q0[3];
  double qs[3][3];
  double extra_sq;
  double wnorm;
  int store_species;
  int n_species;
  // FP32 copies (the FP32 path must not convert from double per element: FP64 pipe)
  float b_coh_f[MPSQ_MAX_SPECIES];
  float xff_f[MPSQ_MAX_SPECIES][9];
  float kappa_f, q0_f[3], qs_f[3][3], extra_f, wnorm_f;
  float xb2_f[MPSQ_MAX_SPECIES][4];  // Cromer-Mann b_i log2(e): exp(-b_i s2) = 2^(-b_i log2(e) s2)
};

template <typename T>
struct WP;  // typed views of WeightArgs
template <>
struct WP<float> {
  static __device__ __forceinline__ float b(const WeightArgs& w, int s) { return w.b_coh_f[s]; }
  static __device__ __forceinline__ float x(const WeightArgs& w, int s, int i) { return w.xff_f[s][i]; }
  static __device__ __forceinline__ float kappa(const WeightArgs& w) { return w.kappa_f; }
  static __device__ __forceinline__ float q0(const WeightArgs& w, int b) { return w.q0_f[b]; }
  static __device__ __forceinline__ float qs(const WeightArgs& w, int k, int b) { return w.qs_f[k][b]; }
  static __device__ __forceinline__ float extra(const WeightArgs& w) { return w.extra_f; }
  static __device__ __forceinline__ float wnorm(const WeightArgs& w) { return w.wnorm_f; }
};
template <>
struct WP<double> {
  static __device__ __forceinline__ double b(const WeightArgs& w, int s) { return w.b_coh[s]; }
  static __device__ __forceinline__ double x(const WeightArgs& w, int s, int i) { return w.xff[s][i]; }
  static __device__ __forceinline__ double kappa(const WeightArgs& w) { return w.kappa; }
  static __device__ __forceinline__ double q0(const WeightArgs& w, int b) { return w.q0[b]; }
  static __device__ __forceinline__ double qs(const WeightArgs& w, int k, int b) { return w.qs[k][b]; }
  static __device__ __forceinline__ double extra(const WeightArgs& w) { return w.extra_sq; }
  static __device__ __forceinline__ double wnorm(const WeightArgs& w) { return w.wnorm; }
};

}  // namespace mpsq

using namespace mpsq;

struct mpsq_job {
  mpsq_job_desc d{};
  cudaStream_t s = nullptr;
  EsKernel es{};
  GridGeom g{};
  SpreadArgs sa{};
  PrepArgs pa{};
  WeightArgs wa{};
  int ngroups = 0;
  float4* traj = nullptr;
  int4* at_ind = nullptr;
  void* fine = nullptr;
  int* counts = nullptr;
  int* starts = nullptr;
  // locality order of the atoms (rebuilt from the first frame of each multi-frame transform)
  int* perm = nullptr;
  int* perm_counts = nullptr;
  int* perm_starts = nullptr;
  bool perm_built = false;
  void* recs = nullptr;
  void* str = nullptr;
  int64_t cap = 0;
  void* corr[3] = {nullptr, nullptr, nullptr};
  void* cs = nullptr;
  void* cs_species = nullptr;
  cufftHandle fft = 0;
  bool have_fft = false;
  // volumes on cuFFT: x transforms over every row, then (z, y) transforms of the kept x columns
  cufftHandle xfft[3] = {0, 0, 0};   // x rows; (z, y) of columns [0, h0]; of [n0 - h0, n0)
  int xfft_h0 = 0;
  bool have_xfft = false;
  int* err = nullptr;
  bool profile = false;
  cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  double stage_ms[4] = {0, 0, 0, 0};
  int64_t stage_frames = 0;
  // pruned fine-grid transform (FP32, 3D)
  bool pruned = false;
  float2* tw[3] = {nullptr, nullptr, nullptr};
  float2* b1 = nullptr;
  int h[3] = {0, 0, 0}, K[3] = {1, 1, 1};
  // second frame lane (pruned FP32 path): its own stream and per-frame scratch, so that two
  // frames are in flight at once and their latency-bound kernels overlap
  bool lane2 = false;
  cudaStream_t s2 = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  void* fine2 = nullptr;
  int* counts2 = nullptr;
  int* starts2 = nullptr;
  void* recs2 = nullptr;
  void* str2 = nullptr;
  // per-atom preparation of the FP32 split path (counting pass -> scatter pass), per lane
  void* prep = nullptr;
  void* prep2 = nullptr;
  float2* b1_2 = nullptr;
  // one-phonon mode: displacement fields (n_species x 2 x n_row2 x n_row1, job precision)
  void* oneph_u = nullptr;
  float* oneph_base = nullptr;
  cufftHandle oneph_fft = 0;
  bool have_oneph_fft = false;
  int n_alloc = 0;  // device allocations made so far (fault injection below)
  // run-time choices (mpsq_job_set_option / mpsq_job_autotune)
  int opt_graph = 0;        // replay the frame loop of a transform call as a captured graph
  int opt_spread = 0;       // 0: tensor-core spreading of real pairs, 1: CUDA-core kernel
  int opt_xrows = 8;        // rows per CTA of the pruned X pass (4 or 8)
  int opt_zslab = 0;        // fine-grid planes per slab of the spread/X/Y pipeline (0: whole)
  int opt_repro = 0;        // 1: tensor-core spreading orders each tile's records by content
  int opt_lanes = 2;        // frame lanes used when a second lane exists (1 or 2)
  struct Graph {
    int32_t first, count;
    cudaGraphExec_t exec;
    int64_t launches;
  };
  std::vector<Graph> graphs;  // captured frame loops, by (first, count)
  // Q slab (q_slab > 0): the store holds kz planes [slab_z0, slab_z0 + slab_planes())
  int64_t slab_nz = 0;
  int64_t slab_z0 = 0;
  int64_t slab_planes() const { return slab_nz ? std::min(slab_nz, g.m[2] - slab_z0) : g.m[2]; }
  int64_t store_modes() const { return g.m[0] * g.m[1] * slab_planes(); }
};

// Device memory of a job: stream-ordered (from the device's memory pool, on the job's stream)
// when the job was created with stream_ordered = 1, plain otherwise.
// Host-side fault injection for tests of the error paths: with MPSQ_FAIL_ALLOC=k in the
// environment the k-th device allocation of every job reports cudaErrorMemoryAllocation
// without calling the allocator.
static bool injected_alloc_failure(mpsq_job* j) {
  const char* e = getenv("MPSQ_FAIL_ALLOC");
  return e && ++j->n_alloc == atoi(e);
}
static cudaError_t job_alloc(mpsq_job* j, void** ptr, size_t bytes) {
  if (injected_alloc_failure(j)) {
    *ptr = nullptr;
    return cudaErrorMemoryAllocation;
  }
  bytes = std::max<size_t>(bytes, 16);
  return j->d.stream_ordered ? cudaMallocAsync(ptr, bytes, j->s) : cudaMalloc(ptr, bytes);
}
static void job_release(mpsq_job* j, void* ptr) {
  if (!ptr) return;
  if (j->d.stream_ordered)
    cudaFreeAsync(ptr, j->s);
  else
    cudaFree(ptr);
}
static cudaError_t job_upload(mpsq_job* j, void* dst, const void* src, size_t bytes) {
  // pageable source: the copy is staged before the call returns
  return j->d.stream_ordered ? cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, j->s)
                             : cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice);
}

namespace mpsq {

// Selection, phases and strengths of one atom of one frame (mp_sqom56.f90:1104-1142): false
// for an atom that is not transformed; otherwise its grid, pair component and strength and
// either its first support cell and offset (FP32 split path) or its folded fine-grid
// coordinate (FP64 and phase-rounding paths).
template <typename T>
struct PointPrep {
  int grid, comp;
  bool split;
  int sc[3];
  float dc[3];
  double g[3];
  typename Cplx<T>::type c;
};

template <typename T>
__device__ __forceinline__ bool prep_point(const float4* __restrict__ frame,
                                           const int4* __restrict__ at_ind, const PrepArgs& p,
                                           const SpreadArgs& a, int64_t j, PointPrep<T>& o) {
  int s = 0;
  while (s + 1 < p.n_species && j >= p.species_offset[s + 1]) ++s;
  if (j < p.species_offset[0] || j >= p.species_offset[p.n_species]) return false;
  const int grid = p.group_of[s];
  if (grid < 0) return false;
  const float4 r = frame[j];
  if (p.input_method == MPSQ_CELL) {
    if (r.x == 0.0f && r.y == 0.0f && r.z == 0.0f) return false;  // vacancy (:1107)
    if (p.use_range && at_ind) {
      const int4 ci = at_ind[j];
      const int c3[3] = {ci.x, ci.y, ci.z};
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const int c = c3[k] - p.n_row[k] / 2 - 1;
        if ((float)c < p.pos_min_f[k] || (float)c > p.pos_max_f[k]) return false;  // (:1109-1111)
      }
    }
  } else {
    const float rr[3] = {r.x, r.y, r.z};
#pragma unroll
    for (int k = 0; k < 3; ++k)  // (:1121-1128)
      if (!(rr[k] >= p.pos_min_f[k] - p.tol_f && rr[k] < p.pos_max_f[k] + p.tol_f)) return false;
  }
  if constexpr (sizeof(T) == 4) {
    if (!p.phase_rounding) {
      // FP32 split precision: exact phase reduction in two-float arithmetic (no FP64 pipe)
      const float rf[3] = {r.x, r.y, r.z};
      int* const sc = o.sc;
      float* const dc = o.dc;
      for (int k = 0; k < 3; ++k) {
        sc[k] = 0;
        dc[k] = 0.0f;
      }
#pragma unroll
      for (int k = 0; k < 3; ++k) {  // unrolled: sc, dc stay in registers
        if (k < p.dim) {
          // (the zero off-diagonal terms of an axis-aligned grid add exactly nothing)
          const F2 gk = p.diag ? affine1_f2(rf[k], p.ahi[k][k], p.alo[k][k], p.bhi[k], p.blo[k])
                               : affine_f2(rf, p.ahi[k], p.alo[k], p.bhi[k], p.blo[k]);
          split_cell_f2(gk, p.nf[k], p.inv_nf[k], a.w, &sc[k], &dc[k]);
        }
      }
      float2 c = make_float2(1.0f, 0.0f);
      if (p.has_qc) {
        const F2 t = affine_f2(rf, p.qhi, p.qlo, 0.0f, 0.0f);
        const float fl = floorf(t.hi);
        const float fr = __fadd_rn(__fsub_rn(t.hi, fl), t.lo);
        float sn, cn;
        sincospif(2.0f * fr, &sn, &cn);
        c = make_float2(cn, -sn);
      }
      if (p.window) {  // spatial Hann window (1+cos x)(1+cos y) (:1118)
        const int nw = p.dim == 2 ? 2 : 3;
        float f = 1.0f;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          if (k >= nw) break;
          float pr = 0.0f;
#pragma unroll
          for (int b = 0; b < 3; ++b) pr = fmaf(p.axis_f[k][b], rf[b] - p.centre_f[b], pr);
          f *= 1.0f + cosf(pr * p.tpe_f[k]);
        }
        c.x *= f;
        c.y *= f;
      }
      o.comp = p.pack ? p.comp_of[s] : 0;
      if (p.pack && c.x == 0.0f) return false;
      o.grid = grid;
      o.split = true;
      o.c.x = (T)c.x;
      o.c.y = (T)c.y;
      return true;
    }
  }
  double x[3] = {0.0, 0.0, 0.0};
  double g[3] = {0.0, 0.0, 0.0};
  const double rd[3] = {(double)r.x, (double)r.y, (double)r.z};
  const float rf[3] = {r.x, r.y, r.z};
  for (int k = 0; k < p.dim; ++k) {
    if (p.phase_rounding) {
      // FP32 dot product and FP32 scale as the reference computes xf, yf (:1115-1116)
      float pr = 0.0f;
      for (int b = 0; b < 3; ++b) pr = __fadd_rn(pr, __fmul_rn(p.axis_f[k][b], __fsub_rn(rf[b], p.centre_f[b])));
      x[k] = (double)__fmul_rn(pr, p.tpe_f[k]);
    } else {
      double pr = 0.0;
      for (int b = 0; b < 3; ++b) pr += p.axis[k][b] * (rd[b] - p.centre[b]);
      x[k] = pr * p.tpe[k];
    }
    g[k] = fold_grid(x[k] * a.gscale[k], (double)a.nf[k], a.ginv[k]);
  }
  typename Cplx<T>::type c;
  if (p.has_qc) {
    if (p.phase_rounding) {
      float arg = 0.0f;
      for (int b = 0; b < 3; ++b) arg = __fadd_rn(arg, __fmul_rn(p.tpq_f[b], rf[b]));
      // the argument carries the reference's FP32 rounding; the exponential itself is
      // evaluated in the job's precision
      if (sizeof(T) == 8) {
        double sn, cn;
        sincos((double)arg, &sn, &cn);
        c.x = (T)cn;
        c.y = (T)(-sn);
      } else {
        float sn, cn;
        sincosf(arg, &sn, &cn);
        c.x = (T)cn;
        c.y = (T)(-sn);
      }
    } else {
      double turns = 0.0;
      for (int b = 0; b < 3; ++b) turns += p.q_center[b] * rd[b];
      turns -= floor(turns);
      if (sizeof(T) == 8) {
        double sn, cn;
        sincospi(2.0 * turns, &sn, &cn);
        c.x = (T)cn;
        c.y = (T)(-sn);
      } else {
        float sn, cn;
        sincospif((float)(2.0 * turns), &sn, &cn);
        c.x = (T)cn;
        c.y = (T)(-sn);
      }
    }
  } else {
    c.x = (T)1;
    c.y = (T)0;
  }
  if (p.window) {  // spatial Hann window (1+cos x)(1+cos y) (:1118)
    const int nw = p.dim == 2 ? 2 : 3;
    T f = (T)1;
    for (int k = 0; k < nw; ++k) f *= (T)1 + (T)cos(x[k]);
    c.x *= f;
    c.y *= f;
  }
  o.comp = p.pack ? p.comp_of[s] : 0;
  if (p.pack && c.x == (T)0) return false;  // zero strength contributes nothing
  o.grid = grid;
  o.split = false;
  o.c = c;
  for (int k = 0; k < 3; ++k) o.g[k] = g[k];
  return true;
}

// Binning of one frame.  Pass 0 (kScatter false) counts, pass 1 scatters; str == nullptr:
// unit strengths (no centre phase, no window), which are not stored.  Thread i takes atom
// perm[i] (a locality order, so that a warp's atoms share tiles and its cursor atomics
// combine) or atom i without a permutation.
template <typename T, bool kScatter>
__global__ void job_bin_kernel(const float4* __restrict__ frame, const int4* __restrict__ at_ind,
                               const int* __restrict__ perm, PrepArgs p, SpreadArgs a,
                               int* cursor, const int* __restrict__ starts,
                               typename RecOf<T>::type* recs, typename Cplx<T>::type* str,
                               int64_t cap, int* err) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n_atoms_frame) return;
  const int64_t j = perm ? perm[i] : i;
  PointPrep<T> q;
  if (!prep_point<T>(frame, at_ind, p, a, j, q)) return;
  if constexpr (sizeof(T) == 4) {
    if (q.split) {
      const float2 c = make_float2(q.c.x, q.c.y);
      emit_cells<float>(a, q.sc, q.dc, q.grid, q.comp, kScatter, cursor, starts, (RecF*)recs,
                        (float2*)str, c, nullptr, 0, cap, err);
      return;
    }
  }
  emit_records<T>(a, q.g, q.grid, q.comp, kScatter, cursor, starts, recs, str, q.c, nullptr, 0,
                  cap, err);
}

// FP32 split path in two passes that prepare each atom once.  Pass 0 runs the selection, the
// exact two-float cell split and the strength, keeps the result per atom (in locality order:
// coalesced) and counts the atom's records per tile; pass 1 reads it back and writes the
// records.  Per atom: int4 {s0 | s1 << 16, s2 | grid << 16 | comp << 24, d0, d1} (y = -1: not
// transformed), d2, and the strength when strengths are not all 1.
struct PrepCache {
  int4* cell;
  float* d2;
  float2* c;   // null: unit strengths
};

__device__ __forceinline__ int low16_signed(int v) { return (v & 0xffff) - ((v & 0x8000) << 1); }

__global__ void job_bin_count_split_kernel(const float4* __restrict__ frame,
                                           const int4* __restrict__ at_ind,
                                           const int* __restrict__ perm, PrepArgs p, SpreadArgs a,
                                           int* cursor, PrepCache pc, int* err) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n_atoms_frame) return;
  const int64_t j = perm ? perm[i] : i;
  PointPrep<float> q;
  if (!prep_point<float>(frame, at_ind, p, a, j, q) || !q.split) {
    pc.cell[i] = make_int4(0, -1, 0, 0);
    return;
  }
  pc.cell[i] = make_int4((int)(((unsigned)q.sc[0] & 0xffffu) | ((unsigned)q.sc[1] << 16)),
                         (int)(((unsigned)q.sc[2] & 0xffffu) | ((unsigned)q.grid << 16) |
                               ((unsigned)q.comp << 24)),
                         __float_as_int(q.dc[0]), __float_as_int(q.dc[1]));
  pc.d2[i] = q.dc[2];
  if (pc.c) pc.c[i] = make_float2(q.c.x, q.c.y);
  emit_cells<float>(a, q.sc, q.dc, q.grid, q.comp, false, cursor, nullptr, nullptr, nullptr,
                    make_float2(0.f, 0.f), nullptr, 0, 0, err);
}

__global__ void job_bin_scatter_split_kernel(int64_t n, PrepCache pc, SpreadArgs a, int* cursor,
                                             const int* __restrict__ starts,
                                             RecF* __restrict__ recs, float2* __restrict__ str,
                                             int64_t cap, int* err) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int4 r = __ldcs(pc.cell + i);
  if (r.y == -1) return;
  const int sc[3] = {low16_signed(r.x), r.x >> 16, low16_signed(r.y)};
  const float dc[3] = {__int_as_float(r.z), __int_as_float(r.w), __ldcs(pc.d2 + i)};
  const float2 c = pc.c ? __ldcs(pc.c + i) : make_float2(1.f, 0.f);
  emit_cells<float>(a, sc, dc, (r.y >> 16) & 0xff, (r.y >> 24) & 0x7f, true, cursor, starts,
                    recs, str, c, nullptr, 0, cap, err);
}

// Locality order of the atoms of one frame: a counting sort by the tile of each atom's first
// support cell (atoms that are not transformed go to a last bucket, key nkeys).  Pass 0
// counts, pass 1 writes perm[starts[key] + slot] = atom.
template <typename T, bool kScatter>
__global__ void job_perm_kernel(const float4* __restrict__ frame, const int4* __restrict__ at_ind,
                                PrepArgs p, SpreadArgs a, int64_t nkeys, int* cursor,
                                const int* __restrict__ starts, int* __restrict__ perm) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= p.n_atoms_frame) return;
  PointPrep<T> q;
  int64_t key = nkeys;
  if (prep_point<T>(frame, at_ind, p, a, j, q)) {
    int t[3] = {0, 0, 0};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      if (k < a.dim) {
        const int c = q.split ? q.sc[k] : (int)ceil(q.g[k] - 0.5 * a.w);
        int tk = c >> a.tshift[k];
        tk = tk < 0 ? tk + a.ntile[k] : (tk >= a.ntile[k] ? tk - a.ntile[k] : tk);
        t[k] = tk;
      }
    }
    key = (int64_t)q.grid * a.n_tiles + ((int64_t)t[2] * a.ntile[1] + t[1]) * a.ntile[0] + t[0];
  }
  if constexpr (!kScatter) {
    atomicAdd(&cursor[key], 1);
  } else {
    const int slot = atomicAdd(&cursor[key], 1);
    perm[starts[key] + slot] = (int)j;
  }
}

// 2^x on the special-function unit (PTX ex2.approx, relative error of order 2^-22; results
// below the normal range flush to zero).
__device__ __forceinline__ float ex2_sfu(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// Species weight at s2 = kappa (|Q|^2 + extra) (mp_sqom56.f90:919-931): b_coh (neutron) or
// the Cromer-Mann factor c + sum_i a_i exp(-b_i s2) (X-ray).  The FP32 path takes each
// exponential as 2^(-(b_i log2 e) s2) on the SFU: one multiply and one SFU operation per term,
// with an error below the FP32 rounding of s2 that feeds it.
template <typename T>
__device__ __forceinline__ T species_weight(const WeightArgs& w, int s, T s2) {
  if (w.weight_mode == MPSQ_WEIGHT_NEUTRON) return WP<T>::b(w, s);
  if (w.weight_mode == MPSQ_WEIGHT_XRAY) {
    if constexpr (sizeof(T) == 4) {
      float f = w.xff_f[s][8];
#pragma unroll
      for (int i = 0; i < 4; ++i) f = fmaf(w.xff_f[s][2 * i], ex2_sfu(-w.xb2_f[s][i] * s2), f);
      return f;
    }
    T f = WP<T>::x(w, s, 8);
    for (int i = 0; i < 4; ++i) f += WP<T>::x(w, s, 2 * i) * exp(-WP<T>::x(w, s, 2 * i + 1) * s2);
    return f;
  }
  return (T)1;
}

// Deconvolution, pair separation, species weighting; writes cs(t, Q) for one frame.
// Grid: x over the m0 modes of a row, y over the m1 rows, z over the nz planes z0.. of the
// store's Q slab (the whole grid: z0 = 0, nz = m2; 32-bit index math).
template <typename T>
__global__ void job_deconv_kernel(SpreadArgs a, int m0, int m1, int m2, int z0, int nz,
                                  const typename Cplx<T>::type* __restrict__ fine,
                                  const T* __restrict__ c0, const T* __restrict__ c1,
                                  const T* __restrict__ c2, WeightArgs w,
                                  typename Cplx<T>::type* __restrict__ cs_frame,
                                  typename Cplx<T>::type* __restrict__ cs_species_frame) {
  using C = typename Cplx<T>::type;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m0) return;
  const int j = blockIdx.y, l = z0 + (int)blockIdx.z;   // kz plane of the slab
  const int row = (int)blockIdx.z * m1 + j;               // row of the store
  const int64_t nm = (int64_t)m0 * m1 * nz;
  const int64_t q = (int64_t)row * m0 + i;
  const int kx = i - m0 / 2, ky = j - m1 / 2, kz = l - m2 / 2;
  const int nf0 = (int)a.nf[0], nf1 = (int)a.nf[1], nf2 = (int)a.nf[2];
  // fine-grid positions of mode k and of -k (periodic)
  const int sx = kx < 0 ? kx + nf0 : kx, sy = ky < 0 ? ky + nf1 : ky, sz = kz < 0 ? kz + nf2 : kz;
  const int mx = kx > 0 ? nf0 - kx : -kx, my = ky > 0 ? nf1 - ky : -ky, mz = kz > 0 ? nf2 - kz : -kz;
  const int64_t src = ((int64_t)sz * nf1 + sy) * nf0 + sx;
  const int64_t srcm = ((int64_t)mz * nf1 + my) * nf0 + mx;
  const T corr = c0[i] * c1[j] * c2[l];
  T s2 = 0;
  if (w.weight_mode == MPSQ_WEIGHT_XRAY) {
    T qv[3];
    for (int b = 0; b < 3; ++b)
      qv[b] = WP<T>::q0(w, b) + (T)kx * WP<T>::qs(w, 0, b) + (T)ky * WP<T>::qs(w, 1, b) +
              (T)kz * WP<T>::qs(w, 2, b);
    s2 = WP<T>::kappa(w) * (qv[0] * qv[0] + qv[1] * qv[1] + qv[2] * qv[2] + WP<T>::extra(w));
  }
  T accr = 0, acci = 0;
  for (int gi = 0; gi < w.ngroups; ++gi) {
    const C G = fine[gi * a.n_fine + src];
    if (w.pair[gi]) {
      const C Gm = fine[gi * a.n_fine + srcm];
      const T ar = (T)0.5 * (G.x + Gm.x) * corr, ai = (T)0.5 * (G.y - Gm.y) * corr;
      const T br = (T)0.5 * (G.y + Gm.y) * corr, bi = (T)(-0.5) * (G.x - Gm.x) * corr;
      const int sa = w.sp_a[gi], sb = w.sp_b[gi];
      const T wa = species_weight<T>(w, sa, s2), wb = species_weight<T>(w, sb, s2);
      accr += wa * ar + wb * br;
      acci += wa * ai + wb * bi;
      if (w.store_species) {
        C va, vb;
        va.x = ar * WP<T>::wnorm(w);
        va.y = ai * WP<T>::wnorm(w);
        vb.x = br * WP<T>::wnorm(w);
        vb.y = bi * WP<T>::wnorm(w);
        cs_species_frame[(int64_t)sa * nm + q] = va;
        cs_species_frame[(int64_t)sb * nm + q] = vb;
      }
    } else {
      const int sa = w.sp_a[gi];
      const T wa = species_weight<T>(w, sa, s2);
      accr += wa * G.x * corr;
      acci += wa * G.y * corr;
      if (w.store_species) {
        C va;
        va.x = G.x * corr * WP<T>::wnorm(w);
        va.y = G.y * corr * WP<T>::wnorm(w);
        cs_species_frame[(int64_t)sa * nm + q] = va;
      }
    }
  }
  C out;
  out.x = accr * WP<T>::wnorm(w);
  out.y = acci * WP<T>::wnorm(w);
  cs_frame[q] = out;
}

// -------------------------------------------------------------------- one-phonon mode
// mp_sqom's j_oneph = 1 branch (code/src/mp_sqom56.f90:1037-1098): per species, the in-plane
// displacements of the atoms are summed over the cell columns of the plane into two real
// fields u_x(k, l), u_y(k, l) on the n_row x n_row cell grid, Fourier transformed (forward,
// exp(-i), unscaled) and divided by n_row, and every Q pixel of the n_bz x n_bz zones takes
// A_j(Q) = exp(-2 pi i q . b_j) (q_x u_qx + q_y u_qy) at the zone-folded cell frequency.
// Plane 1 is (hk0): k, l = cell indices 1, 2, d = r - b - cell + n_row/2.  Plane 2 is (hhl):
// k = mod(c1 - 1 + c2 - 1, n_row) + 1, l = c3, d_x = (d1 + d2 + 2)/sqrt 2, d_y = d3 + 1
// (the reference's "+1" on this plane kept).  Displacements in FP32 in the reference's order.

// u: [n_species][2][n2][n1] complex, zeroed; atoms at exactly (0,0,0) are vacancies (:1049).
template <typename T>
__global__ void oneph_scatter_kernel(const float4* __restrict__ frame, const int4* __restrict__ at_ind,
                                     PrepArgs p, int plane, const float* __restrict__ base,
                                     int n1, int n2, typename Cplx<T>::type* __restrict__ u) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= p.n_atoms_frame) return;
  if (j < p.species_offset[0] || j >= p.species_offset[p.n_species]) return;
  int s = 0;
  while (s + 1 < p.n_species && j >= p.species_offset[s + 1]) ++s;
  if (p.group_of[s] < 0) return;  // masked species are not transformed
  const float4 r = frame[j];
  if (r.x == 0.0f && r.y == 0.0f && r.z == 0.0f) return;
  const int4 c = at_ind[j];
  const float b0 = base[3 * s], b1 = base[3 * s + 1], b2 = base[3 * s + 2];
  int k, l;
  float dx, dy;
  if (plane == 1) {
    k = c.x;
    l = c.y;
    dx = __fadd_rn(__fsub_rn(__fsub_rn(r.x, b0), (float)c.x), (float)(p.n_row[0] / 2));
    dy = __fadd_rn(__fsub_rn(__fsub_rn(r.y, b1), (float)c.y), (float)(p.n_row[1] / 2));
  } else {
    const int per = (p.n_row[0] + p.n_row[1]) / 2;
    k = ((c.x - 1 + c.y - 1) % per + per) % per + 1;
    l = c.z;
    float t = __fadd_rn(__fadd_rn(__fsub_rn(__fsub_rn(r.x, b0), (float)c.x), (float)(p.n_row[0] / 2)), 1.0f);
    t = __fadd_rn(__fadd_rn(__fsub_rn(__fsub_rn(__fadd_rn(t, r.y), b1), (float)c.y), (float)(p.n_row[1] / 2)), 1.0f);
    dx = __fdiv_rn(t, sqrtf(2.0f));
    dy = __fadd_rn(__fadd_rn(__fsub_rn(__fsub_rn(r.z, b2), (float)c.z), (float)(p.n_row[2] / 2)), 1.0f);
  }
  if (k < 1 || k > n1 || l < 1 || l > n2) return;  // outside the cell grid
  const int64_t cell = (int64_t)(l - 1) * n1 + (k - 1);
  const int64_t plane_sz = (int64_t)n1 * n2;
  atomicAdd(&u[(2 * (int64_t)s) * plane_sz + cell].x, (T)dx);
  atomicAdd(&u[(2 * (int64_t)s + 1) * plane_sz + cell].x, (T)dy);
}

// One thread per Q pixel (i, j) of the m0 x m1 plane; pixels beyond the n_bz zones (which the
// reference never writes) are zero.  Species weights, mask and window norm as the NUFFT path.
template <typename T>
__global__ void oneph_expand_kernel(const typename Cplx<T>::type* __restrict__ u, PrepArgs p,
                                    int plane, const float* __restrict__ base, int n1, int n2,
                                    int m0, int m1, int n_bz, float qx_min, float qy_min,
                                    int nqx_min, int nqy_min, WeightArgs w,
                                    typename Cplx<T>::type* __restrict__ cs_frame,
                                    typename Cplx<T>::type* __restrict__ cs_species_frame) {
  using C = typename Cplx<T>::type;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int jq = blockIdx.y;
  if (i >= m0) return;
  const int64_t q = (int64_t)jq * m0 + i;
  const int64_t nm = (int64_t)m0 * m1;
  const int ii = i / n1, jj = jq / n2;
  const bool inside = ii < n_bz && jj < n_bz;
  const int k = i - ii * n1 + 1, l = jq - jj * n2 + 1;
  // q_x = qx_min + (ii - 1) + (k - 1) / n_row in FP32 (1-based ii there)
  const float qx = __fadd_rn(__fadd_rn(qx_min, (float)ii), __fdiv_rn((float)(k - 1), (float)n1));
  const float qy = __fadd_rn(__fadd_rn(qy_min, (float)jj), __fdiv_rn((float)(l - 1), (float)n2));
  int kk = (nqx_min + k) % n1, ll = (nqy_min + l) % n2;
  if (kk == 0) kk = n1;
  if (ll == 0) ll = n2;
  const int64_t cell = (int64_t)(ll - 1) * n1 + (kk - 1);
  const int64_t plane_sz = (int64_t)n1 * n2;
  T s2 = 0;
  if (w.weight_mode == MPSQ_WEIGHT_XRAY) {
    const int kx = i - m0 / 2, ky = jq - m1 / 2;
    T qv[3];
    for (int b = 0; b < 3; ++b)
      qv[b] = WP<T>::q0(w, b) + (T)kx * WP<T>::qs(w, 0, b) + (T)ky * WP<T>::qs(w, 1, b);
    s2 = WP<T>::kappa(w) * (qv[0] * qv[0] + qv[1] * qv[1] + qv[2] * qv[2] + WP<T>::extra(w));
  }
  const float tpi = 6.28318530717958647692f;
  T accr = 0, acci = 0;
  for (int s = 0; s < p.n_species; ++s) {
    if (p.group_of[s] < 0) continue;
    C a;
    a.x = (T)0;
    a.y = (T)0;
    if (inside) {
      const C ux = u[(2 * (int64_t)s) * plane_sz + cell];
      const C uy = u[(2 * (int64_t)s + 1) * plane_sz + cell];
      const T fx = (T)qx / (T)n1, fy = (T)qy / (T)n2;
      const T vr = fx * ux.x + fy * uy.x, vi = fx * ux.y + fy * uy.y;
      const float b0 = base[3 * s], b1 = base[3 * s + 1], b2 = base[3 * s + 2];
      const float dot = plane == 1 ? __fadd_rn(__fmul_rn(qx, b0), __fmul_rn(qy, b1))
                                   : __fadd_rn(__fmul_rn(qx, __fadd_rn(b0, b1)), __fmul_rn(qy, b2));
      const float arg = __fmul_rn(tpi, dot);
      T sn, cn;
      if constexpr (sizeof(T) == 8) {
        sincos((double)arg, &sn, &cn);
      } else {
        sincosf(arg, &sn, &cn);
      }
      a.x = cn * vr + sn * vi;      // (cos - i sin)(vr + i vi)
      a.y = cn * vi - sn * vr;
    }
    const T ws = species_weight<T>(w, s, s2);
    accr += ws * a.x;
    acci += ws * a.y;
    if (w.store_species) {
      C v;
      v.x = a.x * WP<T>::wnorm(w);
      v.y = a.y * WP<T>::wnorm(w);
      cs_species_frame[(int64_t)s * nm + q] = v;
    }
  }
  C out;
  out.x = accr * WP<T>::wnorm(w);
  out.y = acci * WP<T>::wnorm(w);
  cs_frame[q] = out;
}

// ------------------------------------------------------------- pruned fine-grid transform
// Only the 2h+1 central frequencies f in [-h, h] (h = m/2) of each dimension are needed
// (modes -m/2..(m-1)/2 plus the mirror +m/2 that packed-pair separation reads), so the 3D
// FFT runs as three passes that each keep 2h+1 of n outputs:
//   X: fine (n2, n1, n0)   -> b1 (n2, n1, K0)
//   Y: b1                  -> b2 (n2, K1, K0)
//   Z: b2 column tiles and their mirror tiles -> deconvolution, pair separation, species
//      weights, cs(t, Q)
// K = 2h+1; frequency f is stored at index f + h.

// All three passes keep a tile of lines of length N in shared memory as [position][line]
// (8 rows for X, 16 lines for Y, 2 x 8 for Z; lines fastest, so every warp access covers whole
// rows), issue all of a thread's global loads before storing any, transform in place
// (dif_lines) and read the kept frequencies at their digit-reversed positions.
constexpr int kPassLines = 16;

template <int N>
__device__ __forceinline__ void copy_twiddles(float2* tw, const float2* __restrict__ gtw) {
  for (int i = threadIdx.x; i < N; i += blockDim.x) tw[i] = gtw[i];
}
__device__ __forceinline__ int wrap_freq(int f, int n) { return f < 0 ? f + n : f; }

// Pass X: L contiguous rows of length N per CTA of 16 L threads (one grid per blockIdx.y).  A
// thread reads two adjacent complex of two adjacent rows (16 bytes each) and stores them as
// two 16-byte row pairs of the tile; the K0 kept frequencies of each row pair are gathered
// into registers, staged as [row][K0] and stored as one contiguous block.  Small CTAs (8 rows)
// let more of them share an SM, so that the loads of some overlap the transforms of others.
constexpr int kPassLinesX = 8;
template <int N, int L>
__global__ void __launch_bounds__(16 * L, (N < 512 ? 48 / L : 1))
    fftx_dif_kernel(const float2* __restrict__ fine, int64_t n_fine, int n_rows,
                    const float2* __restrict__ gtw, int h0, int K0, float2* __restrict__ b1) {
  constexpr int NT = 16 * L, LP = L / 2, NP = N / 2;
  constexpr int LOADS = (LP * NP + NT - 1) / NT;          // (row pair, x pair) items per thread
  constexpr int OUTS = (LP * (N / 2 + 1) + NT - 1) / NT;  // kept row-pair values (K0 <= N/2+1)
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* xs = reinterpret_cast<float2*>(smem_raw);    // [N][L], then [L][K0]
  float2* tw = xs + N * L;
  const int tid = threadIdx.x, g = blockIdx.y;
  const int row0 = blockIdx.x * L;
  const int rows = min(L, n_rows - row0);
  copy_twiddles<N>(tw, gtw);
  const float2* src = fine + (int64_t)g * n_fine + (int64_t)row0 * N;
  float4 va[LOADS], vb[LOADS];
#pragma unroll
  for (int p = 0; p < LOADS; ++p) {
    const int e = tid + NT * p;
    const int rp = e % LP, xp = e / LP;
    va[p] = vb[p] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (e < LP * NP) {
      if (2 * rp < rows) va[p] = __ldcs(reinterpret_cast<const float4*>(src + (int64_t)(2 * rp) * N + 2 * xp));
      if (2 * rp + 1 < rows) vb[p] = __ldcs(reinterpret_cast<const float4*>(src + (int64_t)(2 * rp + 1) * N + 2 * xp));
    }
  }
#pragma unroll
  for (int p = 0; p < LOADS; ++p) {
    const int e = tid + NT * p;
    if (e < LP * NP) {
      const int rp = e % LP, xp = e / LP, x = 2 * xp;
      const float4 lo = make_float4(va[p].x, va[p].y, vb[p].x, vb[p].y);
      const float4 hi = make_float4(va[p].z, va[p].w, vb[p].z, vb[p].w);
      // 8-line rows are 64 bytes: lanes of odd xp store their second row first, so that each
      // store instruction of a warp covers both halves of the banks (4 wavefronts, not 8)
      const int odd = L == 8 ? (xp & 1) : 0;
      *reinterpret_cast<float4*>(&xs[(x + odd) * L + 2 * rp]) = odd ? hi : lo;
      *reinterpret_cast<float4*>(&xs[(x + 1 - odd) * L + 2 * rp]) = odd ? lo : hi;
    }
  }
  __syncthreads();
  constexpr int NS = dif_stages(N), RL = dif_radix(N, NS - 1);
  if constexpr (NS == 2 && RL > 8 && L * (N / RL) == NT) {
    // two-stage plan: the last stage (contiguous groups of RL, no twiddles) is finished in
    // registers, one (line, group) per thread, and only the kept frequencies are written,
    // straight into the [row][K0] staging layout; output k of group gi is frequency
    // gi + (N / RL) k
    dif_lines_until<N, L, NS - 1>(xs, tw);
    const int ln = tid % L, gi = tid / L;
    float2 v[RL];
#pragma unroll
    for (int k = 0; k < RL; ++k) v[k] = xs[(gi * RL + k) * L + ln];
    dft_r(v, RL);
    __syncthreads();                     // every input has been read
#pragma unroll
    for (int k = 0; k < RL; ++k) {
      const int f = gi + (N / RL) * k;
      const int i = f <= h0 ? f + h0 : (f >= N - h0 ? f - N + h0 : -1);
      if (i >= 0 && i < K0) xs[ln * K0 + i] = v[k];
    }
  } else {
    dif_lines<N, L>(xs, tw);
    float4 o[OUTS];
#pragma unroll
    for (int p = 0; p < OUTS; ++p) {
      const int e = tid + NT * p;
      o[p] = make_float4(0.f, 0.f, 0.f, 0.f);
      if (e < LP * K0)
        o[p] = *reinterpret_cast<const float4*>(&xs[dif_position<N>(wrap_freq(e / LP - h0, N)) * L + 2 * (e % LP)]);
    }
    __syncthreads();
#pragma unroll
    for (int p = 0; p < OUTS; ++p) {
      const int e = tid + NT * p;
      if (e < LP * K0) {
        const int r = 2 * (e % LP), i = e / LP;
        xs[r * K0 + i] = make_float2(o[p].x, o[p].y);
        xs[(r + 1) * K0 + i] = make_float2(o[p].z, o[p].w);
      }
    }
  }
  __syncthreads();
  float2* dst = b1 + ((int64_t)g * n_rows + row0) * K0;
  for (int e = tid; e < rows * K0; e += NT) dst[e] = xs[e];
}

// Pass Y: 16 consecutive x-columns (length N along y) of one z-plane per CTA; a thread moves
// two adjacent columns.
template <int N>
__global__ void __launch_bounds__(256, (N < 512 ? 3 : 1))
    ffty_dif_kernel(const float2* __restrict__ b1, int n2in, int n2, int zoff, int K0,
                    const float2* __restrict__ gtw, int h1, int K1, float2* __restrict__ b2) {
  constexpr int L = kPassLines, LP = L / 2;
  constexpr int LOADS = (LP * N + 255) / 256, BATCH = LOADS < 8 ? LOADS : 8;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* xs = reinterpret_cast<float2*>(smem_raw);    // [N][L]
  float2* tw = xs + N * L;
  const int tid = threadIdx.x;
  const int x0 = blockIdx.x * L, z = blockIdx.y, g = blockIdx.z;
  copy_twiddles<N>(tw, gtw);
  const float2* src = b1 + ((int64_t)g * n2in + z) * (int64_t)N * K0;
  for (int b0 = 0; b0 < LOADS; b0 += BATCH) {
    float2 va[BATCH], vb[BATCH];
#pragma unroll
    for (int p = 0; p < BATCH; ++p) {
      const int e = tid + 256 * (b0 + p);
      const int x = x0 + 2 * (e % LP), y = e / LP;
      va[p] = vb[p] = make_float2(0.f, 0.f);
      if (b0 + p < LOADS && e < LP * N) {
        const float2* q = src + (int64_t)y * K0 + x;
        if (x < K0) va[p] = __ldcs(q);
        if (x + 1 < K0) vb[p] = __ldcs(q + 1);
      }
    }
#pragma unroll
    for (int p = 0; p < BATCH; ++p) {
      const int e = tid + 256 * (b0 + p);
      if (b0 + p < LOADS && e < LP * N)
        *reinterpret_cast<float4*>(&xs[2 * e]) = make_float4(va[p].x, va[p].y, vb[p].x, vb[p].y);
    }
  }
  __syncthreads();
  float2* dst = b2 + ((int64_t)g * n2 + zoff + z) * (int64_t)K1 * K0;
  constexpr int NS = dif_stages(N), RL = dif_radix(N, NS - 1);
  if constexpr (NS == 2 && RL > 8 && L * (N / RL) == 256) {
    // two-stage plan: the last stage is finished in registers, one (column, group) per
    // thread, and the kept frequencies go straight to b2 (the 16 columns of a group are
    // contiguous); output k of group gi is frequency gi + (N / RL) k
    dif_lines_until<N, L, NS - 1>(xs, tw);
    const int ln = tid % L, gi = tid / L;
    float2 v[RL];
#pragma unroll
    for (int k = 0; k < RL; ++k) v[k] = xs[(gi * RL + k) * L + ln];
    dft_r(v, RL);
    const int x = x0 + ln;
    if (x < K0) {
#pragma unroll
      for (int k = 0; k < RL; ++k) {
        const int f = gi + (N / RL) * k;
        const int i = f <= h1 ? f + h1 : (f >= N - h1 ? f - N + h1 : -1);
        if (i >= 0 && i < K1) dst[(int64_t)i * K0 + x] = v[k];
      }
    }
  } else {
    dif_lines<N, L>(xs, tw);
    for (int e = tid; e < LP * K1; e += 256) {
      const int c = 2 * (e % LP), i = e / LP;
      const int x = x0 + c;
      if (x >= K0) continue;
      const float4 v = *reinterpret_cast<const float4*>(&xs[dif_position<N>(wrap_freq(i - h1, N)) * L + c]);
      float2* q = dst + (int64_t)i * K0 + x;
      q[0] = make_float2(v.x, v.y);
      if (x + 1 < K0) q[1] = make_float2(v.z, v.w);
    }
  }
}

// Pass Z fused with the deconvolution: CTA (x-tile, ky index iy <= h1) loads, for every grid,
// the T z-columns P = (iy, x0..x0+T) and their mirrors M = (2h1-iy, 2h0-x), transforms all 2T
// lines and forms the weighted species amplitudes of both the P modes and the M modes: the
// pair separation of a mode k reads G(k) and G(-k), and the lines of P and M hold exactly the
// two for either (so every column is loaded and transformed once).  A row that is its own
// mirror (iy = h1) takes only its P modes; rows beyond the output range are skipped.
template <int N>
__host__ __device__ constexpr int zpass_cols() { return 8; }

// One output mode from its line value G = G(k) and the mirror value Gm = G(-k): pair
// separation, deconvolution, species weights; returns the weighted amplitude (without the
// window norm) and writes the per-species amplitudes when they are stored.
__device__ __forceinline__ float2 zpass_mode(float2 G, float2 Gm, bool pair, int sa, int sb,
                                             float corr, int kx, int ky, int kz,
                                             const WeightArgs& w, int64_t q, int64_t nm,
                                             float2* __restrict__ cs_species_frame) {
  float s2 = 0.f;
  if (w.weight_mode == MPSQ_WEIGHT_XRAY) {
    float qv[3];
#pragma unroll
    for (int b = 0; b < 3; ++b)
      qv[b] = w.q0_f[b] + (float)kx * w.qs_f[0][b] + (float)ky * w.qs_f[1][b] + (float)kz * w.qs_f[2][b];
    s2 = w.kappa_f * (qv[0] * qv[0] + qv[1] * qv[1] + qv[2] * qv[2] + w.extra_f);
  }
  if (pair) {
    const float ar = 0.5f * (G.x + Gm.x) * corr, ai = 0.5f * (G.y - Gm.y) * corr;
    const float br = 0.5f * (G.y + Gm.y) * corr, bi = -0.5f * (G.x - Gm.x) * corr;
    const float wa = species_weight<float>(w, sa, s2), wb = species_weight<float>(w, sb, s2);
    if (w.store_species) {
      cs_species_frame[(int64_t)sa * nm + q] = make_float2(ar * w.wnorm_f, ai * w.wnorm_f);
      cs_species_frame[(int64_t)sb * nm + q] = make_float2(br * w.wnorm_f, bi * w.wnorm_f);
    }
    return make_float2(wa * ar + wb * br, wa * ai + wb * bi);
  }
  const float wa = species_weight<float>(w, sa, s2);
  if (w.store_species)
    cs_species_frame[(int64_t)sa * nm + q] = make_float2(G.x * corr * w.wnorm_f, G.y * corr * w.wnorm_f);
  return make_float2(wa * G.x * corr, wa * G.y * corr);
}

template <int N, bool SLAB>
__global__ void __launch_bounds__(256, (N <= 512 ? 3 : 1))
    fftz_dif_deconv_kernel(const float2* __restrict__ b2, int K0, int K1, int m0, int m1, int m2,
                           int z0, int nz, int h0, int h1, int h2, int ngroups,
                           const float2* __restrict__ gtw,
                           const float* __restrict__ c0, const float* __restrict__ c1,
                           const float* __restrict__ c2, WeightArgs w,
                           float2* __restrict__ cs_frame, float2* __restrict__ cs_species_frame) {
  constexpr int T = zpass_cols<N>(), L = 2 * T, LP = L / 2, TP = T / 2;
  constexpr int LOADS = (LP * N + 255) / 256, BATCH = LOADS < 8 ? LOADS : 8;
  constexpr int OUTS = (TP * (N / 2) + 255) / 256;      // column pairs x m2 (m2 <= N/2)
  // radix-8 stages from length 512 on: the two-stage plan's radix-32 lines would not fit the
  // register budget next to the accumulators of this pass
  constexpr int PZ = N >= 512 ? kDifGreedy : kDifTwoStage;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* xs = reinterpret_cast<float2*>(smem_raw);     // [N][L]: T columns, then T mirrors
  float2* tw = xs + N * L;
  const int tid = threadIdx.x;
  const int x0 = blockIdx.x * T, iy = blockIdx.y;
  const int iym = 2 * h1 - iy;
  const bool mrow = iym < m1 && iym != iy;              // this CTA also forms the row iym
  // modes per frame in the store (SLAB: the store holds kz planes [z0, z0 + nz) only; the
  // whole-store instantiation keeps the registers of the common case)
  const int64_t nm = (int64_t)m0 * m1 * (SLAB ? nz : m2);
  copy_twiddles<N>(tw, gtw);
  float4 acc[OUTS], accm[OUTS];
#pragma unroll
  for (int p = 0; p < OUTS; ++p) acc[p] = accm[p] = make_float4(0.f, 0.f, 0.f, 0.f);
  const float cy = c1[iy], cym = mrow ? c1[iym] : 0.0f;
  const int ky = iy - h1, kym = iym - h1;
  for (int g = 0; g < ngroups; ++g) {
    const float2* src = b2 + (int64_t)g * N * K1 * K0;
    const int pair = w.pair[g];
    const bool need_m = pair || mrow;
    if (g > 0) __syncthreads();  // the previous group's reads of the tile are complete
    for (int b0 = 0; b0 < LOADS; b0 += BATCH) {
      float2 va[BATCH], vb[BATCH];
#pragma unroll
      for (int p = 0; p < BATCH; ++p) {
        const int e = tid + 256 * (b0 + p);
        const int l = 2 * (e % LP), z = e / LP;
        const bool mirror = l >= T;
        const int c = mirror ? l - T : l;
        const int x = x0 + c;
        va[p] = vb[p] = make_float2(0.f, 0.f);
        if (b0 + p < LOADS && e < LP * N && (!mirror || need_m)) {
          const float2* row = src + ((int64_t)z * K1 + (mirror ? iym : iy)) * K0;
          if (x < K0) va[p] = __ldcs(row + (mirror ? 2 * h0 - x : x));
          if (x + 1 < K0) vb[p] = __ldcs(row + (mirror ? 2 * h0 - x - 1 : x + 1));
        }
      }
#pragma unroll
      for (int p = 0; p < BATCH; ++p) {
        const int e = tid + 256 * (b0 + p);
        if (b0 + p < LOADS && e < LP * N)
          *reinterpret_cast<float4*>(&xs[2 * e]) = make_float4(va[p].x, va[p].y, vb[p].x, vb[p].y);
      }
    }
    __syncthreads();
    dif_lines<N, L, DifNoPre, PZ>(xs, tw);
    const int sa = w.sp_a[g], sb = w.sp_b[g];
#pragma unroll
    for (int p = 0; p < OUTS; ++p) {
      const int e = tid + 256 * p;
      const int c = 2 * (e % TP), iz = e / TP;
      const int lz = SLAB ? iz - z0 : iz;                // plane within the store
      if (iz >= m2 || (SLAB && (lz < 0 || lz >= nz)) || x0 + c >= K0) continue;
      const int fz = iz - h2;
      const int pf = dif_position<N, PZ>(wrap_freq(fz, N)), pm = dif_position<N, PZ>(wrap_freq(-fz, N));
      const float4 P2 = *reinterpret_cast<const float4*>(&xs[pf * L + c]);
      const float4 Pm2 = *reinterpret_cast<const float4*>(&xs[pm * L + c]);
      float4 M2 = make_float4(0.f, 0.f, 0.f, 0.f), Mm2 = M2;
      if (need_m) {
        M2 = *reinterpret_cast<const float4*>(&xs[pf * L + T + c]);
        Mm2 = *reinterpret_cast<const float4*>(&xs[pm * L + T + c]);
      }
      const float cz = c2[iz];
#pragma unroll
      for (int hv = 0; hv < 2; ++hv) {
        const int x = x0 + c + hv;       // P column (beyond m0: only its mirror is a mode)
        if (x >= K0) continue;
        const float2 P = hv ? make_float2(P2.z, P2.w) : make_float2(P2.x, P2.y);
        const float2 Pm = hv ? make_float2(Pm2.z, Pm2.w) : make_float2(Pm2.x, Pm2.y);
        const float2 M = hv ? make_float2(M2.z, M2.w) : make_float2(M2.x, M2.y);
        const float2 Mm = hv ? make_float2(Mm2.z, Mm2.w) : make_float2(Mm2.x, Mm2.y);
        // P mode (iy, x, iz): G(k) on the P line, G(-k) on the M line at -fz
        float2 a = make_float2(0.f, 0.f);
        if (x < m0)
          a = zpass_mode(P, Mm, pair, sa, sb, c0[x] * cy * cz, x - h0, ky, fz, w,
                         ((int64_t)lz * m1 + iy) * m0 + x, nm, cs_species_frame);
        // M mode (iym, 2h0 - x, iz): G(k) on the M line, G(-k) on the P line at -fz
        float2 b = make_float2(0.f, 0.f);
        const int xm = 2 * h0 - x;
        if (mrow && xm < m0)
          b = zpass_mode(M, Pm, pair, sa, sb, c0[xm] * cym * cz, xm - h0, kym, fz, w,
                         ((int64_t)lz * m1 + iym) * m0 + xm, nm, cs_species_frame);
        if (hv) {
          acc[p].z += a.x;
          acc[p].w += a.y;
          accm[p].z += b.x;
          accm[p].w += b.y;
        } else {
          acc[p].x += a.x;
          acc[p].y += a.y;
          accm[p].x += b.x;
          accm[p].y += b.y;
        }
      }
    }
  }
#pragma unroll
  for (int p = 0; p < OUTS; ++p) {
    const int e = tid + 256 * p;
    const int c = 2 * (e % TP), iz = e / TP;
    const int x = x0 + c, lz = SLAB ? iz - z0 : iz;
    if (iz >= m2 || (SLAB && (lz < 0 || lz >= nz)) || x >= K0) continue;
    float2* q = cs_frame + ((int64_t)lz * m1 + iy) * m0 + x;
    if (x < m0) q[0] = make_float2(acc[p].x * w.wnorm_f, acc[p].y * w.wnorm_f);
    if (x + 1 < m0) q[1] = make_float2(acc[p].z * w.wnorm_f, acc[p].w * w.wnorm_f);
    if (mrow) {
      float2* qm = cs_frame + ((int64_t)lz * m1 + iym) * m0;
      const int xm = 2 * h0 - x;   // in [0, 2 h0]; the column x + 1 mirrors to xm - 1
      if (xm < m0) qm[xm] = make_float2(accm[p].x * w.wnorm_f, accm[p].y * w.wnorm_f);
      if (x + 1 < K0 && xm - 1 < m0) qm[xm - 1] = make_float2(accm[p].z * w.wnorm_f, accm[p].w * w.wnorm_f);
    }
  }
}

struct PruneLaunch {
  const float2* fine;
  int64_t n_fine;
  float2* b1;
  float2* b2;
  int n[3], m[3], h[3], K[3];
  int ngrid, ngroups;
  int xrows = kPassLinesX;   // rows per CTA of the X pass (4 or 8)
  int z0 = 0, nz = 0;        // kz planes of the store's Q slab
  int fz0 = 0, fnz = 0;      // fine-grid planes [fz0, fz0 + fnz) of the X and Y passes
  const float2* tw[3];
  const float* c[3];
  cudaStream_t s;
};

template <int N>
static size_t pass_smem(int lines) {
  return (size_t)N * lines * sizeof(float2) + (size_t)N * sizeof(float2);
}

template <int N, int L>
static int launch_prune_x_l(const PruneLaunch& p) {
  const int n_rows = p.n[1] * p.fnz;
  const size_t sm = pass_smem<N>(L);
  cudaFuncSetAttribute(fftx_dif_kernel<N, L>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  fftx_dif_kernel<N, L><<<dim3((unsigned)((n_rows + L - 1) / L), (unsigned)p.ngrid), 16 * L, sm,
                          p.s>>>(p.fine, p.n_fine, n_rows, p.tw[0], p.h[0], p.K[0], p.b1);
  MPSQ_LAUNCH_CHECK();
  return MPSQ_OK;
}
template <int N>
static int launch_prune_x(const PruneLaunch& p) {
  return p.xrows == 4 ? launch_prune_x_l<N, 4>(p) : launch_prune_x_l<N, kPassLinesX>(p);
}
template <int N>
static int launch_prune_y(const PruneLaunch& p) {
  const size_t sm = pass_smem<N>(kPassLines);
  cudaFuncSetAttribute(ffty_dif_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  ffty_dif_kernel<N><<<dim3((unsigned)((p.K[0] + kPassLines - 1) / kPassLines), (unsigned)p.fnz,
                            (unsigned)p.ngrid),
                       256, sm, p.s>>>(p.b1, p.fnz, p.n[2], p.fz0, p.K[0], p.tw[1], p.h[1],
                                       p.K[1], p.b2);
  MPSQ_LAUNCH_CHECK();
  return MPSQ_OK;
}
template <int N>
static int launch_prune_z(const PruneLaunch& p, const WeightArgs& w, float2* csf, float2* css) {
  constexpr int T = zpass_cols<N>();
  const size_t sm = pass_smem<N>(2 * T);
  const bool slab = p.z0 != 0 || p.nz != p.m[2];
  if (slab)
    cudaFuncSetAttribute(fftz_dif_deconv_kernel<N, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  else
    cudaFuncSetAttribute(fftz_dif_deconv_kernel<N, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  auto kern = slab ? fftz_dif_deconv_kernel<N, true> : fftz_dif_deconv_kernel<N, false>;
  const int rows = std::min(p.m[1], p.h[1] + 1);   // ky rows iy <= h1; each also forms 2 h1 - iy
  // x tiles cover the K0 = 2 h0 + 1 kept columns: column 2 h0 is the mirror of mode column 0
  kern<<<dim3((unsigned)((p.K[0] + T - 1) / T), (unsigned)rows), 256, sm, p.s>>>(
      p.b2, p.K[0], p.K[1], p.m[0], p.m[1], p.m[2], p.z0, p.nz, p.h[0], p.h[1], p.h[2], p.ngroups,
      p.tw[2],
      p.c[0], p.c[1], p.c[2], w, csf, css);
  MPSQ_LAUNCH_CHECK();
  return MPSQ_OK;
}

// Passes X and Y over the fine-grid planes [fz0, fz0 + fnz).
static int run_pruned_xy(const PruneLaunch& p) {
  int rc = MPSQ_ERR_ARG;
  switch (p.n[0]) {
#define MPSQ_CASE(N) case N: rc = launch_prune_x<N>(p); break;
    MPSQ_FFT_SIZES(MPSQ_CASE)
#undef MPSQ_CASE
  }
  if (rc) return rc;
  rc = MPSQ_ERR_ARG;
  switch (p.n[1]) {
#define MPSQ_CASE(N) case N: rc = launch_prune_y<N>(p); break;
    MPSQ_FFT_SIZES(MPSQ_CASE)
#undef MPSQ_CASE
  }
  return rc;
}
// Pass Z with the deconvolution and weights, over the whole of b2.
static int run_pruned_z(const PruneLaunch& p, const WeightArgs& w, float2* csf, float2* css) {
  int rc = MPSQ_ERR_ARG;
  switch (p.n[2]) {
#define MPSQ_CASE(N) case N: rc = launch_prune_z<N>(p, w, csf, css); break;
    MPSQ_FFT_SIZES(MPSQ_CASE)
#undef MPSQ_CASE
  }
  return rc;
}

static size_t csize(int prec) { return prec == MPSQ_FP64 ? sizeof(double2) : sizeof(float2); }
static size_t rsize(int prec) { return prec == MPSQ_FP64 ? sizeof(RecD) : sizeof(RecF); }

static int job_layout(const mpsq_job_desc* d, EsKernel* es, GridGeom* g, int* ngroups,
                      int group_of[], int comp_of[], int pair[], int sp_a[], int sp_b[],
                      int* pack) {
  if (d->ndim != 2 && d->ndim != 3) return fail(MPSQ_ERR_ARG, "job: ndim must be 2 or 3");
  if (d->precision != MPSQ_FP32 && d->precision != MPSQ_FP64)
    return fail(MPSQ_ERR_ARG, "job: bad precision");
  if (d->n_species < 1 || d->n_species > MPSQ_MAX_SPECIES)
    return fail(MPSQ_ERR_ARG, "job: n_species must be in 1..%d", MPSQ_MAX_SPECIES);
  if (d->n_frames < 1) return fail(MPSQ_ERR_ARG, "job: n_frames must be >= 1");
  if (d->n_atoms_frame < 1) return fail(MPSQ_ERR_ARG, "job: n_atoms_frame must be >= 1");
  if (d->species_offset[0] < 0 || d->species_offset[d->n_species] > d->n_atoms_frame)
    return fail(MPSQ_ERR_ARG, "job: species offsets outside the frame");
  for (int s = 0; s < d->n_species; ++s)
    if (d->species_offset[s + 1] < d->species_offset[s])
      return fail(MPSQ_ERR_ARG, "job: species offsets not increasing");
  if (d->weight_mode < 1 || d->weight_mode > 3) return fail(MPSQ_ERR_ARG, "job: bad weight_mode");
  if (d->q_slab < 0 || (d->q_slab > 0 && d->ndim != 3))
    return fail(MPSQ_ERR_ARG, "job: q_slab must be 0, or > 0 for a 3D job");
  *es = es_params(d->eps, d->precision);
  int rc = make_geom(d->ndim, d->n_modes, es->w, g);
  if (rc) return rc;
  if (d->precision == MPSQ_FP32 && d->ndim == 3 && !d->no_pruned_fft) {
    // FP32 volumes: fine lengths from the compiled pruned transforms (the smallest at or above
    // the 2,3,5-smooth length; an upsampling above 2 only lowers the kernel's error), so that
    // every grid up to 1600 points per axis takes the pruned passes instead of cuFFT
    for (int k = 0; k < 3; ++k) {
      const int64_t n = compiled_fft_size_at_least(g->nf[k]);
      if (n > 0) {
        g->nf[k] = n;
        g->ntile[k] = (int)(n / g->tile[k]);
      }
    }
    g->n_tiles = (int64_t)g->ntile[0] * g->ntile[1] * g->ntile[2];
    g->n_fine = g->nf[0] * g->nf[1] * g->nf[2];
  }
  const bool qc0 = d->q_center[0] == 0.0 && d->q_center[1] == 0.0 && d->q_center[2] == 0.0;
  *pack = (qc0 && !d->no_pack) ? 1 : 0;
  int n = 0;
  int open = -1;  // group with a free imaginary slot
  for (int s = 0; s < d->n_species; ++s) {
    group_of[s] = -1;
    comp_of[s] = 0;
    if (!d->mask[s]) continue;
    if (*pack && open >= 0) {
      group_of[s] = open;
      comp_of[s] = 1;
      pair[open] = 1;
      sp_b[open] = s;
      open = -1;
    } else {
      group_of[s] = n;
      pair[n] = 0;
      sp_a[n] = s;
      sp_b[n] = s;
      if (*pack) open = n;
      ++n;
    }
  }
  *ngroups = n;
  return MPSQ_OK;
}

}  // namespace mpsq

// ================================================================================ C ABI
static void job_free(mpsq_job* j) {
  if (!j) return;
  if (j->have_fft) cufftDestroy(j->fft);
  if (j->have_xfft)
    for (auto h : j->xfft)
      if (h) cufftDestroy(h);
  job_release(j, j->traj);
  job_release(j, j->at_ind);
  job_release(j, j->fine);
  job_release(j, j->counts);
  job_release(j, j->starts);
  job_release(j, j->perm);
  job_release(j, j->perm_counts);
  job_release(j, j->perm_starts);
  job_release(j, j->recs);
  job_release(j, j->str);
  for (int a = 0; a < 3; ++a) job_release(j, j->corr[a]);
  job_release(j, j->cs);
  job_release(j, j->cs_species);
  job_release(j, j->err);
  job_release(j, j->b1);
  for (auto& t : j->tw) job_release(j, t);
  job_release(j, j->fine2);
  job_release(j, j->counts2);
  job_release(j, j->starts2);
  job_release(j, j->recs2);
  job_release(j, j->str2);
  job_release(j, j->prep);
  job_release(j, j->prep2);
  job_release(j, j->b1_2);
  if (j->have_oneph_fft) cufftDestroy(j->oneph_fft);
  job_release(j, j->oneph_u);
  job_release(j, j->oneph_base);
  for (auto& gr : j->graphs) cudaGraphExecDestroy(gr.exec);
  if (j->fork) cudaEventDestroy(j->fork);
  if (j->join) cudaEventDestroy(j->join);
  if (j->s2) cudaStreamDestroy(j->s2);
  for (auto& e : j->ev)
    if (e) cudaEventDestroy(e);
  delete j;
}

// Bytes of the per-atom preparation cache of the FP32 split path (0: not used): cell words
// (16 B) and d2 (4 B) per atom, plus the strength (8 B, at offset 24 n) unless all are 1.
static size_t prep_cache_bytes(int precision, int phase_rounding, bool unit_str, int64_t n) {
  if (precision != MPSQ_FP32 || phase_rounding || n <= 0) return 0;
  return (size_t)n * (unit_str ? 20 : 32);
}
static size_t prep_cache_bytes(const mpsq_job* j) {
  return prep_cache_bytes(j->d.precision, j->pa.phase_rounding, !j->pa.has_qc && !j->pa.window,
                          j->d.n_atoms_frame);
}

extern "C" int mpsq_job_estimate_bytes(const mpsq_job_desc* d, int64_t* bytes) {
  if (!d || !bytes) return fail(MPSQ_ERR_ARG, "estimate: null pointer");
  EsKernel es;
  GridGeom g;
  int ng, gof[MPSQ_MAX_SPECIES], cof[MPSQ_MAX_SPECIES], pr[MPSQ_MAX_SPECIES],
      sa[MPSQ_MAX_SPECIES], sb[MPSQ_MAX_SPECIES], pack;
  int rc = job_layout(d, &es, &g, &ng, gof, cof, pr, sa, sb, &pack);
  if (rc) return rc;
  const int64_t per = d->ndim == 3 ? 8 : 4;
  int64_t b = 0;
  b += (int64_t)d->n_frames * d->n_atoms_frame * 16;                  // trajectory
  b += (int64_t)std::max(1, ng) * g.n_fine * (int64_t)csize(d->precision);  // fine grids
  b += d->n_atoms_frame * per * (int64_t)(rsize(d->precision) + csize(d->precision));
  b += (int64_t)(std::max(1, ng) * g.n_tiles + 1) * 8;
  b += d->n_atoms_frame * 4 + (int64_t)(std::max(1, ng) * g.n_tiles + 2) * 8;  // locality order
  const int64_t prep = (int64_t)prep_cache_bytes(d->precision, d->phase_rounding, false,
                                                 d->n_atoms_frame);  // per-atom preparation
  b += prep;
  const int64_t store = d->q_slab > 0 ? g.m[0] * g.m[1] * std::min<int64_t>(d->q_slab, g.m[2])
                                      : g.n_modes;                      // modes per frame kept
  b += (int64_t)d->n_frames * store * (int64_t)csize(d->precision);     // cs(t,Q)
  if (d->store_species)
    b += (int64_t)d->n_frames * d->n_species * store * (int64_t)csize(d->precision);
  bool pruned = d->precision == MPSQ_FP32 && d->ndim == 3 && !d->no_pruned_fft;
  for (int k = 0; k < 3 && pruned; ++k) pruned = fft_size_compiled((int)g.nf[k]);
  if (pruned) {  // X-pass output, plus a second frame lane (fine grid, bins, records, X output)
    const int64_t b1 = (int64_t)std::max(1, ng) * g.nf[2] * g.nf[1] * (2 * (g.m[0] / 2) + 1) * 8;
    b += b1;
    b += (int64_t)std::max(1, ng) * g.n_fine * 8 + (int64_t)(std::max(1, ng) * g.n_tiles + 1) * 8 +
         d->n_atoms_frame * per * (int64_t)(rsize(d->precision) + csize(d->precision)) + b1 + prep;
  } else {
    // cuFFT work areas (estimate): the strided (z, y) plans of the kept x columns of a 3D grid
    // hold up to their own data each, about a quarter of the grid per plan
    b += g.n_fine * (int64_t)csize(d->precision) / (d->ndim == 3 ? 2 : 4);
  }
  *bytes = b;
  return MPSQ_OK;
}

// Volumes on cuFFT (FP64, and FP32 fine grids off the compiled length ladder) transform only
// what the deconvolution reads: one batch of x transforms over every row, then batched 2D
// (z, y) transforms over the x columns whose frequencies are kept, [0, h0] and [n0 - h0, n0)
// with h0 = m0 / 2 (the modes and their mirrors), strided by n0 within each grid.  About half
// the columns take the (z, y) part, so the transform does ~2/3 of a full 3D one.
static int make_xpruned_fft(mpsq_job* j) {
  const GridGeom& g = j->g;
  const cufftType type = j->d.precision == MPSQ_FP64 ? CUFFT_Z2Z : CUFFT_C2C;
  const long long n0 = g.nf[0], n1 = g.nf[1], n2 = g.nf[2];
  const int h0 = (int)(g.m[0] / 2);
  long long nx[1] = {n0};
  long long nzy[2] = {n2, n1};
  const long long batch[3] = {(long long)j->sa.ngrid * n1 * n2, h0 + 1, h0};
  for (int k = 0; k < 3; ++k) {
    if (batch[k] == 0) continue;
    MPSQ_CUFFT_TRY(cufftCreate(&j->xfft[k]));
    j->have_xfft = true;
    size_t ws = 0;
    cufftResult r = k == 0 ? cufftMakePlanMany64(j->xfft[k], 1, nx, nullptr, 1, n0, nullptr, 1, n0,
                                                 type, batch[k], &ws)
                           : cufftMakePlanMany64(j->xfft[k], 2, nzy, nzy, n0, 1, nzy, n0, 1, type,
                                                 batch[k], &ws);
    if (r == CUFFT_SUCCESS) r = cufftSetStream(j->xfft[k], j->s);
    if (r != CUFFT_SUCCESS)
      return fail(MPSQ_ERR_CUFFT, "cufftMakePlanMany (%s part, %lld x %lld x %lld) status %d",
                  k == 0 ? "x" : "z-y", n0, n1, n2, (int)r);
  }
  j->xfft_h0 = h0;
  return MPSQ_OK;
}

static int exec_xpruned_fft(mpsq_job* j) {
  const int prec = j->d.precision;
  const size_t cs = prec == MPSQ_FP64 ? sizeof(double2) : sizeof(float2);
  char* base = static_cast<char*>(j->fine);
  int rc = exec_fft(j->xfft[0], prec, base, CUFFT_FORWARD);
  if (rc) return rc;
  const int64_t n0 = j->g.nf[0];
  for (int gi = 0; gi < j->sa.ngrid; ++gi) {
    char* grid = base + (size_t)gi * j->g.n_fine * cs;
    rc = exec_fft(j->xfft[1], prec, grid, CUFFT_FORWARD);
    if (!rc && j->xfft[2])
      rc = exec_fft(j->xfft[2], prec, grid + (size_t)(n0 - j->xfft_h0) * cs, CUFFT_FORWARD);
    if (rc) return rc;
  }
  return MPSQ_OK;
}

extern "C" int mpsq_job_create(const mpsq_job_desc* d, void* stream, mpsq_job** out) {
  if (!d || !out) return fail(MPSQ_ERR_ARG, "job_create: null pointer");
  *out = nullptr;
  auto* j = new mpsq_job();
  j->d = *d;
  j->s = (cudaStream_t)stream;
  if (d->stream_ordered) {
    // keep memory that jobs give back in the pool for the next job (process-local setting)
    static std::once_flag once;
    std::call_once(once, [] {
      int dev = 0;
      cudaMemPool_t pool;
      if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        uint64_t keep = ~0ull;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
      }
      cudaGetLastError();
    });
  }
  int gof[MPSQ_MAX_SPECIES], cof[MPSQ_MAX_SPECIES], pr[MPSQ_MAX_SPECIES] = {0},
      sa[MPSQ_MAX_SPECIES] = {0}, sb[MPSQ_MAX_SPECIES] = {0}, pack = 0;
  int rc = job_layout(d, &j->es, &j->g, &j->ngroups, gof, cof, pr, sa, sb, &pack);
  if (rc) {
    delete j;
    return rc;
  }
  const int prec = d->precision;
  // spread geometry
  SpreadArgs& a = j->sa;
  a.dim = d->ndim;
  a.w = j->es.w;
  a.beta = j->es.beta;
  for (int k = 0; k < 3; ++k) {
    a.nf[k] = j->g.nf[k];
    a.tile[k] = j->g.tile[k];
    a.ntile[k] = j->g.ntile[k];
  }
  a.n_tiles = j->g.n_tiles;
  a.n_fine = j->g.n_fine;
  a.ngrid = std::max(1, j->ngroups);
  finish_spread_args(a);
  // preparation parameters
  PrepArgs& p = j->pa;
  p.dim = d->ndim;
  p.n_species = d->n_species;
  for (int s = 0; s <= d->n_species; ++s) p.species_offset[s] = d->species_offset[s];
  for (int s = 0; s < d->n_species; ++s) {
    p.group_of[s] = gof[s];
    p.comp_of[s] = cof[s];
  }
  p.input_method = d->input_method;
  p.phase_rounding = d->phase_rounding;
  p.use_range = d->use_range;
  p.bulk_nsuper1 = d->bulk_nsuper1;
  for (int k = 0; k < 3; ++k) {
    p.n_row[k] = d->n_row[k];
    for (int b = 0; b < 3; ++b) {
      p.axis[k][b] = d->axis[k][b];
      p.axis_f[k][b] = (float)d->axis[k][b];
    }
    p.tpe[k] = d->tpe[k];
    p.tpe_f[k] = (float)d->tpe[k];
    p.centre[k] = d->centre[k];
    p.centre_f[k] = (float)d->centre[k];
    p.pos_min[k] = d->pos_min[k];
    p.pos_max[k] = d->pos_max[k];
    p.pos_min_f[k] = (float)d->pos_min[k];
    p.pos_max_f[k] = (float)d->pos_max[k];
    p.q_center[k] = d->q_center[k];
    p.tpq_f[k] = (float)(2.0 * M_PI) * (float)d->q_center[k];
  }
  p.tol_f = d->bulk_nsuper1 ? (float)d->eps_x : 1.0f;
  p.has_qc = pack ? 0 : !(d->q_center[0] == 0.0 && d->q_center[1] == 0.0 && d->q_center[2] == 0.0);
  p.window = d->spatial_window;
  p.pack = pack;
  p.n_atoms_frame = d->n_atoms_frame;
  p.diag = 1;
  for (int k = 0; k < 3; ++k) {
    const double sc = d->tpe[k] * a.gscale[k];  // radians -> fine-grid units along axis k
    double bk = 0.0;
    for (int b = 0; b < 3; ++b) {
      const double A = d->axis[k][b] * sc;
      p.ahi[k][b] = (float)A;
      p.alo[k][b] = (float)(A - (double)p.ahi[k][b]);
      bk -= A * d->centre[b];
    }
    p.bhi[k] = (float)bk;
    p.blo[k] = (float)(bk - (double)p.bhi[k]);
    p.qhi[k] = (float)d->q_center[k];
    p.qlo[k] = (float)(d->q_center[k] - (double)p.qhi[k]);
    p.nf[k] = (int)j->g.nf[k];
    for (int b = 0; b < 3; ++b)
      if (b != k && (p.ahi[k][b] != 0.0f || p.alo[k][b] != 0.0f)) p.diag = 0;
    p.inv_nf[k] = (float)(1.0 / (double)j->g.nf[k]);
  }
  // weighting parameters
  WeightArgs& w = j->wa;
  w.ngroups = j->ngroups;
  for (int gi = 0; gi < j->ngroups; ++gi) {
    w.pair[gi] = pr[gi];
    w.sp_a[gi] = sa[gi];
    w.sp_b[gi] = sb[gi];
  }
  w.weight_mode = d->weight_mode;
  for (int s = 0; s < d->n_species; ++s) {
    w.b_coh[s] = d->b_coh[s];
    for (int i = 0; i < 9; ++i) w.xff[s][i] = d->xff[s][i];
  }
  w.kappa = d->ff_convention == MPSQ_FF_STANDARD ? 1.0 / (16.0 * M_PI * M_PI) : 1.0 / 16.0;
  for (int b = 0; b < 3; ++b) {
    w.q0[b] = d->qphys_origin[b];
    for (int k = 0; k < 3; ++k) w.qs[k][b] = d->qphys_step[k][b];
  }
  w.extra_sq = d->qphys_extra_sq;
  w.wnorm = d->spatial_window ? (d->ndim == 2 ? 0.25 : 0.125) : 1.0;
  for (int s = 0; s < d->n_species; ++s) {
    w.b_coh_f[s] = (float)w.b_coh[s];
    for (int i = 0; i < 9; ++i) w.xff_f[s][i] = (float)w.xff[s][i];
    for (int i = 0; i < 4; ++i) w.xb2_f[s][i] = (float)(w.xff[s][2 * i + 1] * M_LOG2E);
  }
  w.kappa_f = (float)w.kappa;
  for (int b = 0; b < 3; ++b) {
    w.q0_f[b] = (float)w.q0[b];
    for (int k = 0; k < 3; ++k) w.qs_f[k][b] = (float)w.qs[k][b];
  }
  w.extra_f = (float)w.extra_sq;
  w.wnorm_f = (float)w.wnorm;
  w.store_species = d->store_species;
  w.n_species = d->n_species;

  // device memory
  const int64_t per = d->ndim == 3 ? 8 : 4;
  int64_t nsel = d->species_offset[d->n_species] - d->species_offset[0];
  j->cap = std::max<int64_t>(1, nsel * per);
  if (j->cap > (int64_t)INT32_MAX) {
    job_free(j);
    return fail(MPSQ_ERR_ARG, "job: too many atoms per frame for int32 bins");
  }
  const size_t cs = csize(prec);
  const int64_t nkeys = (int64_t)a.ngrid * j->g.n_tiles;
  cudaError_t e = cudaSuccess;
  auto A = [&](void** ptr, size_t bytes) {
    if (e == cudaSuccess) e = job_alloc(j, ptr, bytes);
  };
  A((void**)&j->traj, (size_t)d->n_frames * d->n_atoms_frame * sizeof(float4));
  A(&j->fine, (size_t)a.ngrid * j->g.n_fine * cs);
  A((void**)&j->counts, sizeof(int) * (nkeys + 1));
  A((void**)&j->starts, sizeof(int) * (nkeys + 1));
  A((void**)&j->perm, sizeof(int) * std::max<int64_t>(d->n_atoms_frame, 1));
  A((void**)&j->perm_counts, sizeof(int) * (nkeys + 2));
  A((void**)&j->perm_starts, sizeof(int) * (nkeys + 2));
  A(&j->recs, (size_t)j->cap * rsize(prec));
  A(&j->str, (size_t)j->cap * cs);
  const size_t prep_b = prep_cache_bytes(j);
  if (prep_b) A(&j->prep, prep_b);
  j->slab_nz = d->q_slab > 0 ? std::min<int64_t>(d->q_slab, j->g.m[2]) : 0;
  const int64_t store = j->store_modes();
  A(&j->cs, (size_t)d->n_frames * store * cs);
  if (d->store_species) A(&j->cs_species, (size_t)d->n_frames * d->n_species * store * cs);
  A((void**)&j->err, sizeof(int));
  for (int k = 0; k < 3 && e == cudaSuccess; ++k) {
    std::vector<double> c(j->g.m[k], 1.0);
    if (k < d->ndim) es_correction(j->es, j->g.nf[k], j->g.m[k], c.data());
    A(&j->corr[k], c.size() * (prec == MPSQ_FP64 ? 8 : 4));
    if (e != cudaSuccess) break;
    if (prec == MPSQ_FP64) {
      e = job_upload(j, j->corr[k], c.data(), c.size() * 8);
    } else {
      std::vector<float> cf(c.begin(), c.end());
      e = job_upload(j, j->corr[k], cf.data(), c.size() * 4);
    }
  }
  if (e == cudaSuccess)
    e = j->d.stream_ordered ? cudaMemsetAsync(j->err, 0, sizeof(int), j->s) : cudaMemset(j->err, 0, sizeof(int));
  if (e != cudaSuccess) {
    job_free(j);
    return fail(e == cudaErrorMemoryAllocation ? MPSQ_ERR_ALLOC : MPSQ_ERR_CUDA, "job_create: %s",
                cudaGetErrorString(e));
  }
  // Pruned fine-grid transform for FP32 volumes whose fine sizes factor into 2, 3, 5.
  bool pruned = prec == MPSQ_FP32 && d->ndim == 3 && !d->no_pruned_fft;
  for (int k = 0; k < 3 && pruned; ++k) pruned = fft_size_compiled((int)j->g.nf[k]);
  if (pruned) {
    for (int k = 0; k < 3; ++k) {
      j->h[k] = (int)(j->g.m[k] / 2);
      j->K[k] = 2 * j->h[k] + 1;
    }
    const int64_t n1 = j->g.nf[1], n2 = j->g.nf[2];
    e = job_alloc(j, (void**)&j->b1, sizeof(float2) * (size_t)a.ngrid * n2 * n1 * j->K[0]);
    for (int k = 0; k < 3 && e == cudaSuccess; ++k) {
      std::vector<float2> t(j->g.nf[k]);
      for (int64_t i = 0; i < j->g.nf[k]; ++i) {
        const double ang = -2.0 * M_PI * (double)i / (double)j->g.nf[k];
        t[i] = make_float2((float)std::cos(ang), (float)std::sin(ang));
      }
      e = job_alloc(j, (void**)&j->tw[k], sizeof(float2) * t.size());
      if (e == cudaSuccess) e = job_upload(j, j->tw[k], t.data(), sizeof(float2) * t.size());
    }
    if (e != cudaSuccess) {
      job_free(j);
      return fail(e == cudaErrorMemoryAllocation ? MPSQ_ERR_ALLOC : MPSQ_ERR_CUDA,
                  "job_create (pruned transform): %s", cudaGetErrorString(e));
    }
    j->pruned = true;
    // second lane (frames alternate between two streams) for multi-frame jobs when its scratch
    // is small next to the free device memory
    const char* lanes = getenv("MPSQ_LANES");
    const size_t extra = (size_t)a.ngrid * j->g.n_fine * cs + 2 * sizeof(int) * (nkeys + 1) +
                         (size_t)j->cap * (rsize(prec) + cs) +
                         sizeof(float2) * (size_t)a.ngrid * n2 * n1 * j->K[0] + prep_b;
    size_t free_b = 0, total_b = 0;
    if (!d->stream_ordered && d->n_frames > 1 && !(lanes && strcmp(lanes, "1") == 0) &&
        cudaMemGetInfo(&free_b, &total_b) == cudaSuccess && extra * 4 < free_b) {
      cudaError_t e2 = cudaStreamCreateWithFlags(&j->s2, cudaStreamNonBlocking);
      if (e2 == cudaSuccess) e2 = cudaEventCreateWithFlags(&j->fork, cudaEventDisableTiming);
      if (e2 == cudaSuccess) e2 = cudaEventCreateWithFlags(&j->join, cudaEventDisableTiming);
      auto A2 = [&](void** ptr, size_t bytes) {
        if (e2 == cudaSuccess) e2 = cudaMalloc(ptr, std::max<size_t>(bytes, 16));
      };
      A2(&j->fine2, (size_t)a.ngrid * j->g.n_fine * cs);
      A2((void**)&j->counts2, sizeof(int) * (nkeys + 1));
      A2((void**)&j->starts2, sizeof(int) * (nkeys + 1));
      A2(&j->recs2, (size_t)j->cap * rsize(prec));
      A2(&j->str2, (size_t)j->cap * cs);
      A2((void**)&j->b1_2, sizeof(float2) * (size_t)a.ngrid * n2 * n1 * j->K[0]);
      if (prep_b) A2(&j->prep2, prep_b);
      if (e2 == cudaSuccess) {
        j->lane2 = true;
      } else {  // run with one lane
        cudaGetLastError();
        cudaFree(j->fine2);
        cudaFree(j->counts2);
        cudaFree(j->starts2);
        cudaFree(j->recs2);
        cudaFree(j->str2);
        cudaFree(j->b1_2);
        cudaFree(j->prep2);
        j->fine2 = j->recs2 = j->str2 = j->prep2 = nullptr;
        j->counts2 = j->starts2 = nullptr;
        j->b1_2 = nullptr;
      }
    }
  } else {
    if (d->ndim == 3) {
      rc = make_xpruned_fft(j);
      if (rc) {
        job_free(j);
        return rc;
      }
    } else {
      rc = make_fft_plan(j->g, a.ngrid, prec, j->s, &j->fft);
      if (rc) {
        job_free(j);
        return rc;
      }
      j->have_fft = true;
    }
  }
  *out = j;
  return MPSQ_OK;
}

extern "C" int mpsq_job_destroy(mpsq_job* j) {
  if (j && !j->d.stream_ordered) {
    if (j->s2) cudaStreamSynchronize(j->s2);
    if (j->s) cudaStreamSynchronize(j->s);
  }
  job_free(j);   // stream-ordered: the frees follow the job's queued work on its stream
  return MPSQ_OK;
}

extern "C" int mpsq_job_set_frames_on(mpsq_job* j, const float* pos, int32_t first,
                                      int32_t count, int host, void* stream) {
  if (!j || !pos) return fail(MPSQ_ERR_ARG, "set_frames: null pointer");
  if (first < 0 || count < 0 || first + count > j->d.n_frames)
    return fail(MPSQ_ERR_ARG, "set_frames: frames [%d, %d) outside [0, %d)", first, first + count,
                j->d.n_frames);
  const size_t bytes = (size_t)count * j->d.n_atoms_frame * sizeof(float4);
  float4* dst = j->traj + (size_t)first * j->d.n_atoms_frame;
  MPSQ_CUDA_TRY(cudaMemcpyAsync(dst, pos, bytes, host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice,
                                (cudaStream_t)stream));
  return MPSQ_OK;
}

extern "C" int mpsq_job_set_frames(mpsq_job* j, const float* pos, int32_t first, int32_t count,
                                   int host) {
  if (!j) return fail(MPSQ_ERR_ARG, "set_frames: null job");
  return mpsq_job_set_frames_on(j, pos, first, count, host, j->s);
}

extern "C" int mpsq_job_set_cell_index(mpsq_job* j, const int32_t* at_ind, int host) {
  if (!j || !at_ind) return fail(MPSQ_ERR_ARG, "set_cell_index: null pointer");
  if (!j->at_ind) MPSQ_CUDA_TRY(job_alloc(j, (void**)&j->at_ind, (size_t)j->d.n_atoms_frame * sizeof(int4)));
  MPSQ_CUDA_TRY(cudaMemcpyAsync(j->at_ind, at_ind, (size_t)j->d.n_atoms_frame * sizeof(int4),
                                host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, j->s));
  return MPSQ_OK;
}

// Planes per slab of the z-slab pipeline for this job (0: whole-grid passes).  It applies to
// FP32 volumes on the pruned transform whose packed pairs spread on the tensor cores, with a
// slab that leaves room for the Y output at the start of the fine buffer.
static int zslab_planes(const mpsq_job* j) {
  const int zs = j->opt_zslab;
  if (zs <= 0 || !j->pruned || j->d.precision != MPSQ_FP32 || j->d.ndim != 3) return 0;
  const SpreadArgs& a = j->sa;
  if (!j->pa.pack || j->opt_spread != 0 || !spread_pair_mma_enabled() || a.w < 3 || a.w > 8 ||
      a.tile[0] != 16 || a.tile[1] != 16 || a.tile[2] != 16)
    return 0;
  const int64_t n0 = j->g.nf[0], n1 = j->g.nf[1], n2 = j->g.nf[2];
  if (zs >= n2 || n2 % 16 != 0) return 0;
  if (n2 * j->K[1] * j->K[0] + zs * n1 * n0 > a.n_fine) return 0;
  return zs;
}

template <typename T>
static int job_transform_body(mpsq_job* j, int32_t first, int32_t count) {
  using C = typename Cplx<T>::type;
  using R = typename RecOf<T>::type;
  cudaStream_t s = j->s;  // the stream of the current frame's lane
  const SpreadArgs& a = j->sa;
  const int64_t nkeys = (int64_t)a.ngrid * a.n_tiles;
  const int bt = 256;
  const unsigned nb = (unsigned)((j->d.n_atoms_frame + bt - 1) / bt);
  const int64_t nm = j->store_modes();
  const bool prof = j->profile;
  auto mark = [&](int k) -> int {
    if (prof) MPSQ_CUDA_TRY(cudaEventRecord(j->ev[k], s));
    return MPSQ_OK;
  };
  // two lanes: even frames of the call on the job's stream, odd ones on the second lane,
  // which first waits for everything queued on the job's stream (uploads included); the
  // job's stream waits for the second lane at the end
  const bool two = j->lane2 && j->opt_lanes == 2 && !prof && count > 1;
  cudaStream_t const main_s = j->s;
  // locality order from the first frame (atoms move little between frames; any order gives the
  // same records, a spatial one lets a warp's cursor atomics combine)
  if (count > 1 && j->ngroups > 0) {
    const float4* f0 = j->traj + (size_t)first * j->d.n_atoms_frame;
    MPSQ_CUDA_TRY(cudaMemsetAsync(j->perm_counts, 0, sizeof(int) * (nkeys + 2), main_s));
    job_perm_kernel<T, false><<<nb, bt, 0, main_s>>>(f0, j->at_ind, j->pa, a, nkeys,
                                                      j->perm_counts, j->perm_starts, j->perm);
    MPSQ_LAUNCH_CHECK();
    int rc = launch_scan<T>(j->perm_counts, j->perm_starts, nkeys + 1, main_s);
    if (rc) return rc;
    MPSQ_CUDA_TRY(cudaMemsetAsync(j->perm_counts, 0, sizeof(int) * (nkeys + 2), main_s));
    job_perm_kernel<T, true><<<nb, bt, 0, main_s>>>(f0, j->at_ind, j->pa, a, nkeys,
                                                     j->perm_counts, j->perm_starts, j->perm);
    MPSQ_LAUNCH_CHECK();
    j->perm_built = true;
  }
  const int* const perm = j->perm_built ? j->perm : nullptr;
  // unit strengths (no centre phase, no spatial window) are implied, not stored
  const bool unit_str = !j->pa.has_qc && !j->pa.window;
  if (two) {
    MPSQ_CUDA_TRY(cudaEventRecord(j->fork, main_s));
    MPSQ_CUDA_TRY(cudaStreamWaitEvent(j->s2, j->fork, 0));
  }
  for (int32_t t = first; t < first + count; ++t) {
    const bool odd = two && ((t - first) & 1);
    s = odd ? j->s2 : main_s;
    int* const counts = odd ? j->counts2 : j->counts;
    int* const starts = odd ? j->starts2 : j->starts;
    void* const recs = odd ? j->recs2 : j->recs;
    void* const str = unit_str ? nullptr : (odd ? j->str2 : j->str);
    void* const fine = odd ? j->fine2 : j->fine;
    float2* const b1 = odd ? j->b1_2 : j->b1;
    const float4* frame = j->traj + (size_t)t * j->d.n_atoms_frame;
    // FP32 split path: atoms prepared once, by the counting pass
    const bool cached = sizeof(T) == 4 && j->prep != nullptr;
    PrepCache pc{};
    if (cached) {
      char* base = static_cast<char*>(odd ? j->prep2 : j->prep);
      const size_t n = (size_t)j->d.n_atoms_frame;
      pc.cell = reinterpret_cast<int4*>(base);
      pc.d2 = reinterpret_cast<float*>(base + 16 * n);
      pc.c = unit_str ? nullptr : reinterpret_cast<float2*>(base + 24 * n);
    }
    if (mark(0)) return MPSQ_ERR_CUDA;
    PhaseRange bin_range("mpsq:sort");
    MPSQ_CUDA_TRY(cudaMemsetAsync(counts, 0, sizeof(int) * (nkeys + 1), s));
    if (j->ngroups > 0) {
      if (cached)
        job_bin_count_split_kernel<<<nb, bt, 0, s>>>(frame, j->at_ind, perm, j->pa, a, counts, pc,
                                                     j->err);
      else
        job_bin_kernel<T, false><<<nb, bt, 0, s>>>(frame, j->at_ind, perm, j->pa, a, counts,
                                                   starts, (R*)recs, (C*)str, j->cap, j->err);
      MPSQ_LAUNCH_CHECK();
    }
    int rc = launch_scan<T>(counts, starts, nkeys, s);
    if (rc) return rc;
    MPSQ_CUDA_TRY(cudaMemsetAsync(counts, 0, sizeof(int) * (nkeys + 1), s));
    if (j->ngroups > 0) {
      if (cached)
        job_bin_scatter_split_kernel<<<nb, bt, 0, s>>>(j->d.n_atoms_frame, pc, a, counts, starts,
                                                       (RecF*)recs, (float2*)str, j->cap, j->err);
      else
        job_bin_kernel<T, true><<<nb, bt, 0, s>>>(frame, j->at_ind, perm, j->pa, a, counts,
                                                  starts, (R*)recs, (C*)str, j->cap, j->err);
      MPSQ_LAUNCH_CHECK();
    }
    if (mark(1)) return MPSQ_ERR_CUDA;
    nvtxRangePop();                       // end of mpsq:sort
    nvtxRangePushA("mpsq:spread");
    const int zs = prof ? 0 : zslab_planes(j);
    if (zs == 0) {   // otherwise spread slab by slab with the X and Y passes, below
      rc = launch_spread<T>(a, (const R*)recs, (const C*)str, starts, j->pa.pack != 0, (C*)fine,
                            s, j->opt_spread == 0, j->opt_repro != 0);
      if (rc) return rc;
    }
    if (mark(2)) return MPSQ_ERR_CUDA;
    nvtxRangePop();                       // end of mpsq:spread
    nvtxRangePushA("mpsq:fft+deconv");    // popped by bin_range at the end of the frame
    C* csf = (C*)j->cs + (size_t)t * nm;
    C* css = j->cs_species ? (C*)j->cs_species + (size_t)t * j->d.n_species * nm : nullptr;
    bool done = false;
    if constexpr (sizeof(T) == 4) {
      if (j->pruned) {
        PruneLaunch pl;
        pl.fine = (const float2*)fine;
        pl.n_fine = a.n_fine;
        pl.b1 = b1;
        pl.b2 = (float2*)fine;  // the fine grids are dead after pass X
        for (int k = 0; k < 3; ++k) {
          pl.n[k] = (int)j->g.nf[k];
          pl.m[k] = (int)j->g.m[k];
          pl.h[k] = j->h[k];
          pl.K[k] = j->K[k];
          pl.tw[k] = j->tw[k];
          pl.c[k] = (const float*)j->corr[k];
        }
        pl.ngrid = a.ngrid;
        pl.ngroups = j->ngroups;
        pl.xrows = j->opt_xrows;
        pl.z0 = (int)j->slab_z0;
        pl.nz = (int)j->slab_planes();
        pl.fz0 = 0;
        pl.fnz = pl.n[2];
        pl.s = s;
        if (zs > 0) {
          // z-slab pipeline: the tiles of zs fine-grid planes are spread into a slab-sized
          // region at the end of the fine buffer (beyond the Y output at its start), and the
          // X and Y passes of those planes follow at once, so the slab and its X output
          // (reused for every slab) are read back from L2
          const int64_t n0 = j->g.nf[0], n1 = j->g.nf[1], n2 = j->g.nf[2];
          const int64_t nl = (int64_t)a.ntile[0] * a.ntile[1];
          float2* fslab = (float2*)fine + (int64_t)a.ngrid * (a.n_fine - zs * n1 * n0);
          for (int64_t z0 = 0; z0 < n2; z0 += zs) {
            const int nzp = (int)std::min<int64_t>(zs, n2 - z0);
            const int64_t gstride = nzp * n1 * n0;
            for (int g = 0; g < a.ngrid; ++g) {
              rc = launch_spread_pair_mma(a, (const RecF*)recs, nullptr, (const float2*)str, 0,
                                          starts, (int)((nzp / 16) * nl), 1, fslab, s,
                                          (int64_t)g * a.n_tiles + (z0 / 16) * nl, (int)z0,
                                          gstride, j->opt_repro != 0);
              if (rc) return rc;
            }
            pl.fine = fslab;
            pl.n_fine = gstride;
            pl.fz0 = (int)z0;
            pl.fnz = nzp;
            rc = run_pruned_xy(pl);
            if (rc) return rc;
          }
        } else {
          rc = run_pruned_xy(pl);
          if (rc) return rc;
        }
        if (prof) MPSQ_CUDA_TRY(cudaEventRecord(j->ev[3], s));
        rc = run_pruned_z(pl, j->wa, (float2*)csf, (float2*)css);
        if (rc) return rc;
        done = true;
      }
    }
    if (!done) {
      rc = j->have_xfft ? exec_xpruned_fft(j) : exec_fft(j->fft, j->d.precision, j->fine,
                                                          CUFFT_FORWARD);
      if (rc) return rc;
      if (mark(3)) return MPSQ_ERR_CUDA;
      const dim3 dgrid((unsigned)((j->g.m[0] + 127) / 128), (unsigned)j->g.m[1],
                       (unsigned)j->slab_planes());
      job_deconv_kernel<T><<<dgrid, 128, 0, s>>>(
          a, (int)j->g.m[0], (int)j->g.m[1], (int)j->g.m[2], (int)j->slab_z0,
          (int)j->slab_planes(), (const C*)j->fine, (const T*)j->corr[0],
          (const T*)j->corr[1], (const T*)j->corr[2], j->wa, csf, css);
      MPSQ_LAUNCH_CHECK();
    }
    if (prof) {
      if (mark(4)) return MPSQ_ERR_CUDA;
      MPSQ_CUDA_TRY(cudaEventSynchronize(j->ev[4]));
      for (int k = 0; k < 4; ++k) {
        float ms = 0.0f;
        MPSQ_CUDA_TRY(cudaEventElapsedTime(&ms, j->ev[k], j->ev[k + 1]));
        j->stage_ms[k] += ms;
      }
      j->stage_frames += 1;
    }
  }
  if (two) {
    MPSQ_CUDA_TRY(cudaEventRecord(j->join, j->s2));
    MPSQ_CUDA_TRY(cudaStreamWaitEvent(main_s, j->join, 0));
  }
  return MPSQ_OK;
}

static int job_transform_direct(mpsq_job* j, int32_t first, int32_t count) {
  return j->d.precision == MPSQ_FP64 ? job_transform_body<double>(j, first, count)
                                     : job_transform_body<float>(j, first, count);
}

// The frame loop of one transform call captured once as a CUDA graph (per (first, count)) and
// replayed: the same kernels and copies, issued by one graph launch instead of ~7 launches per
// frame.  Capture runs on a private stream (the job's stream may be the legacy default stream,
// which cannot be captured); the graph is launched on the job's stream.
static int job_transform_graph(mpsq_job* j, int32_t first, int32_t count) {
  for (const auto& gr : j->graphs) {
    if (gr.first == first && gr.count == count) {
      MPSQ_CUDA_TRY(cudaGraphLaunch(gr.exec, j->s));
      count_launch((int)gr.launches);
      return MPSQ_OK;
    }
  }
  cudaStream_t cap = nullptr;
  MPSQ_CUDA_TRY(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
  cudaStream_t const user = j->s;
  const int64_t n0 = g_launches.load();
  cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
  int rc = MPSQ_OK;
  if (e == cudaSuccess) {
    j->s = cap;
    rc = job_transform_direct(j, first, count);
    j->s = user;
  }
  cudaGraph_t graph = nullptr;
  if (e == cudaSuccess) {
    const cudaError_t e2 = cudaStreamEndCapture(cap, &graph);
    if (rc == MPSQ_OK) e = e2;
  }
  const int64_t launches = g_launches.load() - n0;
  count_launch(-(int)launches);      // captured, not run
  cudaGraphExec_t exec = nullptr;
  if (e == cudaSuccess && rc == MPSQ_OK) e = cudaGraphInstantiate(&exec, graph, 0);
  if (graph) cudaGraphDestroy(graph);
  cudaStreamDestroy(cap);
  if (rc) return rc;
  if (e != cudaSuccess) return fail(MPSQ_ERR_CUDA, "transform graph: %s", cudaGetErrorString(e));
  if (j->graphs.size() >= 16) {      // bounded cache: drop the oldest
    cudaGraphExecDestroy(j->graphs.front().exec);
    j->graphs.erase(j->graphs.begin());
  }
  j->graphs.push_back({first, count, exec, launches});
  MPSQ_CUDA_TRY(cudaGraphLaunch(exec, j->s));
  count_launch((int)launches);
  return MPSQ_OK;
}

extern "C" int mpsq_job_transform(mpsq_job* j, int32_t first, int32_t count) {
  if (!j) return fail(MPSQ_ERR_ARG, "transform: null job");
  if (first < 0 || count < 0 || first + count > j->d.n_frames)
    return fail(MPSQ_ERR_ARG, "transform: frames outside the trajectory");
  if (j->opt_graph && !j->profile && count > 0) return job_transform_graph(j, first, count);
  return job_transform_direct(j, first, count);
}

static void drop_graphs(mpsq_job* j) {
  for (auto& gr : j->graphs) cudaGraphExecDestroy(gr.exec);
  j->graphs.clear();
}

extern "C" int mpsq_job_set_option(mpsq_job* j, int option, int value) {
  if (!j) return fail(MPSQ_ERR_ARG, "set_option: null job");
  switch (option) {
    case MPSQ_OPT_GRAPH:
      if (value != 0 && value != 1) return fail(MPSQ_ERR_ARG, "set_option: graph must be 0 or 1");
      j->opt_graph = value;
      break;
    case MPSQ_OPT_SPREAD:
      if (value != 0 && value != 1) return fail(MPSQ_ERR_ARG, "set_option: spread must be 0 or 1");
      j->opt_spread = value;
      break;
    case MPSQ_OPT_XROWS:
      if (value != 4 && value != 8) return fail(MPSQ_ERR_ARG, "set_option: X rows must be 4 or 8");
      j->opt_xrows = value;
      break;
    case MPSQ_OPT_LANES:
      if (value != 1 && value != 2) return fail(MPSQ_ERR_ARG, "set_option: lanes must be 1 or 2");
      j->opt_lanes = value;
      break;
    case MPSQ_OPT_ZSLAB:
      if (value < 0 || value % 16 != 0 || value > 4096)
        return fail(MPSQ_ERR_ARG, "set_option: z-slab planes must be 0 or a multiple of 16");
      j->opt_zslab = value;
      break;
    case MPSQ_OPT_REPRODUCIBLE:
      if (value != 0 && value != 1)
        return fail(MPSQ_ERR_ARG, "set_option: reproducible must be 0 or 1");
      j->opt_repro = value;
      break;
    default:
      return fail(MPSQ_ERR_ARG, "set_option: unknown option %d", option);
  }
  drop_graphs(j);   // captured graphs hold the previous choice
  return MPSQ_OK;
}

// Autotuner: times the transform of frames [first, first + count) under every combination of
// the run-time choices that applies to this job (spreading kernel, X-pass rows, frame lanes,
// graph replay, z-slab pipeline), keeps the fastest and, given a cache file, records it there
// under a key of the job's shape and the device's SM count, so that later jobs of the same
// shape take the choice without timing.
// Cache lines: "<key> <graph> <spread> <xrows> <lanes> <zslab> <ms>".
static std::string tune_key(const mpsq_job* j) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  char buf[256];
  snprintf(buf, sizeof(buf), "mpsq-tune-2:p%d:d%d:n%lldx%lldx%lld:w%d:g%d:pk%d:pr%d:l%d:sm%d",
           j->d.precision, j->d.ndim, (long long)j->g.nf[0], (long long)j->g.nf[1],
           (long long)j->g.nf[2], j->es.w, j->sa.ngrid, j->pa.pack, j->pruned ? 1 : 0,
           j->lane2 ? 1 : 0, sms);
  return buf;
}

extern "C" int mpsq_job_autotune(mpsq_job* j, int32_t first, int32_t count, const char* cache_path,
                                 int* choice, double* best_ms) {
  if (!j) return fail(MPSQ_ERR_ARG, "autotune: null job");
  if (first < 0 || count < 1 || first + count > j->d.n_frames)
    return fail(MPSQ_ERR_ARG, "autotune: frames outside the trajectory");
  const std::string key = tune_key(j);
  int best[5] = {j->opt_graph, j->opt_spread, j->opt_xrows, j->opt_lanes, j->opt_zslab};
  double best_t = -1.0;
  if (cache_path && *cache_path) {
    if (FILE* f = fopen(cache_path, "r")) {
      char line[512], k[256];
      while (fgets(line, sizeof(line), f)) {
        int g, sp, xr, ln, zs;
        double ms;
        if (sscanf(line, "%255s %d %d %d %d %d %lf", k, &g, &sp, &xr, &ln, &zs, &ms) == 7 &&
            key == k) {
          best[0] = g;
          best[1] = sp;
          best[2] = xr;
          best[3] = ln;
          best[4] = zs;
          best_t = ms;
        }
      }
      fclose(f);
    }
  }
  const bool cached = best_t >= 0.0;
  if (!cached) {
    const bool fma_ok = j->d.precision == MPSQ_FP32 && j->d.ndim == 3 && j->pa.pack != 0;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    MPSQ_CUDA_TRY(cudaEventCreate(&e0));
    MPSQ_CUDA_TRY(cudaEventCreate(&e1));
    int rc = MPSQ_OK;
    // candidate settings {graph, spread, xrows, lanes, zslab}; the z-slab pipeline is tried at
    // 64 planes where it applies (tensor-core spreading of pairs on the pruned transform)
    const int zs_saved = j->opt_zslab, sp_saved = j->opt_spread;
    j->opt_spread = 0;
    j->opt_zslab = 64;
    const bool zs_ok = zslab_planes(j) > 0;
    j->opt_zslab = zs_saved;
    j->opt_spread = sp_saved;
    std::vector<std::array<int, 5>> cand;
    for (int g = 0; g <= 1; ++g)
      for (int sp = 0; sp <= (fma_ok ? 1 : 0); ++sp)
        for (int xr : {8, 4})
          for (int ln = 2; ln >= 1; --ln)
            for (int zs : {0, 64})
              if ((j->pruned || xr == 8) && (j->lane2 || ln == 1) && (!zs || (zs_ok && sp == 0)))
                cand.push_back({g, sp, xr, ln, zs});
    for (size_t c = 0; c < cand.size() && !rc; ++c) {
      const std::array<int, 5>& o = cand[c];
      j->opt_graph = o[0];
      j->opt_spread = o[1];
      j->opt_xrows = o[2];
      j->opt_lanes = o[3];
      j->opt_zslab = o[4];
      drop_graphs(j);
      rc = mpsq_job_transform(j, first, count);           // warm-up (and capture)
      if (!rc && cudaEventRecord(e0, j->s) != cudaSuccess) rc = MPSQ_ERR_CUDA;
      for (int r = 0; r < 2 && !rc; ++r) rc = mpsq_job_transform(j, first, count);
      if (!rc && cudaEventRecord(e1, j->s) != cudaSuccess) rc = MPSQ_ERR_CUDA;
      if (!rc && cudaEventSynchronize(e1) != cudaSuccess) rc = MPSQ_ERR_CUDA;
      float ms = 0.0f;
      if (!rc && cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) rc = MPSQ_ERR_CUDA;
      ms *= 0.5f;
      if (!rc && (best_t < 0.0 || ms < best_t)) {
        best_t = ms;
        for (int i = 0; i < 5; ++i) best[i] = o[i];
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) {
      if (rc == MPSQ_ERR_CUDA) fail(MPSQ_ERR_CUDA, "autotune: %s", cudaGetErrorString(cudaGetLastError()));
      return rc;
    }
  }
  j->opt_graph = best[0];
  j->opt_spread = best[1];
  j->opt_xrows = best[2];
  j->opt_lanes = best[3];
  j->opt_zslab = best[4];
  drop_graphs(j);
  if (!cached && cache_path && *cache_path) {
    if (FILE* f = fopen(cache_path, "a")) {
      fprintf(f, "%s %d %d %d %d %d %.4f\n", key.c_str(), best[0], best[1], best[2], best[3],
              best[4], best_t);
      fclose(f);
    }
  }
  if (choice) {
    choice[0] = best[0];
    choice[1] = best[1];
    choice[2] = best[2];
    choice[3] = best[3];
  }
  if (best_ms) *best_ms = best_t;
  return MPSQ_OK;
}

extern "C" int mpsq_job_get_option(const mpsq_job* j, int option, int* value) {
  if (!j || !value) return fail(MPSQ_ERR_ARG, "get_option: null pointer");
  switch (option) {
    case MPSQ_OPT_GRAPH: *value = j->opt_graph; break;
    case MPSQ_OPT_SPREAD: *value = j->opt_spread; break;
    case MPSQ_OPT_XROWS: *value = j->opt_xrows; break;
    case MPSQ_OPT_LANES: *value = j->opt_lanes; break;
    case MPSQ_OPT_ZSLAB: *value = j->opt_zslab; break;
    case MPSQ_OPT_REPRODUCIBLE: *value = j->opt_repro; break;
    default: return fail(MPSQ_ERR_ARG, "get_option: unknown option %d", option);
  }
  return MPSQ_OK;
}

template <typename T>
static int job_onephonon_t(mpsq_job* j, int32_t first, int32_t count, int32_t plane, int32_t n_bz,
                           float qx_min, float qy_min) {
  using C = typename Cplx<T>::type;
  const int n1 = j->d.n_row[0], n2 = j->d.n_row[1];
  const int m0 = (int)j->d.n_modes[0], m1 = (int)j->d.n_modes[1];
  const int ns = j->d.n_species;
  const size_t usz = (size_t)ns * 2 * n1 * n2 * sizeof(C);
  if (!j->oneph_u) MPSQ_CUDA_TRY(job_alloc(j, &j->oneph_u, usz));
  if (!j->have_oneph_fft) {
    int n[2] = {n2, n1};
    MPSQ_CUFFT_TRY(cufftPlanMany(&j->oneph_fft, 2, n, nullptr, 1, n1 * n2, nullptr, 1, n1 * n2,
                                 sizeof(T) == 8 ? CUFFT_Z2Z : CUFFT_C2C, 2 * ns));
    j->have_oneph_fft = true;
  }
  MPSQ_CUFFT_TRY(cufftSetStream(j->oneph_fft, j->s));
  // nqx_min = n_row * (qx_min - floor(qx_min)), FP32, truncated (:1039-1040)
  const int nqx_min = (int)(float)((float)n1 * (qx_min - std::floor(qx_min)));
  const int nqy_min = (int)(float)((float)n2 * (qy_min - std::floor(qy_min)));
  const int bt = 256;
  const unsigned nb = (unsigned)((j->d.n_atoms_frame + bt - 1) / bt);
  const int64_t nm = j->g.n_modes;
  for (int32_t t = first; t < first + count; ++t) {
    MPSQ_CUDA_TRY(cudaMemsetAsync(j->oneph_u, 0, usz, j->s));
    oneph_scatter_kernel<T><<<nb, bt, 0, j->s>>>(j->traj + (size_t)t * j->d.n_atoms_frame,
                                                  j->at_ind, j->pa, plane, j->oneph_base, n1, n2,
                                                  (C*)j->oneph_u);
    MPSQ_LAUNCH_CHECK();
    if constexpr (sizeof(T) == 8) {
      MPSQ_CUFFT_TRY(cufftExecZ2Z(j->oneph_fft, (cufftDoubleComplex*)j->oneph_u,
                                  (cufftDoubleComplex*)j->oneph_u, CUFFT_FORWARD));
    } else {
      MPSQ_CUFFT_TRY(cufftExecC2C(j->oneph_fft, (cufftComplex*)j->oneph_u,
                                  (cufftComplex*)j->oneph_u, CUFFT_FORWARD));
    }
    C* csf = (C*)j->cs + (size_t)t * nm;
    C* css = j->cs_species ? (C*)j->cs_species + (size_t)t * ns * nm : nullptr;
    oneph_expand_kernel<T><<<dim3((unsigned)((m0 + 127) / 128), (unsigned)m1), 128, 0, j->s>>>(
        (const C*)j->oneph_u, j->pa, plane, j->oneph_base, n1, n2, m0, m1, n_bz, qx_min, qy_min,
        nqx_min, nqy_min, j->wa, csf, css);
    MPSQ_LAUNCH_CHECK();
  }
  return MPSQ_OK;
}

extern "C" int mpsq_job_transform_onephonon(mpsq_job* j, int32_t first, int32_t count,
                                            int32_t plane, int32_t n_bz, float qx_min,
                                            float qy_min, const float* at_base) {
  if (!j || !at_base) return fail(MPSQ_ERR_ARG, "transform_onephonon: null pointer");
  if (first < 0 || count < 0 || first + count > j->d.n_frames)
    return fail(MPSQ_ERR_ARG, "transform_onephonon: frames outside the trajectory");
  if (j->d.input_method != MPSQ_CELL || j->d.ndim != 2)
    return fail(MPSQ_ERR_ARG, "transform_onephonon: CELL input on a Q plane only (the reference "
                "turns the mode off for BULK input)");
  if (plane != 1 && plane != 2)
    return fail(MPSQ_ERR_ARG, "transform_onephonon: plane must be 1 (hk0) or 2 (hhl), got %d", plane);
  const int* nr = j->d.n_row;
  if (nr[0] != nr[1] || (plane == 2 && nr[2] != nr[0]))
    return fail(MPSQ_ERR_ARG, "transform_onephonon: needs n_row(1) = n_row(2) (= n_row(3) on "
                "(hhl)); the reference's index ranges mix the axes otherwise");
  if (n_bz < 1 || (int64_t)n_bz * nr[0] > j->d.n_modes[0] || (int64_t)n_bz * nr[1] > j->d.n_modes[1])
    return fail(MPSQ_ERR_ARG, "transform_onephonon: %d zones of %d cells exceed the %lld x %lld plane",
                n_bz, nr[0], (long long)j->d.n_modes[0], (long long)j->d.n_modes[1]);
  if (!j->at_ind) return fail(MPSQ_ERR_STATE, "transform_onephonon: set the cell indices first");
  if (!j->oneph_base) MPSQ_CUDA_TRY(job_alloc(j, (void**)&j->oneph_base, sizeof(float) * 3 * MPSQ_MAX_SPECIES));
  MPSQ_CUDA_TRY(cudaMemcpyAsync(j->oneph_base, at_base, sizeof(float) * 3 * j->d.n_species,
                                cudaMemcpyHostToDevice, j->s));
  // (a host-to-device copy from pageable memory has left the caller's buffer on return)
  return j->d.precision == MPSQ_FP64
             ? job_onephonon_t<double>(j, first, count, plane, n_bz, qx_min, qy_min)
             : job_onephonon_t<float>(j, first, count, plane, n_bz, qx_min, qy_min);
}

extern "C" int mpsq_job_profile(mpsq_job* j, int enable) {
  if (!j) return fail(MPSQ_ERR_ARG, "profile: null job");
  if (enable)
    for (auto& e : j->ev)
      if (!e) MPSQ_CUDA_TRY(cudaEventCreate(&e));
  j->profile = enable != 0;
  return MPSQ_OK;
}

extern "C" int mpsq_job_stage_ms(mpsq_job* j, double* ms4, int64_t* frames, int reset) {
  if (!j) return fail(MPSQ_ERR_ARG, "stage_ms: null job");
  if (ms4)
    for (int k = 0; k < 4; ++k) ms4[k] = j->stage_ms[k];
  if (frames) *frames = j->stage_frames;
  if (reset) {
    for (double& v : j->stage_ms) v = 0.0;
    j->stage_frames = 0;
  }
  return MPSQ_OK;
}

extern "C" int mpsq_job_amplitudes(mpsq_job* j, void** cs_dev) {
  if (!j || !cs_dev) return fail(MPSQ_ERR_ARG, "amplitudes: null pointer");
  *cs_dev = j->cs;
  return MPSQ_OK;
}

extern "C" int mpsq_job_info(const mpsq_job* j, int* width, int64_t* fine_grid, int* n_grids,
                             int* pruned, int* lanes) {
  if (!j) return fail(MPSQ_ERR_ARG, "job_info: null job");
  if (width) *width = j->es.w;
  if (fine_grid)
    for (int k = 0; k < 3; ++k) fine_grid[k] = j->g.nf[k];
  if (n_grids) *n_grids = j->sa.ngrid;
  if (pruned) *pruned = j->pruned ? 1 : 0;
  if (lanes) *lanes = j->lane2 ? 2 : 1;
  return MPSQ_OK;
}

extern "C" int mpsq_job_set_q_slab(mpsq_job* j, int64_t z0) {
  if (!j) return fail(MPSQ_ERR_ARG, "set_q_slab: null job");
  if (j->slab_nz == 0) return fail(MPSQ_ERR_STATE, "set_q_slab: job created without q_slab");
  if (z0 < 0 || z0 >= j->g.m[2])
    return fail(MPSQ_ERR_ARG, "set_q_slab: z0 = %lld outside [0, %lld)", (long long)z0,
                (long long)j->g.m[2]);
  j->slab_z0 = z0;
  drop_graphs(j);   // captured graphs hold the previous slab
  return MPSQ_OK;
}

extern "C" int mpsq_job_sync(mpsq_job* j) {
  if (!j) return fail(MPSQ_ERR_ARG, "sync: null job");
  MPSQ_CUDA_TRY(cudaStreamSynchronize(j->s));
  return check_dev_error(j->err, j->s);
}

// ---- accessor used by the time-axis unit
namespace mpsq {
JobView job_view(mpsq_job* j) {
  JobView v;
  v.precision = j->d.precision;
  v.s = j->s;
  v.cs = j->cs;
  v.cs_species = j->cs_species;
  v.n_q = j->store_modes();
  v.slab = j->slab_nz > 0;
  v.n_frames = j->d.n_frames;
  v.n_species = j->d.n_species;
  for (int k = 0; k < 3; ++k) v.m[k] = j->g.m[k];
  v.store_species = j->d.store_species;
  return v;
}
}  // namespace mpsq
