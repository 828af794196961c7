// Time-axis kernels on the amplitude store cs(t, Q) of a job (frame-major, Q fastest):
//  * total S(Q) = sum_t |cs|^2 / nfile                      (mp_sqom56.f90:1381-1387)
//  * E=const map, sliding Hann window, one frequency bin     (:1437-1478, window :941-948)
//  * E(Q) dispersion cut, windowed DFT per start frame       (:1480-1517)
//  * Gaussian-window spectrum over the whole run (one FFT per Q in shared memory)
//  * I(Q,t) maps and path cuts (the j_sq /= 1 branch, :1467-1472, :1504-1510)
//  * atom-pair forms of the E=const map and E(Q) cut (raw sum of two species, :1460-1464)
// The ω-resolved forms subtract the elastic mean <cs>_t first (:1177-1185, :1359-1376) and
// optionally scale by 1/|Q| (:1373).  Sums over frames are compensated (FP32) or FP64.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "fft_smem.cuh"
#include "mpsq_internal.h"

namespace mpsq {

template <typename T> struct Acc;  // compensated accumulator
template <> struct Acc<float> {
  float s = 0.0f, c = 0.0f;
  __device__ __forceinline__ void add(float v) {
    const float y = v - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};
template <> struct Acc<double> {
  double s = 0.0;
  __device__ __forceinline__ void add(double v) { s += v; }
  __device__ __forceinline__ double value() const { return s; }
};

template <typename T>
__global__ void sq_total_kernel(const typename Cplx<T>::type* __restrict__ cs, int64_t nq,
                                int nt, double scale, float* __restrict__ out) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  Acc<T> a;
  for (int t = 0; t < nt; ++t) {
    const auto v = cs[(int64_t)t * nq + q];
    a.add(v.x * v.x + v.y * v.y);
  }
  out[q] = (float)(a.value() * scale);
}

// The time series a map is formed from: x(t, q) = a[t*stride + q] (+ b[t*stride + q]).  The
// job's weighted amplitudes (a = cs, stride n_Q, centred: the elastic mean is subtracted) or
// the raw sum of two stored species amplitudes (the atom-pair modes, not centred).
template <typename T>
struct Series {
  const typename Cplx<T>::type* a;
  const typename Cplx<T>::type* b;
  int64_t stride;
  int center;
};

// Loads a [nt x QT] tile of the series into shared memory, subtracts the column means (if
// centred) and applies the optional 1/|Q| factor.  Thread layout: column = tid % QT,
// part = tid / QT.
template <typename T>
__device__ void load_centered_tile(Series<T> src, int64_t nq, int nt, int64_t q0, int QT,
                                   const float* __restrict__ q2n, typename Cplx<T>::type* xs,
                                   T* red_re, T* red_im) {
  using C = typename Cplx<T>::type;
  const int tid = threadIdx.x, NT = blockDim.x;
  for (int e = tid; e < nt * QT; e += NT) {
    const int t = e / QT, c = e % QT;
    const int64_t q = q0 + c;
    C v;
    v.x = 0;
    v.y = 0;
    if (q < nq) {
      v = src.a[(int64_t)t * src.stride + q];
      if (src.b) {
        const C u = src.b[(int64_t)t * src.stride + q];
        v.x += u.x;
        v.y += u.y;
      }
    }
    xs[e] = v;
  }
  __syncthreads();
  if (!src.center) {
    if (q2n) {
      for (int e = tid; e < nt * QT; e += NT) {
        const int64_t q = q0 + e % QT;
        const T f = q < nq ? (T)q2n[q] : (T)1;
        C v = xs[e];
        v.x *= f;
        v.y *= f;
        xs[e] = v;
      }
      __syncthreads();
    }
    return;
  }
  const int col = tid % QT, part = tid / QT, nparts = NT / QT;
  T sr = 0, si = 0;
  if (part < nparts)
    for (int t = part; t < nt; t += nparts) {
      sr += xs[t * QT + col].x;
      si += xs[t * QT + col].y;
    }
  red_re[tid] = sr;
  red_im[tid] = si;
  __syncthreads();
  if (tid < QT) {
    T mr = 0, mi = 0;
    for (int p = 0; p < nparts; ++p) {
      mr += red_re[p * QT + tid];
      mi += red_im[p * QT + tid];
    }
    red_re[NT + tid] = mr / (T)nt;
    red_im[NT + tid] = mi / (T)nt;
  }
  __syncthreads();
  for (int e = tid; e < nt * QT; e += NT) {
    const int c = e % QT;
    const int64_t q = q0 + c;
    const T f = (q2n && q < nq) ? (T)q2n[q] : (T)1;
    C v = xs[e];
    v.x = (v.x - red_re[NT + c]) * f;
    v.y = (v.y - red_im[NT + c]) * f;
    xs[e] = v;
  }
  __syncthreads();
}

// E=const map: S(Q) = sum_{t0} | sum_i ph_i x(t0+i) |^2 with ph_i = t_wind_i exp(-2 pi i
// (j_freq-1)(i - n_int/2)/n_int) (0-based i), times scale.
template <typename T>
__global__ void econst_kernel(Series<T> cs, int64_t nq, int nt,
                              int QT, int n_int, const float* __restrict__ t_wind, int jf,
                              const float* __restrict__ q2n, double scale,
                              float* __restrict__ out) {
  using C = typename Cplx<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int NT = blockDim.x;
  C* xs = reinterpret_cast<C*>(smem_raw);
  C* ph = xs + (size_t)nt * QT;
  T* red_re = reinterpret_cast<T*>(ph + n_int);
  T* red_im = red_re + NT + QT;
  const int64_t q0 = (int64_t)blockIdx.x * QT;
  const int tid = threadIdx.x;
  for (int i = tid; i < n_int; i += NT) {
    const long long r = ((long long)jf * (long long)(i - n_int / 2)) % n_int;
    T sn, cn;
    if (sizeof(T) == 8) {
      double s_, c_;
      sincospi(-2.0 * (double)r / n_int, &s_, &c_);
      sn = (T)s_;
      cn = (T)c_;
    } else {
      float s_, c_;
      sincospif(-2.0f * (float)r / (float)n_int, &s_, &c_);
      sn = (T)s_;
      cn = (T)c_;
    }
    C v;
    v.x = cn * (T)t_wind[i];
    v.y = sn * (T)t_wind[i];
    ph[i] = v;
  }
  load_centered_tile<T>(cs, nq, nt, q0, QT, q2n, xs, red_re, red_im);
  const int col = tid % QT, part = tid / QT, nparts = NT / QT;
  const int n0 = nt - n_int + 1;
  Acc<T> acc;
  if (part < nparts)
    for (int t0 = part; t0 < n0; t0 += nparts) {
      T xr = 0, xi = 0;
      for (int i = 0; i < n_int; ++i) {
        const C a = ph[i], b = xs[(t0 + i) * QT + col];
        xr += a.x * b.x - a.y * b.y;
        xi += a.x * b.y + a.y * b.x;
      }
      acc.add(xr * xr + xi * xi);
    }
  __syncthreads();
  red_re[tid] = (T)acc.value();
  __syncthreads();
  if (tid < QT) {
    double s = 0.0;
    for (int p = 0; p < nparts; ++p) s += (double)red_re[p * QT + tid];
    const int64_t q = q0 + tid;
    if (q < nq) out[q] = (float)(s * scale);
  }
}

// Dispersion: for path point p (one CTA), acc[f] = sum_{t0} |sum_i w_i x(t0+i) e^{-2 pi i f i/n}|^2.
template <typename T>
__global__ void dispersion_kernel(Series<T> cs, int64_t nq,
                                  int nt, const int64_t* __restrict__ qidx, int n_int,
                                  const float* __restrict__ t_wind, int n_freq,
                                  const float* __restrict__ q2n, double scale,
                                  float* __restrict__ out) {
  using C = typename Cplx<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int NT = blockDim.x, tid = threadIdx.x;
  C* xs = reinterpret_cast<C*>(smem_raw);
  C* tw = xs + nt;
  T* red_re = reinterpret_cast<T*>(tw + n_int);
  T* red_im = red_re + NT + 1;
  const int64_t q = qidx[blockIdx.x];
  if (q < 0 || q >= nq) {
    for (int f = tid; f < n_freq; f += NT) out[(int64_t)blockIdx.x * n_freq + f] = 0.0f;
    return;
  }
  for (int i = tid; i < n_int; i += NT) {
    T sn, cn;
    if (sizeof(T) == 8) {
      double s_, c_;
      sincospi(-2.0 * (double)i / n_int, &s_, &c_);
      sn = (T)s_;
      cn = (T)c_;
    } else {
      float s_, c_;
      sincospif(-2.0f * (float)i / (float)n_int, &s_, &c_);
      sn = (T)s_;
      cn = (T)c_;
    }
    C v;
    v.x = cn;
    v.y = sn;
    tw[i] = v;
  }
  // the column of this path point (QT = 1 tile)
  load_centered_tile<T>(cs, nq, nt, q, 1, q2n, xs, red_re, red_im);
  // window folded into the series once per start frame: x_w(i) = w_i x(t0+i)
  const int n0 = nt - n_int + 1;
  for (int f = tid; f < n_freq; f += NT) {
    Acc<T> acc;
    for (int t0 = 0; t0 < n0; ++t0) {
      T xr = 0, xi = 0;
      int r = 0;
      for (int i = 0; i < n_int; ++i) {
        const C b = xs[t0 + i];
        const T wv = (T)t_wind[i];
        const C a = tw[r];
        xr += wv * (a.x * b.x - a.y * b.y);
        xi += wv * (a.x * b.y + a.y * b.x);
        r += f;
        if (r >= n_int) r -= n_int;
      }
      acc.add(xr * xr + xi * xi);
    }
    out[(int64_t)blockIdx.x * n_freq + f] = (float)(acc.value() * scale);
  }
}

// Gaussian-window spectrum: per Q column, X_k = sum_t g_t (x_t - <x>) e^{-2 pi i k t/nt},
// out[k][q] = |X_k|^2 * scale for k < n_freq.  nt = 2^p <= 1024, radix-2 in shared memory.
template <typename T>
__global__ void gauss_fft_kernel(Series<T> cs, int64_t nq,
                                 int nt, int logn, int QT, const float* __restrict__ gwin,
                                 int n_freq, const float* __restrict__ q2n, double scale,
                                 float* __restrict__ out) {
  using C = typename Cplx<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int NT = blockDim.x, tid = threadIdx.x;
  C* xs = reinterpret_cast<C*>(smem_raw);
  C* tw = xs + (size_t)nt * QT;
  T* red_re = reinterpret_cast<T*>(tw + nt / 2);
  T* red_im = red_re + NT + QT;
  const int64_t q0 = (int64_t)blockIdx.x * QT;
  for (int i = tid; i < nt / 2; i += NT) {
    T sn, cn;
    if (sizeof(T) == 8) {
      double s_, c_;
      sincospi(-2.0 * (double)i / nt, &s_, &c_);
      sn = (T)s_;
      cn = (T)c_;
    } else {
      float s_, c_;
      sincospif(-2.0f * (float)i / (float)nt, &s_, &c_);
      sn = (T)s_;
      cn = (T)c_;
    }
    C v;
    v.x = cn;
    v.y = sn;
    tw[i] = v;
  }
  load_centered_tile<T>(cs, nq, nt, q0, QT, q2n, xs, red_re, red_im);
  // window
  for (int e = tid; e < nt * QT; e += NT) {
    const T g = (T)gwin[e / QT];
    C v = xs[e];
    v.x *= g;
    v.y *= g;
    xs[e] = v;
  }
  __syncthreads();
  // bit reversal
  for (int e = tid; e < nt * QT; e += NT) {
    const int t = e / QT, c = e % QT;
    const int r = (int)(__brev((unsigned)t) >> (32 - logn));
    if (r > t) {
      const C a = xs[t * QT + c];
      xs[t * QT + c] = xs[r * QT + c];
      xs[r * QT + c] = a;
    }
  }
  __syncthreads();
  const int nb = (nt / 2) * QT;
  for (int s = 0; s < logn; ++s) {
    const int half = 1 << s;
    const int stride = nt >> (s + 1);  // twiddle index step
    for (int e = tid; e < nb; e += NT) {
      const int c = e % QT, b = e / QT;
      const int grp = b >> s, pos = b & (half - 1);
      const int i = (grp << (s + 1)) + pos, jj = i + half;
      const C wv = tw[pos * stride];
      const C u = xs[i * QT + c], v0 = xs[jj * QT + c];
      C v;
      v.x = v0.x * wv.x - v0.y * wv.y;
      v.y = v0.x * wv.y + v0.y * wv.x;
      C a, b2;
      a.x = u.x + v.x;
      a.y = u.y + v.y;
      b2.x = u.x - v.x;
      b2.y = u.y - v.y;
      xs[i * QT + c] = a;
      xs[jj * QT + c] = b2;
    }
    __syncthreads();
  }
  for (int e = tid; e < n_freq * QT; e += NT) {
    const int k = e / QT, c = e % QT;
    const int64_t q = q0 + c;
    if (q >= nq) continue;
    const C v = xs[k * QT + c];
    out[(int64_t)k * nq + q] = (float)((double)(v.x * v.x + v.y * v.y) * scale);
  }
}

// I(Q,t) map at lag `lag`: out[q] = Re sum_{i<n_int} x(i+lag) conj(x(i)) / n_int * scale.
template <typename T>
__global__ void iqt_kernel(Series<T> cs, int64_t nq, int nt, int QT, int n_int, int lag,
                           const float* __restrict__ q2n, double scale, float* __restrict__ out) {
  using C = typename Cplx<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int NT = blockDim.x, tid = threadIdx.x;
  C* xs = reinterpret_cast<C*>(smem_raw);
  T* red_re = reinterpret_cast<T*>(xs + (size_t)nt * QT);
  T* red_im = red_re + NT + QT;
  const int64_t q0 = (int64_t)blockIdx.x * QT;
  load_centered_tile<T>(cs, nq, nt, q0, QT, q2n, xs, red_re, red_im);
  const int col = tid % QT, part = tid / QT, nparts = NT / QT;
  Acc<T> acc;
  if (part < nparts)
    for (int i = part; i < n_int; i += nparts) {
      const C a = xs[(i + lag) * QT + col], b = xs[i * QT + col];
      acc.add(a.x * b.x + a.y * b.y);   // Re(a conj b)
    }
  __syncthreads();
  red_re[tid] = (T)acc.value();
  __syncthreads();
  if (tid < QT) {
    double s = 0.0;
    for (int p = 0; p < nparts; ++p) s += (double)red_re[p * QT + tid];
    const int64_t q = q0 + tid;
    if (q < nq) out[q] = (float)(s / n_int * scale);
  }
}

// I(Q,t) along a path: one CTA per path point, out[p * n_lag + t] = Re sum_{i<n_int}
// x(t+i) conj(x(i)) * scale for t < n_lag = nt - n_int + 1.
template <typename T>
__global__ void iqt_dispersion_kernel(Series<T> cs, int64_t nq, int nt,
                                      const int64_t* __restrict__ qidx, int n_int,
                                      const float* __restrict__ q2n, double scale,
                                      float* __restrict__ out) {
  using C = typename Cplx<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int NT = blockDim.x, tid = threadIdx.x;
  C* xs = reinterpret_cast<C*>(smem_raw);
  T* red_re = reinterpret_cast<T*>(xs + nt);
  T* red_im = red_re + NT + 1;
  const int n_lag = nt - n_int + 1;
  const int64_t q = qidx[blockIdx.x];
  if (q < 0 || q >= nq) {
    for (int t = tid; t < n_lag; t += NT) out[(int64_t)blockIdx.x * n_lag + t] = 0.0f;
    return;
  }
  load_centered_tile<T>(cs, nq, nt, q, 1, q2n, xs, red_re, red_im);
  for (int t = tid; t < n_lag; t += NT) {
    Acc<T> acc;
    for (int i = 0; i < n_int; ++i) {
      const C a = xs[t + i], b = xs[i];
      acc.add(a.x * b.x + a.y * b.y);
    }
    out[(int64_t)blockIdx.x * n_lag + t] = (float)(acc.value() * scale);
  }
}

// FP32 Gaussian-window spectrum with an in-place mixed-radix decimation-in-frequency FFT.  One
// CTA holds the N x 8 tile cs(t, q0..q0+7) (64 bytes per time row; 8 columns measured 10 %
// faster than 16 at N = 512); every thread issues all its loads before using them.  The
// elastic mean is subtracted and the window applied in the first stage; the spectrum is read
// back at the digit-reversed positions.
constexpr int kGaussQ = 8;

// First-stage hook: subtract the column's elastic mean and apply the time window.
struct GaussPre {
  const float* gw;
  const float2* mean;
  template <int R>
  __device__ __forceinline__ void operator()(float2 (&v)[R], int base, int M, int line) const {
    const float2 m = mean[line];
#pragma unroll
    for (int k = 0; k < R; ++k) {
      const float g = gw[base + M * k];
      v[k] = make_float2((v[k].x - m.x) * g, (v[k].y - m.y) * g);
    }
  }
};

template <int N>
__global__ void __launch_bounds__(256)
    gauss_dif_kernel(const float2* __restrict__ cs, int64_t nq, const float* __restrict__ gwin,
                     int n_freq, const float* __restrict__ q2n, float scale,
                     float* __restrict__ out) {
  constexpr int QT = kGaussQ, CP = QT / 2, RPP = 256 / CP, RL = N / RPP;
  static_assert(CP <= 32 && 32 % CP == 0 && N % RPP == 0, "Gaussian tile shape");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* xs = reinterpret_cast<float2*>(smem_raw);       // [N][QT]
  float2* tw = xs + N * QT;                                 // exp(-2 pi i n / N)
  float4* part = reinterpret_cast<float4*>(tw + N);         // [8 warps][CP column pairs]
  float2* mean = reinterpret_cast<float2*>(part + 8 * CP);  // [QT]
  float* gw = reinterpret_cast<float*>(mean + QT);          // [N]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t q0 = (int64_t)blockIdx.x * QT;
  dif_twiddles<N>(tw);
  for (int i = tid; i < N; i += blockDim.x) gw[i] = gwin[i];
  // rows t = tid / CP + RPP i, columns q0 + 2 (tid % CP) + {0, 1}
  const int c2 = tid % CP, r0 = tid / CP;
  const int64_t qa = q0 + 2 * c2;
  float4 v[RL];
  if ((nq & 1) == 0) {           // rows start on 16-byte boundaries: one float4 per pair
#pragma unroll
    for (int i = 0; i < RL; ++i) {
      const int64_t t = r0 + RPP * i;
      v[i] = qa < nq ? __ldcs(reinterpret_cast<const float4*>(cs + t * nq + qa))
                     : make_float4(0.f, 0.f, 0.f, 0.f);
    }
  } else {
#pragma unroll
    for (int i = 0; i < RL; ++i) {
      const int64_t t = r0 + RPP * i;
      const float2 a = qa < nq ? __ldcs(cs + t * nq + qa) : make_float2(0.f, 0.f);
      const float2 b = qa + 1 < nq ? __ldcs(cs + t * nq + qa + 1) : make_float2(0.f, 0.f);
      v[i] = make_float4(a.x, a.y, b.x, b.y);
    }
  }
  float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
  for (int i = 0; i < RL; ++i) {
    s.x += v[i].x; s.y += v[i].y; s.z += v[i].z; s.w += v[i].w;
    *reinterpret_cast<float4*>(&xs[(r0 + RPP * i) * QT + 2 * c2]) = v[i];
  }
  // column sums: the lanes c2 + CP k of a warp, then the 8 warps
#pragma unroll
  for (int o = CP; o < 32; o <<= 1) {
    s.x += __shfl_xor_sync(0xffffffffu, s.x, o);
    s.y += __shfl_xor_sync(0xffffffffu, s.y, o);
    s.z += __shfl_xor_sync(0xffffffffu, s.z, o);
    s.w += __shfl_xor_sync(0xffffffffu, s.w, o);
  }
  if (lane < CP) part[warp * CP + lane] = s;
  __syncthreads();
  if (tid < QT) {
    float mr = 0.f, mi = 0.f;
    for (int w = 0; w < 8; ++w) {
      const float4 p = part[w * CP + (tid >> 1)];
      mr += (tid & 1) ? p.z : p.x;
      mi += (tid & 1) ? p.w : p.y;
    }
    mean[tid] = make_float2(mr / (float)N, mi / (float)N);
  }
  __syncthreads();
  dif_lines<N, QT>(xs, tw, GaussPre{gw, mean});
  for (int e = tid; e < n_freq * QT; e += blockDim.x) {
    const int q = e % QT, f = e / QT;
    const int64_t qq = q0 + q;
    if (qq >= nq) continue;
    const float2 X = xs[dif_position<N>(f) * QT + q];
    float val = (X.x * X.x + X.y * X.y) * scale;
    if (q2n) {
      const float w = q2n[qq];
      val *= w * w;
    }
    out[(int64_t)f * nq + qq] = val;
  }
}

template <int N>
static size_t gauss_dif_smem() {
  return (size_t)N * kGaussQ * sizeof(float2) + (size_t)N * sizeof(float2) + 8 * (kGaussQ / 2) * sizeof(float4) +
         kGaussQ * sizeof(float2) + (size_t)N * sizeof(float);
}

template <int N>
static int launch_gauss_dif(const float2* cs, int64_t nq, const float* gwin, int n_freq,
                            const float* q2n, float scale, float* out, cudaStream_t s) {
  const size_t smem = gauss_dif_smem<N>();
  cudaFuncSetAttribute(gauss_dif_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  const unsigned nb = (unsigned)((nq + kGaussQ - 1) / kGaussQ);
  gauss_dif_kernel<N><<<nb, 256, smem, s>>>(cs, nq, gwin, n_freq, q2n, scale, out);
  return MPSQ_OK;
}

// ------------------------------------------------------------------------------- host
static int tile_cols(int nt, size_t csz, size_t extra, size_t limit) {
  int qt = 32;
  while (qt > 1 && (size_t)nt * qt * csz + extra > limit) qt >>= 1;
  if ((size_t)nt * qt * csz + extra > limit) return 0;
  return qt;
}

struct OutBuf {
  float* dev = nullptr;
  bool owned = false;
};

static int out_prepare(float* out, int host, size_t n, OutBuf* b) {
  if (!out) return fail(MPSQ_ERR_ARG, "null output pointer");
  if (host) {
    MPSQ_CUDA_TRY(cudaMalloc(&b->dev, std::max<size_t>(16, n * sizeof(float))));
    b->owned = true;
  } else {
    b->dev = out;
  }
  return MPSQ_OK;
}
static int out_finish(float* out, int host, size_t n, OutBuf* b, cudaStream_t s) {
  if (host) {
    cudaError_t e = cudaMemcpyAsync(out, b->dev, n * sizeof(float), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(b->dev);
    if (e != cudaSuccess) return fail(MPSQ_ERR_CUDA, "output copy: %s", cudaGetErrorString(e));
  }
  return MPSQ_OK;
}

// Small host array -> temporary device copy, stream-ordered (allocated and freed on the
// job's stream, so that a call does not wait for the work queued before it).
template <typename X>
static int dev_copy(const X* h, size_t n, X** d, cudaStream_t s) {
  *d = nullptr;
  if (!h) return MPSQ_OK;
  MPSQ_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(d), std::max<size_t>(16, n * sizeof(X)), s));
  MPSQ_CUDA_TRY(cudaMemcpyAsync(*d, h, n * sizeof(X), cudaMemcpyHostToDevice, s));
  return MPSQ_OK;
}
template <typename X>
static void dev_free(X* d, cudaStream_t s) {
  if (d) cudaFreeAsync(d, s);
}

}  // namespace mpsq

using namespace mpsq;

extern "C" int mpsq_job_sq_total(mpsq_job* j, double norm2, float* out, int host) {
  if (!j) return fail(MPSQ_ERR_ARG, "sq_total: null job");
  PhaseRange range("mpsq:reduce");
  JobView v = job_view(j);
  OutBuf b;
  int rc = out_prepare(out, host, v.n_q, &b);
  if (rc) return rc;
  const double scale = 1.0 / ((double)v.n_frames * (norm2 > 0 ? norm2 : 1.0));
  const unsigned nb = (unsigned)((v.n_q + 255) / 256);
  if (v.precision == MPSQ_FP64)
    sq_total_kernel<double><<<nb, 256, 0, v.s>>>((const double2*)v.cs, v.n_q, v.n_frames, scale, b.dev);
  else
    sq_total_kernel<float><<<nb, 256, 0, v.s>>>((const float2*)v.cs, v.n_q, v.n_frames, scale, b.dev);
  MPSQ_LAUNCH_CHECK();
  return out_finish(out, host, v.n_q, &b, v.s);
}

// q2_norm and t_wind are host arrays (n_Q and n_int floats).
namespace {
// Source of a map: the weighted amplitudes (centred) or the raw sum of two stored species.
struct SeriesArgs {
  const void* a;
  const void* b;
  int64_t stride;
  int center;
};
SeriesArgs weighted_series(const JobView& v) { return {v.cs, nullptr, v.n_q, 1}; }
int pair_series(const JobView& v, int32_t sp1, int32_t sp2, const char* where, SeriesArgs* out) {
  if (!v.store_species || !v.cs_species)
    return fail(MPSQ_ERR_STATE, "%s: the atom-pair modes need a job created with store_species = 1", where);
  if (sp1 < 0 || sp2 < 0 || sp1 >= v.n_species || sp2 >= v.n_species)
    return fail(MPSQ_ERR_ARG, "%s: species %d, %d outside 0..%d", where, sp1, sp2, v.n_species - 1);
  const size_t csz = v.precision == MPSQ_FP64 ? 16 : 8;
  const char* base = (const char*)v.cs_species;
  out->a = base + (size_t)sp1 * v.n_q * csz;
  out->b = base + (size_t)sp2 * v.n_q * csz;
  out->stride = (int64_t)v.n_species * v.n_q;
  out->center = 0;
  return MPSQ_OK;
}
template <typename T>
Series<T> typed(const SeriesArgs& s) {
  using C = typename Cplx<T>::type;
  return Series<T>{(const C*)s.a, (const C*)s.b, s.stride, s.center};
}

int econst_impl(mpsq_job* j, const SeriesArgs& src, int32_t n_int, const float* t_wind,
                int32_t j_freq, const float* q2_norm, double scale, float* out, int host) {
  JobView v = job_view(j);
  if (n_int < 1 || n_int > v.n_frames)
    return fail(MPSQ_ERR_ARG, "sqw_econst: n_int %d outside 1..n_frames (%d)", n_int, v.n_frames);
  if (j_freq < 1) return fail(MPSQ_ERR_ARG, "sqw_econst: j_freq must be >= 1");
  const size_t csz = v.precision == MPSQ_FP64 ? 16 : 8;
  const int NT = 256;
  const size_t extra = (size_t)n_int * csz + (size_t)2 * (NT + 32) * (csz / 2);
  const int QT = tile_cols(v.n_frames, csz, extra, 200 * 1024);
  if (QT == 0) return fail(MPSQ_ERR_ARG, "sqw_econst: %d frames do not fit in shared memory", v.n_frames);
  const size_t smem = (size_t)v.n_frames * QT * csz + (size_t)n_int * csz + (size_t)2 * (NT + QT) * (csz / 2);
  float *dw = nullptr, *dq = nullptr;
  int rc = dev_copy(t_wind, n_int, &dw, v.s);
  if (!rc) rc = dev_copy(q2_norm, q2_norm ? v.n_q : 0, &dq, v.s);
  OutBuf b;
  if (!rc) rc = out_prepare(out, host, v.n_q, &b);
  if (rc) {
    dev_free(dw, v.s);
    dev_free(dq, v.s);
    return rc;
  }
  const unsigned nb = (unsigned)((v.n_q + QT - 1) / QT);
  const int jf = j_freq - 1;
  if (v.precision == MPSQ_FP64) {
    cudaFuncSetAttribute(econst_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    econst_kernel<double><<<nb, NT, smem, v.s>>>(typed<double>(src), v.n_q, v.n_frames, QT, n_int,
                                                 dw, jf, dq, scale, b.dev);
  } else {
    cudaFuncSetAttribute(econst_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    econst_kernel<float><<<nb, NT, smem, v.s>>>(typed<float>(src), v.n_q, v.n_frames, QT, n_int, dw,
                                                jf, dq, scale, b.dev);
  }
  count_launch();
  cudaError_t e = cudaGetLastError();
  rc = e == cudaSuccess ? out_finish(out, host, v.n_q, &b, v.s)
                        : fail(MPSQ_ERR_CUDA, "econst launch: %s", cudaGetErrorString(e));
  dev_free(dw, v.s);
  dev_free(dq, v.s);
  return rc;
}

int dispersion_impl(mpsq_job* j, const SeriesArgs& src, int32_t n_int, const float* t_wind,
                    int32_t n_path, const int64_t* q_index, int32_t n_freq,
                    const float* q2_norm, double scale, float* out, int host) {
  JobView v = job_view(j);
  if (n_int < 1 || n_int > v.n_frames) return fail(MPSQ_ERR_ARG, "sqw_dispersion: bad n_int");
  if (n_path < 1 || n_freq < 1 || n_freq > n_int) return fail(MPSQ_ERR_ARG, "sqw_dispersion: bad sizes");
  const size_t csz = v.precision == MPSQ_FP64 ? 16 : 8;
  const int NT = 128;
  const size_t smem = (size_t)v.n_frames * csz + (size_t)n_int * csz + (size_t)2 * (NT + 2) * (csz / 2);
  if (smem > 200 * 1024) return fail(MPSQ_ERR_ARG, "sqw_dispersion: too many frames");
  float *dw = nullptr, *dq = nullptr;
  int64_t* di = nullptr;
  int rc = dev_copy(t_wind, n_int, &dw, v.s);
  if (!rc) rc = dev_copy(q2_norm, q2_norm ? v.n_q : 0, &dq, v.s);
  if (!rc) rc = dev_copy(q_index, n_path, &di, v.s);
  OutBuf b;
  if (!rc) rc = out_prepare(out, host, (size_t)n_path * n_freq, &b);
  if (rc) {
    dev_free(dw, v.s);
    dev_free(dq, v.s);
    dev_free(di, v.s);
    return rc;
  }
  if (v.precision == MPSQ_FP64) {
    cudaFuncSetAttribute(dispersion_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    dispersion_kernel<double><<<n_path, NT, smem, v.s>>>(typed<double>(src), v.n_q, v.n_frames, di,
                                                         n_int, dw, n_freq, dq, scale, b.dev);
  } else {
    cudaFuncSetAttribute(dispersion_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    dispersion_kernel<float><<<n_path, NT, smem, v.s>>>(typed<float>(src), v.n_q, v.n_frames, di,
                                                        n_int, dw, n_freq, dq, scale, b.dev);
  }
  count_launch();
  cudaError_t e = cudaGetLastError();
  rc = e == cudaSuccess ? out_finish(out, host, (size_t)n_path * n_freq, &b, v.s)
                        : fail(MPSQ_ERR_CUDA, "dispersion launch: %s", cudaGetErrorString(e));
  dev_free(dw, v.s);
  dev_free(dq, v.s);
  dev_free(di, v.s);
  return rc;
}
}  // namespace

extern "C" int mpsq_job_sqw_econst(mpsq_job* j, int32_t n_int, const float* t_wind,
                                   int32_t j_freq, const float* q2_norm, double scale,
                                   float* out, int host) {
  PhaseRange range("mpsq:time");
  if (!j || !t_wind) return fail(MPSQ_ERR_ARG, "sqw_econst: null pointer");
  return econst_impl(j, weighted_series(job_view(j)), n_int, t_wind, j_freq, q2_norm, scale, out,
                     host);
}

extern "C" int mpsq_job_sqw_econst_pair(mpsq_job* j, int32_t n_int, const float* t_wind,
                                        int32_t j_freq, int32_t sp1, int32_t sp2, double scale,
                                        float* out, int host) {
  PhaseRange range("mpsq:time");
  if (!j || !t_wind) return fail(MPSQ_ERR_ARG, "sqw_econst_pair: null pointer");
  SeriesArgs src;
  const int rc = pair_series(job_view(j), sp1, sp2, "sqw_econst_pair", &src);
  if (rc) return rc;
  return econst_impl(j, src, n_int, t_wind, j_freq, nullptr, scale, out, host);
}

extern "C" int mpsq_job_sqw_dispersion(mpsq_job* j, int32_t n_int, const float* t_wind,
                                       int32_t n_path, const int64_t* q_index, int32_t n_freq,
                                       const float* q2_norm, double scale, float* out,
                                       int host) {
  PhaseRange range("mpsq:time");
  if (!j || !t_wind || !q_index) return fail(MPSQ_ERR_ARG, "sqw_dispersion: null pointer");
  return dispersion_impl(j, weighted_series(job_view(j)), n_int, t_wind, n_path, q_index, n_freq,
                         q2_norm, scale, out, host);
}

extern "C" int mpsq_job_sqw_dispersion_pair(mpsq_job* j, int32_t n_int, const float* t_wind,
                                            int32_t n_path, const int64_t* q_index,
                                            int32_t n_freq, int32_t sp1, int32_t sp2,
                                            double scale, float* out, int host) {
  PhaseRange range("mpsq:time");
  if (!j || !t_wind || !q_index) return fail(MPSQ_ERR_ARG, "sqw_dispersion_pair: null pointer");
  SeriesArgs src;
  const int rc = pair_series(job_view(j), sp1, sp2, "sqw_dispersion_pair", &src);
  if (rc) return rc;
  return dispersion_impl(j, src, n_int, t_wind, n_path, q_index, n_freq, nullptr, scale, out,
                         host);
}

extern "C" int mpsq_job_iqt(mpsq_job* j, int32_t n_int, int32_t lag, const float* q2_norm,
                            double scale, float* out, int host) {
  PhaseRange range("mpsq:time");
  if (!j) return fail(MPSQ_ERR_ARG, "iqt: null job");
  JobView v = job_view(j);
  if (n_int < 1 || lag < 0 || lag + n_int > v.n_frames)
    return fail(MPSQ_ERR_ARG, "iqt: lag %d + n_int %d exceeds n_frames %d", lag, n_int, v.n_frames);
  const size_t csz = v.precision == MPSQ_FP64 ? 16 : 8;
  const int NT = 256;
  const size_t extra = (size_t)2 * (NT + 32) * (csz / 2);
  const int QT = tile_cols(v.n_frames, csz, extra, 200 * 1024);
  if (QT == 0) return fail(MPSQ_ERR_ARG, "iqt: %d frames do not fit in shared memory", v.n_frames);
  const size_t smem = (size_t)v.n_frames * QT * csz + (size_t)2 * (NT + QT) * (csz / 2);
  float* dq = nullptr;
  int rc = dev_copy(q2_norm, q2_norm ? v.n_q : 0, &dq, v.s);
  OutBuf b;
  if (!rc) rc = out_prepare(out, host, v.n_q, &b);
  if (rc) {
    dev_free(dq, v.s);
    return rc;
  }
  const unsigned nb = (unsigned)((v.n_q + QT - 1) / QT);
  const SeriesArgs src = weighted_series(v);
  if (v.precision == MPSQ_FP64) {
    cudaFuncSetAttribute(iqt_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    iqt_kernel<double><<<nb, NT, smem, v.s>>>(typed<double>(src), v.n_q, v.n_frames, QT, n_int, lag,
                                              dq, scale, b.dev);
  } else {
    cudaFuncSetAttribute(iqt_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    iqt_kernel<float><<<nb, NT, smem, v.s>>>(typed<float>(src), v.n_q, v.n_frames, QT, n_int, lag,
                                             dq, scale, b.dev);
  }
  count_launch();
  cudaError_t e = cudaGetLastError();
  rc = e == cudaSuccess ? out_finish(out, host, v.n_q, &b, v.s)
                        : fail(MPSQ_ERR_CUDA, "iqt launch: %s", cudaGetErrorString(e));
  dev_free(dq, v.s);
  return rc;
}

extern "C" int mpsq_job_iqt_dispersion(mpsq_job* j, int32_t n_int, int32_t n_path,
                                       const int64_t* q_index, const float* q2_norm,
                                       double scale, float* out, int host) {
  PhaseRange range("mpsq:time");
  if (!j || !q_index) return fail(MPSQ_ERR_ARG, "iqt_dispersion: null pointer");
  JobView v = job_view(j);
  if (n_int < 1 || n_int > v.n_frames || n_path < 1)
    return fail(MPSQ_ERR_ARG, "iqt_dispersion: bad sizes");
  const int n_lag = v.n_frames - n_int + 1;
  const size_t csz = v.precision == MPSQ_FP64 ? 16 : 8;
  const int NT = 128;
  const size_t smem = (size_t)v.n_frames * csz + (size_t)2 * (NT + 2) * (csz / 2);
  if (smem > 200 * 1024) return fail(MPSQ_ERR_ARG, "iqt_dispersion: too many frames");
  float* dq = nullptr;
  int64_t* di = nullptr;
  int rc = dev_copy(q2_norm, q2_norm ? v.n_q : 0, &dq, v.s);
  if (!rc) rc = dev_copy(q_index, n_path, &di, v.s);
  OutBuf b;
  if (!rc) rc = out_prepare(out, host, (size_t)n_path * n_lag, &b);
  if (rc) {
    dev_free(dq, v.s);
    dev_free(di, v.s);
    return rc;
  }
  const SeriesArgs src = weighted_series(v);
  if (v.precision == MPSQ_FP64) {
    cudaFuncSetAttribute(iqt_dispersion_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    iqt_dispersion_kernel<double><<<n_path, NT, smem, v.s>>>(typed<double>(src), v.n_q, v.n_frames,
                                                             di, n_int, dq, scale, b.dev);
  } else {
    cudaFuncSetAttribute(iqt_dispersion_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    iqt_dispersion_kernel<float><<<n_path, NT, smem, v.s>>>(typed<float>(src), v.n_q, v.n_frames,
                                                            di, n_int, dq, scale, b.dev);
  }
  count_launch();
  cudaError_t e = cudaGetLastError();
  rc = e == cudaSuccess ? out_finish(out, host, (size_t)n_path * n_lag, &b, v.s)
                        : fail(MPSQ_ERR_CUDA, "iqt_dispersion launch: %s", cudaGetErrorString(e));
  dev_free(dq, v.s);
  dev_free(di, v.s);
  return rc;
}

extern "C" int mpsq_job_sqw_gauss(mpsq_job* j, double fwhm_frames, int32_t n_freq,
                                  const float* q2_norm, double scale, float* out, int host) {
  PhaseRange range("mpsq:time");
  if (!j) return fail(MPSQ_ERR_ARG, "sqw_gauss: null job");
  JobView v = job_view(j);
  const int nt = v.n_frames;
  if (nt < 2 || nt > 1024 || (nt & (nt - 1)))
    return fail(MPSQ_ERR_ARG, "sqw_gauss: n_frames (%d) must be a power of two in 2..1024", nt);
  if (n_freq < 1 || n_freq > nt) return fail(MPSQ_ERR_ARG, "sqw_gauss: n_freq outside 1..n_frames");
  if (!(fwhm_frames > 0)) return fail(MPSQ_ERR_ARG, "sqw_gauss: fwhm must be > 0");
  int logn = 0;
  while ((1 << logn) < nt) ++logn;
  const size_t csz = v.precision == MPSQ_FP64 ? 16 : 8;
  const int NT = 256;
  const size_t extra = (size_t)(nt / 2) * csz + (size_t)2 * (NT + 32) * (csz / 2);
  const int QT = tile_cols(nt, csz, extra, 160 * 1024);
  if (QT == 0) return fail(MPSQ_ERR_ARG, "sqw_gauss: tile does not fit");
  const size_t smem = (size_t)nt * QT * csz + (size_t)(nt / 2) * csz + (size_t)2 * (NT + QT) * (csz / 2);
  std::vector<float> g(nt);
  const double tc = 0.5 * (nt - 1);
  for (int t = 0; t < nt; ++t) {
    const double u = (t - tc) / fwhm_frames;
    g[t] = (float)std::exp(-4.0 * std::log(2.0) * u * u);
  }
  float *dg = nullptr, *dq = nullptr;
  int rc = dev_copy(g.data(), nt, &dg, v.s);
  if (!rc) rc = dev_copy(q2_norm, q2_norm ? v.n_q : 0, &dq, v.s);
  OutBuf b;
  if (!rc) rc = out_prepare(out, host, (size_t)n_freq * v.n_q, &b);
  if (rc) {
    dev_free(dg, v.s);
    dev_free(dq, v.s);
    return rc;
  }
  const unsigned nb = (unsigned)((v.n_q + QT - 1) / QT);
  if (v.precision == MPSQ_FP64) {
    cudaFuncSetAttribute(gauss_fft_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    gauss_fft_kernel<double><<<nb, NT, smem, v.s>>>(typed<double>(weighted_series(v)), v.n_q, nt, logn, QT, dg,
                                                    n_freq, dq, scale, b.dev);
  } else if (nt >= 64) {
    const float2* cs = (const float2*)v.cs;
    const float sc = (float)scale;
    switch (nt) {
      case 64: launch_gauss_dif<64>(cs, v.n_q, dg, n_freq, dq, sc, b.dev, v.s); break;
      case 128: launch_gauss_dif<128>(cs, v.n_q, dg, n_freq, dq, sc, b.dev, v.s); break;
      case 256: launch_gauss_dif<256>(cs, v.n_q, dg, n_freq, dq, sc, b.dev, v.s); break;
      case 512: launch_gauss_dif<512>(cs, v.n_q, dg, n_freq, dq, sc, b.dev, v.s); break;
      default: launch_gauss_dif<1024>(cs, v.n_q, dg, n_freq, dq, sc, b.dev, v.s); break;
    }
  } else {
    cudaFuncSetAttribute(gauss_fft_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    gauss_fft_kernel<float><<<nb, NT, smem, v.s>>>(typed<float>(weighted_series(v)), v.n_q, nt, logn, QT, dg,
                                                   n_freq, dq, scale, b.dev);
  }
  count_launch();
  cudaError_t e = cudaGetLastError();
  rc = e == cudaSuccess ? out_finish(out, host, (size_t)n_freq * v.n_q, &b, v.s)
                        : fail(MPSQ_ERR_CUDA, "gauss launch: %s", cudaGetErrorString(e));
  dev_free(dg, v.s);
  dev_free(dq, v.s);
  return rc;
}

// ------------------------------------------------------------- spherical |Q| histogram
namespace mpsq {
// Fortran NORM2 of a 3-vector as the scaled sum of squares (the recurrence of BLAS snrm2):
// scale tracks the largest |component|, ssq the sum of squares relative to it.  Every
// operation is a separately rounded FP32 op (no contraction into fused multiply-adds).
__device__ __forceinline__ float norm2_scaled(float x, float y, float z) {
  float scale = 0.0f, ssq = 1.0f;
  const float c[3] = {x, y, z};
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float a = fabsf(c[i]);
    if (a != 0.0f) {
      if (scale < a) {
        const float r = __fdiv_rn(scale, a);
        ssq = __fadd_rn(1.0f, __fmul_rn(ssq, __fmul_rn(r, r)));
        scale = a;
      } else {
        const float r = __fdiv_rn(a, scale);
        ssq = __fadd_rn(ssq, __fmul_rn(r, r));
      }
    }
  }
  return __fmul_rn(scale, __fsqrt_rn(ssq));
}

__device__ __forceinline__ float dot3_rn(float3 a, float v0, float v1, float v2) {
  return __fadd_rn(__fadd_rn(__fmul_rn(a.x, v0), __fmul_rn(a.y, v1)), __fmul_rn(a.z, v2));
}

// Grid-stride over modes; a CTA accumulates its bins in shared memory (FP32 partial sums of a
// few thousand products) and flushes them to the FP64 output with atomics.
template <typename T>
__global__ void radial_hist_kernel(const typename Cplx<T>::type* __restrict__ amps, int s_stride,
                                   int S, int64_t nq, int nt, int m0, int m1, int m2, float3 r0,
                                   float3 r1, float3 r2, float3 dq, float q_step, float q_range,
                                   int n_hist, float scale2, int use_smem,
                                   double* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* h = reinterpret_cast<float*>(smem_raw);
  const int nb = S * S * n_hist;
  if (use_smem) {
    for (int e = threadIdx.x; e < nb; e += blockDim.x) h[e] = 0.0f;
    __syncthreads();
  }
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nq;
       q += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(q % m0), j = (int)((q / m0) % m1), l = (int)(q / ((int64_t)m0 * m1));
    // v = k * d_q, Q = a_cell_inv v, |Q| = NORM2(Q), all in FP32 (mp_sql56.f90:1041)
    const float v0 = __fmul_rn((float)(i - m0 / 2), dq.x);
    const float v1 = __fmul_rn((float)(j - m1 / 2), dq.y);
    const float v2 = __fmul_rn((float)(l - m2 / 2), dq.z);
    const float qn = norm2_scaled(dot3_rn(r0, v0, v1, v2), dot3_rn(r1, v0, v1, v2),
                                  dot3_rn(r2, v0, v1, v2));
    if (!(qn <= q_range)) continue;
    const int bin = (int)roundf(__fdiv_rn(qn, q_step));   // NINT: half away from zero
    if (bin < 0 || bin >= n_hist) continue;
    for (int t = 0; t < nt; ++t) {
      for (int a = 0; a < S; ++a) {
        const auto A = amps[((int64_t)t * s_stride + a) * nq + q];
        for (int b = 0; b < S; ++b) {
          const auto B = amps[((int64_t)t * s_stride + b) * nq + q];
          const float v = (float)(A.x * B.x + A.y * B.y) * scale2;
          const int e = (a * S + b) * n_hist + bin;
          if (use_smem)
            atomicAdd(&h[e], v);
          else
            atomicAdd(&out[e], (double)v);
        }
      }
    }
  }
  if (use_smem) {
    __syncthreads();
    for (int e = threadIdx.x; e < nb; e += blockDim.x)
      if (h[e] != 0.0f) atomicAdd(&out[e], (double)h[e]);
  }
}
}  // namespace mpsq

extern "C" int mpsq_job_radial_hist(mpsq_job* j, const double* a_cell_inv, const double* d_q,
                                    double q_step, double q_range, int32_t n_hist,
                                    double amp_scale, double* out, int host) {
  if (!j || !a_cell_inv || !d_q || !out) return fail(MPSQ_ERR_ARG, "radial_hist: null pointer");
  JobView v = job_view(j);
  if (v.slab) return fail(MPSQ_ERR_STATE, "radial_hist: needs the whole Q store (job has a q_slab)");
  if (n_hist < 1 || !(q_step > 0)) return fail(MPSQ_ERR_ARG, "radial_hist: bad bins");
  const void* amps = v.cs;
  int S = 1, s_stride = 1;
  if (v.store_species) {
    amps = v.cs_species;
    S = v.n_species;
    s_stride = v.n_species;
  } else if (v.n_species != 1) {
    return fail(MPSQ_ERR_STATE, "radial_hist: per-species amplitudes need store_species = 1");
  }
  const size_t nb = (size_t)S * S * n_hist;
  double* dev = nullptr;
  MPSQ_CUDA_TRY(cudaMalloc(&dev, nb * sizeof(double)));
  MPSQ_CUDA_TRY(cudaMemsetAsync(dev, 0, nb * sizeof(double), v.s));
  const size_t smem = nb * sizeof(float);
  const int use_smem = smem <= 96 * 1024 ? 1 : 0;
  const double* A = a_cell_inv;
  const float3 r0 = make_float3((float)A[0], (float)A[1], (float)A[2]);
  const float3 r1 = make_float3((float)A[3], (float)A[4], (float)A[5]);
  const float3 r2 = make_float3((float)A[6], (float)A[7], (float)A[8]);
  const float3 dq = make_float3((float)d_q[0], (float)d_q[1], (float)d_q[2]);
  const float scale2 = (float)(amp_scale * amp_scale);
  const unsigned blocks = (unsigned)std::min<int64_t>((v.n_q + 255) / 256, 152 * 8);
  if (v.precision == MPSQ_FP64) {
    cudaFuncSetAttribute(radial_hist_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024);
    radial_hist_kernel<double><<<blocks, 256, use_smem ? smem : 0, v.s>>>(
        (const double2*)amps, s_stride, S, v.n_q, v.n_frames, (int)v.m[0], (int)v.m[1], (int)v.m[2],
        r0, r1, r2, dq, (float)q_step, (float)q_range, n_hist, scale2, use_smem, dev);
  } else {
    cudaFuncSetAttribute(radial_hist_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024);
    radial_hist_kernel<float><<<blocks, 256, use_smem ? smem : 0, v.s>>>(
        (const float2*)amps, s_stride, S, v.n_q, v.n_frames, (int)v.m[0], (int)v.m[1], (int)v.m[2],
        r0, r1, r2, dq, (float)q_step, (float)q_range, n_hist, scale2, use_smem, dev);
  }
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) {
    if (host) {
      e = cudaMemcpyAsync(out, dev, nb * sizeof(double), cudaMemcpyDeviceToHost, v.s);
    } else {
      e = cudaMemcpyAsync(out, dev, nb * sizeof(double), cudaMemcpyDeviceToDevice, v.s);
    }
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(v.s);
  cudaFree(dev);
  if (e != cudaSuccess) return fail(MPSQ_ERR_CUDA, "radial_hist: %s", cudaGetErrorString(e));
  return MPSQ_OK;
}
