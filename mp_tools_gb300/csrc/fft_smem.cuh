// Shared-memory FFT building blocks for the pruned fine-grid transform: a self-sorting
// (Stockham) forward DFT of `nl` lines of length n = 2^a 3^b 5^c held in shared memory, with
// radix-4/2/3/5 stages and a precomputed twiddle table tw[k] = exp(-2 pi i k / n).
//
// Stage recurrence (DIT, L = product of the radices already applied, Ls = L r, m = n/Ls):
//   out[k*Ls + j + q*L] = sum_p w_r^{qp} ( w_Ls^{jp} in[(k + m p)*L + j] ),
//   j in [0, L), k in [0, m), q in [0, r); after the last stage out[f] = DFT[f].
#pragma once

#include <cuda_runtime.h>

namespace mpsq {

constexpr int kMaxFftStages = 24;

struct SmemFftPlan {
  int n = 0;
  int nst = 0;
  int radix[kMaxFftStages] = {};
};

// Radices in application order; false if n has a prime factor other than 2, 3, 5.
inline bool make_smem_fft_plan(int n, SmemFftPlan* p) {
  SmemFftPlan q;
  q.n = n;
  int r = n;
  while (r % 4 == 0 && q.nst < kMaxFftStages) {
    q.radix[q.nst++] = 4;
    r /= 4;
  }
  while (r % 2 == 0 && q.nst < kMaxFftStages) {
    q.radix[q.nst++] = 2;
    r /= 2;
  }
  while (r % 3 == 0 && q.nst < kMaxFftStages) {
    q.radix[q.nst++] = 3;
    r /= 3;
  }
  while (r % 5 == 0 && q.nst < kMaxFftStages) {
    q.radix[q.nst++] = 5;
    r /= 5;
  }
  if (r != 1) return false;
  *p = q;
  return true;
}

__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// In-place forward radix-r butterfly on v[0..r).
__device__ __forceinline__ void butterfly(float2* v, int r) {
  if (r == 4) {
    const float2 a = make_float2(v[0].x + v[2].x, v[0].y + v[2].y);
    const float2 b = make_float2(v[0].x - v[2].x, v[0].y - v[2].y);
    const float2 c = make_float2(v[1].x + v[3].x, v[1].y + v[3].y);
    const float2 d = make_float2(v[1].x - v[3].x, v[1].y - v[3].y);
    v[0] = make_float2(a.x + c.x, a.y + c.y);
    v[2] = make_float2(a.x - c.x, a.y - c.y);
    v[1] = make_float2(b.x + d.y, b.y - d.x);  // b - i d
    v[3] = make_float2(b.x - d.y, b.y + d.x);  // b + i d
  } else if (r == 2) {
    const float2 a = v[0], b = v[1];
    v[0] = make_float2(a.x + b.x, a.y + b.y);
    v[1] = make_float2(a.x - b.x, a.y - b.y);
  } else if (r == 3) {
    // w = exp(-2 pi i/3) = c + i s, c = -1/2, s = -sqrt(3)/2
    const float s = -0.86602540378443864676f;
    const float2 t1 = make_float2(v[1].x + v[2].x, v[1].y + v[2].y);
    const float2 t2 = make_float2(v[1].x - v[2].x, v[1].y - v[2].y);
    const float2 m = make_float2(v[0].x - 0.5f * t1.x, v[0].y - 0.5f * t1.y);
    const float2 ist = make_float2(-s * t2.y, s * t2.x);  // i s t2
    v[0] = make_float2(v[0].x + t1.x, v[0].y + t1.y);
    v[1] = make_float2(m.x + ist.x, m.y + ist.y);
    v[2] = make_float2(m.x - ist.x, m.y - ist.y);
  } else {  // r == 5: direct sum with w5^k = exp(-2 pi i k/5)
    const float c1 = 0.30901699437494742410f, s1 = -0.95105651629515357212f;
    const float c2 = -0.80901699437494742410f, s2 = -0.58778525229247312917f;
    const float2 w[5] = {make_float2(1.f, 0.f), make_float2(c1, s1), make_float2(c2, s2),
                         make_float2(c2, -s2), make_float2(c1, -s1)};
    float2 u[5];
#pragma unroll
    for (int q = 0; q < 5; ++q) {
      float2 acc = v[0];
#pragma unroll
      for (int p = 1; p < 5; ++p) {
        const float2 t = cmulf(w[(q * p) % 5], v[p]);
        acc.x += t.x;
        acc.y += t.y;
      }
      u[q] = acc;
    }
#pragma unroll
    for (int q = 0; q < 5; ++q) v[q] = u[q];
  }
}

// Compile-time Stockham stages: transform length N and line count NL are template
// parameters so every index computation reduces to shifts and multiply-adds.  Element
// (line, i) lives at buf[line*LS + i*ES].  LINE_FAST maps consecutive threads to consecutive
// lines (lines adjacent in memory), otherwise to consecutive butterflies of one line.
template <int N>
constexpr int next_radix(int rem) {
  return rem % 4 == 0 ? 4 : (rem % 2 == 0 ? 2 : (rem % 3 == 0 ? 3 : 5));
}

template <int N, int L, int NL, int LS, int ES, bool LINE_FAST>
struct StockhamStages {
  static __device__ __forceinline__ float2* run(float2* in, float2* out,
                                                const float2* __restrict__ tw) {
    if constexpr (L >= N) {
      return in;
    } else {
      constexpr int r = next_radix<N>(N / L);
      constexpr int Ls = L * r, m = N / Ls, nb = N / r;
      for (int e = threadIdx.x; e < nb * NL; e += blockDim.x) {
        const int line = LINE_FAST ? e % NL : e / nb;
        const int b = LINE_FAST ? e / NL : e % nb;
        const int j = b % L, k = b / L;
        float2 v[5];
        const float2* src = in + line * LS;
#pragma unroll
        for (int q = 0; q < r; ++q) {
          const float2 a = src[((k + m * q) * L + j) * ES];
          v[q] = q == 0 ? a : cmulf(a, tw[j * q * m]);  // j q m < L r m = N
        }
        butterfly(v, r);
        float2* dst = out + line * LS;
#pragma unroll
        for (int q = 0; q < r; ++q) dst[(k * Ls + j + q * L) * ES] = v[q];
      }
      __syncthreads();
      return StockhamStages<N, Ls, NL, LS, ES, LINE_FAST>::run(out, in, tw);
    }
  }
};

// Forward DFT of NL lines of length N (all threads of the block call it; it synchronises
// internally).  Returns the buffer holding the result.
template <int N, int NL, int LS, int ES, bool LINE_FAST>
__device__ __forceinline__ float2* smem_fft(float2* b0, float2* b1, const float2* __restrict__ tw) {
  return StockhamStages<N, 1, NL, LS, ES, LINE_FAST>::run(b0, b1, tw);
}

// Lengths with compiled transform passes (2,3,5-smooth multiples of 16).
#define MPSQ_FFT_SIZES(X) X(64) X(96) X(128) X(160) X(192) X(256) X(320) X(384) X(480) X(512) \
  X(640) X(768) X(1024) X(1152)

inline bool fft_size_compiled(int n) {
  switch (n) {
#define MPSQ_CASE(N) case N:
    MPSQ_FFT_SIZES(MPSQ_CASE)
#undef MPSQ_CASE
    return true;
    default:
      return false;
  }
}

}  // namespace mpsq
