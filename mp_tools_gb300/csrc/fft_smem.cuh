// Shared-memory FFT building blocks for the pruned fine-grid transform and the time-axis
// spectrum: forward DFTs of lines of length n = 2^a 3^b 5^c held in shared memory, computed in
// place by mixed-radix decimation in frequency (radix 24, 16, 12, 8, 6, 4, 2, 3, 5) with a
// twiddle table tw[k] = exp(-2 pi i k / n); outputs are read at digit-reversed positions.
#pragma once

#include <cuda_runtime.h>

namespace mpsq {

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

// Forward 8-point DFT in place: v[k'] = sum_k v[k] exp(-2 pi i k k'/8), as two 4-point DFTs
// of the even and odd samples combined with w8^k' = exp(-i pi k'/4).
__device__ __forceinline__ void dft8(float2* v) {
  const float r = 0.70710678118654752440f;
  float2 e[4], o[4];
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const float2 a0 = v[h], a1 = v[h + 2], a2 = v[h + 4], a3 = v[h + 6];
    const float2 b0 = make_float2(a0.x + a2.x, a0.y + a2.y);
    const float2 b1 = make_float2(a0.x - a2.x, a0.y - a2.y);
    const float2 b2 = make_float2(a1.x + a3.x, a1.y + a3.y);
    const float2 b3 = make_float2(a1.x - a3.x, a1.y - a3.y);
    float2* d = h ? o : e;
    d[0] = make_float2(b0.x + b2.x, b0.y + b2.y);
    d[2] = make_float2(b0.x - b2.x, b0.y - b2.y);
    d[1] = make_float2(b1.x + b3.y, b1.y - b3.x);   // b1 - i b3
    d[3] = make_float2(b1.x - b3.y, b1.y + b3.x);   // b1 + i b3
  }
  const float2 t1 = make_float2((o[1].x + o[1].y) * r, (o[1].y - o[1].x) * r);    // w8 o1
  const float2 t2 = make_float2(o[2].y, -o[2].x);                                 // -i o2
  const float2 t3 = make_float2((o[3].y - o[3].x) * r, -(o[3].x + o[3].y) * r);   // w8^3 o3
  v[0] = make_float2(e[0].x + o[0].x, e[0].y + o[0].y);
  v[4] = make_float2(e[0].x - o[0].x, e[0].y - o[0].y);
  v[1] = make_float2(e[1].x + t1.x, e[1].y + t1.y);
  v[5] = make_float2(e[1].x - t1.x, e[1].y - t1.y);
  v[2] = make_float2(e[2].x + t2.x, e[2].y + t2.y);
  v[6] = make_float2(e[2].x - t2.x, e[2].y - t2.y);
  v[3] = make_float2(e[3].x + t3.x, e[3].y + t3.y);
  v[7] = make_float2(e[3].x - t3.x, e[3].y - t3.y);
}

// Forward 6-point DFT in place: two 3-point DFTs of the even and odd samples combined with
// w6^k' = exp(-i pi k'/3).
__device__ __forceinline__ void dft6(float2* v) {
  float2 e[3] = {v[0], v[2], v[4]}, o[3] = {v[1], v[3], v[5]};
  butterfly(e, 3);
  butterfly(o, 3);
  const float h = 0.5f, s = 0.86602540378443864676f;
  const float2 t1 = make_float2(h * o[1].x + s * o[1].y, h * o[1].y - s * o[1].x);    // w6 o1
  const float2 t2 = make_float2(-h * o[2].x + s * o[2].y, -h * o[2].y - s * o[2].x);  // w6^2 o2
  v[0] = make_float2(e[0].x + o[0].x, e[0].y + o[0].y);
  v[3] = make_float2(e[0].x - o[0].x, e[0].y - o[0].y);
  v[1] = make_float2(e[1].x + t1.x, e[1].y + t1.y);
  v[4] = make_float2(e[1].x - t1.x, e[1].y - t1.y);
  v[2] = make_float2(e[2].x + t2.x, e[2].y + t2.y);
  v[5] = make_float2(e[2].x - t2.x, e[2].y - t2.y);
}

// Forward 16-point DFT in place, 4 x 4 Cooley-Tukey: for n = 4 n1 + n2 and k = k1 + 4 k2,
// X[k] = sum_n2 W4^(n2 k2) [W16^(n2 k1) sum_n1 x[4 n1 + n2] W4^(n1 k1)].
__device__ __forceinline__ float2 cmulc(float2 a, float c, float s) {  // a (c + i s)
  return make_float2(a.x * c - a.y * s, a.x * s + a.y * c);
}
__device__ __forceinline__ void dft16(float2* v) {
  const float c1 = 0.92387953251128675613f, s1 = 0.38268343236508977173f;  // cos, sin pi/8
  const float r = 0.70710678118654752440f;
  float2 y[4][4];
#pragma unroll
  for (int n2 = 0; n2 < 4; ++n2) {
    float2 a[4] = {v[n2], v[4 + n2], v[8 + n2], v[12 + n2]};
    butterfly(a, 4);
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) y[n2][k1] = a[k1];
  }
  // W16^m = exp(-2 pi i m/16) for m = n2 k1: 1, 2, 3 | 2, 4, 6 | 3, 6, 9
  y[1][1] = cmulc(y[1][1], c1, -s1);
  y[1][2] = cmulc(y[1][2], r, -r);
  y[1][3] = cmulc(y[1][3], s1, -c1);
  y[2][1] = cmulc(y[2][1], r, -r);
  y[2][2] = make_float2(y[2][2].y, -y[2][2].x);  // -i
  y[2][3] = cmulc(y[2][3], -r, -r);
  y[3][1] = cmulc(y[3][1], s1, -c1);
  y[3][2] = cmulc(y[3][2], -r, -r);
  y[3][3] = cmulc(y[3][3], -c1, s1);
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) {
    float2 b[4] = {y[0][k1], y[1][k1], y[2][k1], y[3][k1]};
    butterfly(b, 4);
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) v[k1 + 4 * k2] = b[k2];
  }
}

// Forward 12-point DFT in place, 4 x 3: n = 3 n1 + n2, k = k1 + 4 k2,
// X[k] = sum_n2 W3^(n2 k2) [W12^(n2 k1) sum_n1 x[3 n1 + n2] W4^(n1 k1)].
__device__ __forceinline__ void dft12(float2* v) {
  const float h = 0.5f, s3 = 0.86602540378443864676f;
  float2 y[3][4];
#pragma unroll
  for (int n2 = 0; n2 < 3; ++n2) {
    float2 a[4] = {v[n2], v[3 + n2], v[6 + n2], v[9 + n2]};
    butterfly(a, 4);
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) y[n2][k1] = a[k1];
  }
  // W12^m for m = n2 k1: 1, 2, 3 | 2, 4, 6
  y[1][1] = cmulc(y[1][1], s3, -h);
  y[1][2] = cmulc(y[1][2], h, -s3);
  y[1][3] = make_float2(y[1][3].y, -y[1][3].x);  // -i
  y[2][1] = cmulc(y[2][1], h, -s3);
  y[2][2] = cmulc(y[2][2], -h, -s3);
  y[2][3] = make_float2(-y[2][3].x, -y[2][3].y);  // -1
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) {
    float2 b[3] = {y[0][k1], y[1][k1], y[2][k1]};
    butterfly(b, 3);
#pragma unroll
    for (int k2 = 0; k2 < 3; ++k2) v[k1 + 4 * k2] = b[k2];
  }
}

// Forward 24-point DFT in place, 8 x 3: n = 3 n1 + n2, k = k1 + 8 k2,
// X[k] = sum_n2 W3^(n2 k2) [W24^(n2 k1) sum_n1 x[3 n1 + n2] W8^(n1 k1)].
__device__ __forceinline__ void dft24(float2* v) {
  // cos and sin of 2 pi m / 24, m = 0..14
  const float cs[15][2] = {
      {1.0f, 0.0f},
      {0.96592582628906828675f, 0.25881904510252076235f},
      {0.86602540378443864676f, 0.5f},
      {0.70710678118654752440f, 0.70710678118654752440f},
      {0.5f, 0.86602540378443864676f},
      {0.25881904510252076235f, 0.96592582628906828675f},
      {0.0f, 1.0f},
      {-0.25881904510252076235f, 0.96592582628906828675f},
      {-0.5f, 0.86602540378443864676f},
      {-0.70710678118654752440f, 0.70710678118654752440f},
      {-0.86602540378443864676f, 0.5f},
      {-0.96592582628906828675f, 0.25881904510252076235f},
      {-1.0f, 0.0f},
      {-0.96592582628906828675f, -0.25881904510252076235f},
      {-0.86602540378443864676f, -0.5f}};
  float2 y[3][8];
#pragma unroll
  for (int n2 = 0; n2 < 3; ++n2) {
    float2 a[8];
#pragma unroll
    for (int n1 = 0; n1 < 8; ++n1) a[n1] = v[3 * n1 + n2];
    dft8(a);
#pragma unroll
    for (int k1 = 0; k1 < 8; ++k1) y[n2][k1] = a[k1];
  }
#pragma unroll
  for (int n2 = 1; n2 < 3; ++n2)
#pragma unroll
    for (int k1 = 1; k1 < 8; ++k1) {
      const int m = n2 * k1;                              // W24^m = cos - i sin
      y[n2][k1] = cmulc(y[n2][k1], cs[m][0], -cs[m][1]);
    }
#pragma unroll
  for (int k1 = 0; k1 < 8; ++k1) {
    float2 b[3] = {y[0][k1], y[1][k1], y[2][k1]};
    butterfly(b, 3);
#pragma unroll
    for (int k2 = 0; k2 < 3; ++k2) v[k1 + 8 * k2] = b[k2];
  }
}

// Forward 32-point DFT in place, 8 x 4: n = 4 n1 + n2, k = k1 + 8 k2,
// X[k] = sum_n2 W4^(n2 k2) [W32^(n2 k1) sum_n1 x[4 n1 + n2] W8^(n1 k1)].
__device__ __forceinline__ void dft32(float2* v) {
  // cos and sin of 2 pi m / 32, m = 0..21 (the products n2 k1 that occur)
  const float cs[22][2] = {
      {1.0f, 0.0f},
      {0.98078528040323044913f, 0.19509032201612826785f},
      {0.92387953251128675613f, 0.38268343236508977173f},
      {0.83146961230254523708f, 0.55557023301960222474f},
      {0.70710678118654752440f, 0.70710678118654752440f},
      {0.55557023301960222474f, 0.83146961230254523708f},
      {0.38268343236508977173f, 0.92387953251128675613f},
      {0.19509032201612826785f, 0.98078528040323044913f},
      {0.0f, 1.0f},
      {-0.19509032201612826785f, 0.98078528040323044913f},
      {-0.38268343236508977173f, 0.92387953251128675613f},
      {-0.55557023301960222474f, 0.83146961230254523708f},
      {-0.70710678118654752440f, 0.70710678118654752440f},
      {-0.83146961230254523708f, 0.55557023301960222474f},
      {-0.92387953251128675613f, 0.38268343236508977173f},
      {-0.98078528040323044913f, 0.19509032201612826785f},
      {-1.0f, 0.0f},
      {-0.98078528040323044913f, -0.19509032201612826785f},
      {-0.92387953251128675613f, -0.38268343236508977173f},
      {-0.83146961230254523708f, -0.55557023301960222474f},
      {-0.70710678118654752440f, -0.70710678118654752440f},
      {-0.55557023301960222474f, -0.83146961230254523708f}};
  float2 y[4][8];
#pragma unroll
  for (int n2 = 0; n2 < 4; ++n2) {
    float2 a[8];
#pragma unroll
    for (int n1 = 0; n1 < 8; ++n1) a[n1] = v[4 * n1 + n2];
    dft8(a);
#pragma unroll
    for (int k1 = 0; k1 < 8; ++k1) y[n2][k1] = a[k1];
  }
#pragma unroll
  for (int n2 = 1; n2 < 4; ++n2)
#pragma unroll
    for (int k1 = 1; k1 < 8; ++k1) {
      const int m = n2 * k1;                              // W32^m = cos - i sin
      y[n2][k1] = cmulc(y[n2][k1], cs[m][0], -cs[m][1]);
    }
#pragma unroll
  for (int k1 = 0; k1 < 8; ++k1) {
    float2 b[4] = {y[0][k1], y[1][k1], y[2][k1], y[3][k1]};
    butterfly(b, 4);
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) v[k1 + 8 * k2] = b[k2];
  }
}

// Radices of an in-place decimation-in-frequency transform of length N = 2^a 3^b 5^c, in
// application order.  Two stages when N = r0 r1 with r0 in {16, 24, 12, 8, 32} and r1 in
// {32, 24, 16, 12, 8, 6} (fewer passes through shared memory); otherwise 8 while 8 divides
// what remains, then 6, 4, 2, 3 or 5.
__host__ __device__ constexpr bool dif_final(int r) {
  return r == 32 || r == 24 || r == 16 || r == 12 || r == 8 || r == 6;
}
__host__ __device__ constexpr int dif_first(int N) {
  return (N % 16 == 0 && dif_final(N / 16)) ? 16
         : (N % 24 == 0 && dif_final(N / 24)) ? 24
         : (N % 12 == 0 && dif_final(N / 12)) ? 12
         : (N % 8 == 0 && dif_final(N / 8)) ? 8
         : (N % 32 == 0 && dif_final(N / 32)) ? 32
                                              : 0;
}
__host__ __device__ constexpr int dif_greedy(int rem) {
  return rem % 8 == 0 ? 8 : rem % 6 == 0 ? 6 : rem % 4 == 0 ? 4 : rem % 2 == 0 ? 2 : rem % 3 == 0 ? 3 : 5;
}
// P selects the plan: kDifTwoStage (the two-stage split where one exists) or kDifGreedy
// (radix 8 first: smaller register footprint for kernels that hold more state).
constexpr int kDifGreedy = 0, kDifTwoStage = 1;
__host__ __device__ constexpr int dif_radix(int N, int s, int P = kDifTwoStage) {
  if (P == kDifTwoStage && dif_first(N)) return s == 0 ? dif_first(N) : N / dif_first(N);
  int rem = N;
  for (int i = 0; i < s; ++i) rem /= dif_greedy(rem);
  return dif_greedy(rem);
}
__host__ __device__ constexpr int dif_stages(int N, int P = kDifTwoStage) {
  if (P == kDifTwoStage && dif_first(N)) return 2;
  int s = 0;
  for (int rem = N; rem > 1; rem /= dif_greedy(rem)) ++s;
  return s;
}
__host__ __device__ constexpr int dif_block(int N, int s, int P = kDifTwoStage) {
  int b = N;
  for (int i = 0; i < s; ++i) b /= dif_radix(N, i, P);
  return b;
}
__device__ __forceinline__ void dft_r(float2* v, int r) {
  if (r == 32) dft32(v);
  else if (r == 24) dft24(v);
  else if (r == 16) dft16(v);
  else if (r == 12) dft12(v);
  else if (r == 8) dft8(v);
  else if (r == 6) dft6(v);
  else butterfly(v, r);
}

// Position of frequency f in the output of the in-place DIF transform (mixed-radix digit
// reversal: stage s leaves digit k'_s of f = k'_0 + r_0 (k'_1 + r_1 (...)) at stride M_s).
template <int N, int P = kDifTwoStage>
__device__ __forceinline__ int dif_position(int f) {
  int p = 0, block = N;
#pragma unroll
  for (int s = 0; s < dif_stages(N, P); ++s) {
    const int r = dif_radix(N, s, P);
    block /= r;
    p += (f % r) * block;
    f /= r;
  }
  return p;
}

// In-place forward DFT of L lines of length N held in shared memory as xs[i * L + line]
// (lines fastest, so a warp touches whole 128-byte rows at every stage), by mixed-radix
// decimation in frequency: stage s transforms groups {base + M k} with a radix-r DFT and
// multiplies output k' by exp(-2 pi i j k' / B) (B = M r the stage's block, j = base mod M).
// The result for frequency f sits at position dif_position<N>(f).  `pre` may rewrite the
// first stage's inputs (pre(v, base, M, line) with v[k] = x[base + M k]).  All threads of the
// block call it; it ends with __syncthreads().
struct DifNoPre {
  template <int R>
  __device__ __forceinline__ void operator()(float2 (&)[R], int, int, int) const {}
};

template <int N, int L, int S, int P, int SE, class Pre>
__device__ __forceinline__ void dif_lines_from(float2* __restrict__ xs,
                                               const float2* __restrict__ tw, const Pre& pre) {
  if constexpr (S < SE) {
    constexpr int r = dif_radix(N, S, P);
    constexpr int B = dif_block(N, S, P);
    constexpr int M = B / r;
    if constexpr (r > 8) {
      // large radix: one line per thread (register budget), 8-byte accesses
      for (int e = threadIdx.x; e < L * (N / r); e += blockDim.x) {
        const int ln = e % L, gi = e / L;
        const int j = gi % M, base = (gi / M) * B + j;
        float2 va[r];
#pragma unroll
        for (int k = 0; k < r; ++k) va[k] = xs[(base + M * k) * L + ln];
        if constexpr (S == 0) pre(va, base, M, ln);
        dft_r(va, r);
        if constexpr (M > 1) {
#pragma unroll
          for (int k = 1; k < r; ++k) va[k] = cmulf(va[k], tw[(N / B) * j * k]);
        }
#pragma unroll
        for (int k = 0; k < r; ++k) xs[(base + M * k) * L + ln] = va[k];
      }
      __syncthreads();
      dif_lines_from<N, L, S + 1, P, SE>(xs, tw, pre);
      return;
    }
    constexpr int LP = L / 2;      // a thread transforms two adjacent lines (16-byte accesses)
    for (int e = threadIdx.x; e < LP * (N / r); e += blockDim.x) {
      const int lp = e % LP, gi = e / LP;
      const int j = gi % M, base = (gi / M) * B + j;
      float2 va[r], vb[r];
#pragma unroll
      for (int k = 0; k < r; ++k) {
        const float4 q = *reinterpret_cast<const float4*>(&xs[(base + M * k) * L + 2 * lp]);
        va[k] = make_float2(q.x, q.y);
        vb[k] = make_float2(q.z, q.w);
      }
      if constexpr (S == 0) {
        pre(va, base, M, 2 * lp);
        pre(vb, base, M, 2 * lp + 1);
      }
      dft_r(va, r);
      dft_r(vb, r);
      if constexpr (M > 1) {
#pragma unroll
        for (int k = 1; k < r; ++k) {
          const float2 w = tw[(N / B) * j * k];
          va[k] = cmulf(va[k], w);
          vb[k] = cmulf(vb[k], w);
        }
      }
#pragma unroll
      for (int k = 0; k < r; ++k)
        *reinterpret_cast<float4*>(&xs[(base + M * k) * L + 2 * lp]) =
            make_float4(va[k].x, va[k].y, vb[k].x, vb[k].y);
    }
    __syncthreads();
    dif_lines_from<N, L, S + 1, P, SE>(xs, tw, pre);
  }
}
// L must be even; xs must be 16-byte aligned.
template <int N, int L, class Pre = DifNoPre, int P = kDifTwoStage>
__device__ __forceinline__ void dif_lines(float2* __restrict__ xs, const float2* __restrict__ tw,
                                          const Pre& pre = Pre()) {
  static_assert(L % 2 == 0, "dif_lines transforms lines in pairs");
  dif_lines_from<N, L, 0, P, dif_stages(N, P)>(xs, tw, pre);
}
// The first SE stages only (a caller that finishes the last stage in registers).
template <int N, int L, int SE, class Pre = DifNoPre, int P = kDifTwoStage>
__device__ __forceinline__ void dif_lines_until(float2* __restrict__ xs,
                                                const float2* __restrict__ tw,
                                                const Pre& pre = Pre()) {
  static_assert(L % 2 == 0, "dif_lines transforms lines in pairs");
  dif_lines_from<N, L, 0, P, SE>(xs, tw, pre);
}

// tw[n] = exp(-2 pi i n / N), n < N (all threads of the block; no barrier).
template <int N>
__device__ __forceinline__ void dif_twiddles(float2* tw) {
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    float sn, cn;
    sincospif(-2.0f * (float)i / (float)N, &sn, &cn);
    tw[i] = make_float2(cn, sn);
  }
}

// Fine-grid lengths with compiled pruned passes: the two-stage plans (64 = 8*8, 96 = 16*6,
// 128 = 16*8, 192 = 16*12, 256 = 16*16, 384 = 16*24, 512 = 16*32, 768 = 24*32, 1024 = 32*32)
// and greedy plans (160, 320, 640, 960, 1152, 1280, 1536, 1600), a ladder with steps of at
// most 1.5 that covers fine grids up to 1600 points per axis (the largest a pass's shared-memory
// tile holds); each is exercised on the GPU by a parity test against the FP64 direct sum.
#define MPSQ_FFT_SIZES(X)                                                                    \
  X(64) X(96) X(128) X(160) X(192) X(256) X(320) X(384) X(512) X(640) X(768) X(960) X(1024)   \
  X(1152) X(1280) X(1536) X(1600)

// The smallest compiled length >= n, or 0 above the largest.
inline int64_t compiled_fft_size_at_least(int64_t n) {
  int64_t best = 0;
#define MPSQ_MIN(N) if (N >= n && (best == 0 || N < best)) best = N;
  MPSQ_FFT_SIZES(MPSQ_MIN)
#undef MPSQ_MIN
  return best;
}

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
