// Tensor-core spreading of packed real species pairs (3D, FP32 results).
//
// Within one 16^3 tile the spread of the tile's point records onto z-plane p is a small
// matrix product
//     G_p[y, x] = sum_k A_p[y, k] B[k, x],   A_p[y, k] = s_k ky_k[y] kz_k[p],   B[k, x] = kx_k[x]
// over the records k (kx, ky, kz: the ES kernel values of record k along each axis, zero
// outside its w-cell support; s_k its real strength).  A record adds into the real part of the
// grid when it belongs to the first species of the pair and into the imaginary part otherwise
// (the pair is separated after the transform by Hermitian symmetry), so the two components
// are two independent products over disjoint record sets.
//
// The products run on the tensor cores as mma.sync m16n8k16 (f16 operands, FP32
// accumulators).  FP32 accuracy is kept by splitting each operand v into two f16 terms:
// hi = v with its 13 low mantissa bits cleared (exact in f16), lo = v - hi (exact in FP32,
// rounded to f16), and accumulating Ah*Bh + Ah*Bl + Al*Bh; the dropped Al*Bl term and the
// rounding of lo are below 2^-21 of each product.  From width 8 on (tolerances near 1e-7) the
// Al*Bl term is accumulated too (one more MMA per product term set, ~20 % less error at ~1.3 %
// more step time).  A and B carry a factor 2^10 so that the lo
// terms of kernel values down to ~1e-4 stay in the f16 normal range; the tile is scaled by
// 2^-20 when it is written.  Strengths must satisfy |s| <= 8 (the spatial Hann window's
// maximum), which keeps |A| <= 2^13 well inside the f16 range.
//
// Organisation (one CTA = one tile, 8 warps, warp w owns z-planes 2w and 2w+1):
//  * records are staged in chunks of up to 240; each chunk is counting-sorted in shared
//    memory by (component, start z) and laid out as K-blocks of 16 records that share one
//    component (the second component's block starts on a multiple of 16); thread t then
//    evaluates the kernel of the record in slot t, so a warp writes consecutive columns;
//  * a warp skips every plane outside the union of a K-block's z-supports (sorted start z
//    makes that union narrow);
//  * the accumulators stay in registers; every cell of the tile is written once at the end
//    with 16-byte stores (no zero fill, no global atomics).
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "mpsq_internal.h"

namespace mpsq {
namespace {

constexpr int kCh = 256;            // staging slots per chunk
constexpr int kCap = kCh - 16;      // records per chunk (room for the alignment gap)
constexpr int kKp = kCh + 8;        // float row pitch: conflict-free 64-bit fragment loads
constexpr int kKh = kCh / 2 + 4;    // f16-pair row pitch: conflict-free 32-bit fragment loads

template <int W>
struct MmaSmem {
  static constexpr int kKeys = W + 15;   // start z in [-(W-1), 15]
  float ky[16][kKp];                     // s * ky * 2^10, row y, column slot
  float kz[16][kKp];                     // kz, row z
  uint32_t kxh[16][kKh];                 // hi(kx * 2^10) as f16 pairs (slots 2j, 2j+1), row x
  uint32_t kxl[16][kKh];                 // lo(kx * 2^10)
  int lz[kCh];                           // start z of the record in each slot
  RecF rec[kCh];                         // the record sorted into each slot
  float str[kCh];                        // its real strength
  int member[kCh];                       // the chunk's records grouped by key (chunk order)
  unsigned long long order[kCh];         // their first ordering word (cell offsets, dz bits)
  int count[2 * kKeys];
  int base[2 * kKeys];
  int tcount[2 * kKeys];                 // records per key over the whole tile (large tiles)
  int n0, b1, n1, msel;
};

// The ES kernel value of cell i of a support, phi(z) = exp(beta (sqrt(1 - z^2) - 1)) at
// z = (2 (u + i) - W) / W, u in [0, 1) the point's offset inside its first cell, as a
// polynomial in v = 2u - 1 per cell (Chebyshev interpolation on the host, monomial
// coefficients, Horner on the FMA pipe; no exp/sqrt on the special-function unit).  Degree
// W + 2 up to width 6, 8 at width 7, W from width 8 on: the lowest degrees whose FP32 Horner
// evaluation error (below 1e-7 of the kernel's peak, set by FP32 rounding) is no larger than
// that of W + 2.
template <int W>
struct EsPoly {
  static constexpr int kDeg = W >= 8 ? W : (W == 7 ? 8 : W + 2);
  float c[W][kDeg + 1];   // c[i][k]: coefficient of v^k for cell i
};

template <int W>
__device__ __forceinline__ float es_cell(const EsPoly<W>& p, int i, float v) {
  float r = p.c[i][EsPoly<W>::kDeg];
#pragma unroll
  for (int k = EsPoly<W>::kDeg - 1; k >= 0; --k) r = fmaf(r, v, p.c[i][k]);
  return r;
}

// Chebyshev interpolation of phi on each cell, converted to monomials in v (FP64 on the host).
template <int W>
EsPoly<W> make_es_poly(double beta) {
  constexpr int P = EsPoly<W>::kDeg;
  EsPoly<W> out{};
  for (int i = 0; i < W; ++i) {
    double f[P + 1], a[P + 1];
    for (int j = 0; j <= P; ++j) {
      const double v = std::cos(M_PI * (j + 0.5) / (P + 1));
      const double z = (2.0 * ((v + 1.0) * 0.5 + i) - W) / W;
      f[j] = std::exp(beta * (std::sqrt(std::max(1.0 - z * z, 0.0)) - 1.0));
    }
    for (int k = 0; k <= P; ++k) {
      double s = 0.0;
      for (int j = 0; j <= P; ++j) s += f[j] * std::cos(M_PI * k * (j + 0.5) / (P + 1));
      a[k] = 2.0 * s / (P + 1);
    }
    a[0] *= 0.5;
    // sum_k a_k T_k(v) in monomials: T_0 = 1, T_1 = v, T_{k+1} = 2 v T_k - T_{k-1}
    double t0[P + 1] = {}, t1[P + 1] = {}, m[P + 1] = {};
    t0[0] = 1.0;
    t1[1] = 1.0;
    for (int q = 0; q <= P; ++q) m[q] += a[0] * t0[q];
    if (P >= 1)
      for (int q = 0; q <= P; ++q) m[q] += a[1] * t1[q];
    for (int k = 2; k <= P; ++k) {
      double tk[P + 1] = {};
      for (int q = 0; q <= P; ++q) tk[q] = (q > 0 ? 2.0 * t1[q - 1] : 0.0) - t0[q];
      for (int q = 0; q <= P; ++q) m[q] += a[k] * tk[q];
      for (int q = 0; q <= P; ++q) {
        t0[q] = t1[q];
        t1[q] = tk[q];
      }
    }
    for (int q = 0; q <= P; ++q) out.c[i][q] = (float)m[q];
  }
  return out;
}

__device__ __forceinline__ float clear_low13(float v) {
  return __uint_as_float(__float_as_uint(v) & 0xFFFFE000u);
}

// Two FP32 lanes per instruction (PTX mul/sub .f32x2, IEEE round-to-nearest per lane).
__device__ __forceinline__ float2 mul_f32x2(float2 a, float2 b) {
  unsigned long long pa, pb, r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(pa) : "f"(a.x), "f"(a.y));
  asm("mov.b64 %0, {%1, %2};" : "=l"(pb) : "f"(b.x), "f"(b.y));
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pa), "l"(pb));
  float2 o;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(o.x), "=f"(o.y) : "l"(r));
  return o;
}
__device__ __forceinline__ float2 sub_f32x2(float2 a, float2 b) {
  unsigned long long pa, pb, r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(pa) : "f"(a.x), "f"(a.y));
  asm("mov.b64 %0, {%1, %2};" : "=l"(pb) : "f"(b.x), "f"(b.y));
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pa), "l"(pb));
  float2 o;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(o.x), "=f"(o.y) : "l"(r));
  return o;
}

__device__ __forceinline__ uint32_t pack_f16x2(float first, float second) {
  const __half2 h = __floats2half2_rn(first, second);   // first -> low 16 bits
  uint32_t u;
  memcpy(&u, &h, sizeof(u));
  return u;
}

__device__ __forceinline__ void mma_16816(float (&c)[4], const uint32_t (&a)[4], uint32_t b0,
                                          uint32_t b1) {
  asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 "
               "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
               : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
               : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Four 8x8 f16 matrices from shared memory (ldmatrix): lane i gives the address of row i % 8 of
// matrix i / 8 (16 bytes); r[q] receives row lane / 4, columns 2 (lane % 4) .. +1 of matrix q.
__device__ __forceinline__ void ldmatrix_x4(uint32_t (&r)[4], const void* row_addr) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(row_addr);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(a));
}

// Split f16 A fragment (hi, lo) of plane p for the K-block starting at slot `first`:
// rows g, g+8 (y) x columns 2t, 2t+1, 2t+8, 2t+9 (records), A = (s ky)[y] * kz[p].
template <int W>
__device__ __forceinline__ void build_a(const MmaSmem<W>& sm, int p, int first, int t,
                                        float2 yA0, float2 yA1, float2 yB0, float2 yB1,
                                        uint32_t (&ah)[4], uint32_t (&al)[4]) {
  const float2 zA = *reinterpret_cast<const float2*>(&sm.kz[p][first + 2 * t]);
  const float2 zB = *reinterpret_cast<const float2*>(&sm.kz[p][first + 2 * t + 8]);
  // products and lo terms two lanes per instruction
  const float2 a[4] = {mul_f32x2(yA0, zA), mul_f32x2(yA1, zA), mul_f32x2(yB0, zB),
                       mul_f32x2(yB1, zB)};
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const float2 h = make_float2(clear_low13(a[j].x), clear_low13(a[j].y));
    ah[j] = pack_f16x2(h.x, h.y);
    const float2 l = sub_f32x2(a[j], h);
    al[j] = pack_f16x2(l.x, l.y);
  }
}

// One component's K-blocks [kb0, kb1) of the staged chunk into acc[plane][n-tile][4].
template <int W>
__device__ __forceinline__ void mma_region(const MmaSmem<W>& sm, int kb0, int kb1, int end,
                                           int p0, int g, int t, float (&acc)[2][2][4]) {
  for (int kb = kb0; kb < kb1; ++kb) {
    const int first = kb * 16;
    const int last = min(first + 15, end - 1);
    const int zlo = sm.lz[first], zhi = sm.lz[last] + W - 1;
    const bool use0 = p0 >= zlo && p0 <= zhi;
    const bool use1 = p0 + 1 >= zlo && p0 + 1 <= zhi;
    if (!use0 && !use1) continue;                       // warp-uniform
    // B fragments of both n-tiles (hi and lo) by ldmatrix: matrix q = lane / 8 covers x rows
    // (q / 2) * 8 .. +7 and records (q % 2) * 8 .. +7 of the K-block; the four registers are
    // b0, b1 of n-tile 0 and b0, b1 of n-tile 1
    uint32_t bh4[4], bl4[4];
    {
      const int lane = 4 * g + t, q = lane >> 3, r = lane & 7;
      const int row = (q >> 1) * 8 + r, col = kb * 8 + (q & 1) * 4;   // u32 column (f16 pairs)
      ldmatrix_x4(bh4, &sm.kxh[row][col]);
      ldmatrix_x4(bl4, &sm.kxl[row][col]);
    }
    const uint32_t bh[2][2] = {{bh4[0], bh4[1]}, {bh4[2], bh4[3]}};
    const uint32_t bl[2][2] = {{bl4[0], bl4[1]}, {bl4[2], bl4[3]}};
    const float2 yA0 = *reinterpret_cast<const float2*>(&sm.ky[g][first + 2 * t]);
    const float2 yA1 = *reinterpret_cast<const float2*>(&sm.ky[g + 8][first + 2 * t]);
    const float2 yB0 = *reinterpret_cast<const float2*>(&sm.ky[g][first + 2 * t + 8]);
    const float2 yB1 = *reinterpret_cast<const float2*>(&sm.ky[g + 8][first + 2 * t + 8]);
    // each product term is issued to every accumulator chain before the next term, so that
    // consecutive MMAs are independent (the smallest terms first)
    if (use0 && use1) {   // both planes: four independent accumulator chains
      uint32_t ah0[4], al0[4], ah1[4], al1[4];
      build_a(sm, p0, first, t, yA0, yA1, yB0, yB1, ah0, al0);
      build_a(sm, p0 + 1, first, t, yA0, yA1, yB0, yB1, ah1, al1);
      if constexpr (W >= 8) {
#pragma unroll
        for (int nt = 0; nt < 2; ++nt) {
          mma_16816(acc[0][nt], al0, bl[nt][0], bl[nt][1]);
          mma_16816(acc[1][nt], al1, bl[nt][0], bl[nt][1]);
        }
      }
#pragma unroll
      for (int nt = 0; nt < 2; ++nt) {
        mma_16816(acc[0][nt], al0, bh[nt][0], bh[nt][1]);
        mma_16816(acc[1][nt], al1, bh[nt][0], bh[nt][1]);
      }
#pragma unroll
      for (int nt = 0; nt < 2; ++nt) {
        mma_16816(acc[0][nt], ah0, bl[nt][0], bl[nt][1]);
        mma_16816(acc[1][nt], ah1, bl[nt][0], bl[nt][1]);
      }
#pragma unroll
      for (int nt = 0; nt < 2; ++nt) {
        mma_16816(acc[0][nt], ah0, bh[nt][0], bh[nt][1]);
        mma_16816(acc[1][nt], ah1, bh[nt][0], bh[nt][1]);
      }
    } else if (use0) {
      uint32_t ah[4], al[4];
      build_a(sm, p0, first, t, yA0, yA1, yB0, yB1, ah, al);
      if constexpr (W >= 8) {
#pragma unroll
        for (int nt = 0; nt < 2; ++nt) mma_16816(acc[0][nt], al, bl[nt][0], bl[nt][1]);
      }
#pragma unroll
      for (int nt = 0; nt < 2; ++nt) mma_16816(acc[0][nt], al, bh[nt][0], bh[nt][1]);
#pragma unroll
      for (int nt = 0; nt < 2; ++nt) mma_16816(acc[0][nt], ah, bl[nt][0], bl[nt][1]);
#pragma unroll
      for (int nt = 0; nt < 2; ++nt) mma_16816(acc[0][nt], ah, bh[nt][0], bh[nt][1]);
    } else {
      uint32_t ah[4], al[4];
      build_a(sm, p0 + 1, first, t, yA0, yA1, yB0, yB1, ah, al);
      if constexpr (W >= 8) {
#pragma unroll
        for (int nt = 0; nt < 2; ++nt) mma_16816(acc[1][nt], al, bl[nt][0], bl[nt][1]);
      }
#pragma unroll
      for (int nt = 0; nt < 2; ++nt) mma_16816(acc[1][nt], al, bh[nt][0], bh[nt][1]);
#pragma unroll
      for (int nt = 0; nt < 2; ++nt) mma_16816(acc[1][nt], ah, bl[nt][0], bl[nt][1]);
#pragma unroll
      for (int nt = 0; nt < 2; ++nt) mma_16816(acc[1][nt], ah, bh[nt][0], bh[nt][1]);
    }
  }
}

template <int W, bool REPRO>
__global__ void __launch_bounds__(256, 3)
    spread3_pair_mma_kernel(SpreadArgs a, const RecF* __restrict__ recs,
                            const int* __restrict__ idx, const float2* __restrict__ cv,
                            int64_t c_stride, const int* __restrict__ starts,
                            float2* __restrict__ fine, const EsPoly<W> poly, int64_t key0,
                            int z0, int64_t gstride) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  MmaSmem<W>& sm = *reinterpret_cast<MmaSmem<W>*>(smem_raw);
  constexpr int K1 = MmaSmem<W>::kKeys;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int g = lane >> 2, t = lane & 3;
  const int p0 = 2 * warp;
  const int64_t key = key0 + blockIdx.x;
  const int trans = blockIdx.y;
  const int keygrid = (int)(key / a.n_tiles);
  const int tile = (int)(key - (int64_t)keygrid * a.n_tiles);
  const int tx = tile % a.ntile[0];
  const int ty = (tile / a.ntile[0]) % a.ntile[1];
  const int tz = tile / (a.ntile[0] * a.ntile[1]);
  float acc_re[2][2][4], acc_im[2][2][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
      for (int k = 0; k < 4; ++k) acc_re[i][j][k] = acc_im[i][j][k] = 0.0f;
  const int r0 = starts[key], r1 = starts[key + 1];
  // Chunks of at most kCap records, in binning order.  Reproducible order (REPRO): all of the
  // tile's records when they fit one chunk; otherwise whole (component, start z) keys, counted
  // first, packed greedily into chunks (keys in order), so that the partition, like the order
  // inside a chunk, does not depend on the order the records were binned in.  A single key
  // with more than kCap records (an extremely dense tile) takes the binning order.
  auto key_of = [&](const RecF& q) {
    const int lz = ((q.packed >> 16) & 0xff) - 64;
    return ((q.packed >> 24) & 1) * K1 + min(max(lz + W - 1, 0), K1 - 1);
  };
  auto strength = [&](int r) {
    return !cv ? 1.0f : (idx ? cv[(int64_t)trans * c_stride + idx[r]] : cv[r]).x;
  };
  bool by_key = false;
  if (REPRO && r1 - r0 > kCap) {
    for (int e = tid; e < 2 * K1; e += 256) sm.tcount[e] = 0;
    __syncthreads();
    for (int r = r0 + tid; r < r1; r += 256) atomicAdd(&sm.tcount[key_of(recs[r])], 1);
    __syncthreads();
    by_key = true;
    for (int e = 0; e < 2 * K1; ++e) by_key = by_key && sm.tcount[e] <= kCap;
  }
  int c0 = r0, kb = 0;
  for (;;) {
    int n = 0, kb_hi = kb;
    if (by_key) {
      if (kb >= 2 * K1) break;
      while (kb_hi < 2 * K1 && n + sm.tcount[kb_hi] <= kCap) n += sm.tcount[kb_hi++];
    } else {
      if (c0 >= r1) break;
      n = min(kCap, r1 - c0);
    }
    {  // zero the staging arrays (alignment-gap slots and out-of-support rows must read 0)
      uint4* z4 = reinterpret_cast<uint4*>(&sm.ky[0][0]);
      constexpr int nz = (int)((sizeof(sm.ky) + sizeof(sm.kz) + sizeof(sm.kxh) + sizeof(sm.kxl)) / 16);
      for (int e = tid; e < nz; e += 256) z4[e] = make_uint4(0u, 0u, 0u, 0u);
      for (int e = tid; e < 2 * K1; e += 256) sm.count[e] = 0;
      if (tid == 0) sm.msel = 0;
    }
    __syncthreads();
    // 1. the chunk's records into slots 0..n-1 in any order (by position, or selected by key)
    RecF rec;
    float sv = 0.0f;
    int k = 0, rank = 0;
    if (!REPRO) {
      if (tid < n) {
        rec = recs[c0 + tid];
        sv = strength(c0 + tid);
      }
    } else if (!by_key) {
      if (tid < n) {
        sm.rec[tid] = recs[c0 + tid];
        sm.str[tid] = strength(c0 + tid);
      }
    } else {
      for (int r = r0 + tid; r < r1; r += 256) {
        const RecF q = recs[r];
        const int k = key_of(q);
        if (k >= kb && k < kb_hi) {
          const int at = atomicAdd(&sm.msel, 1);
          sm.rec[at] = q;
          sm.str[at] = strength(r);
        }
      }
    }
    if (REPRO) __syncthreads();
    // 2. group the records by key (component, start z)
    if (tid < n) {
      if (REPRO) {
        rec = sm.rec[tid];
        sv = sm.str[tid];
      }
      k = key_of(rec);
      rank = atomicAdd(&sm.count[k], 1);
    }
    __syncthreads();
    // 3. exclusive scan of the key counts (one warp; K1 <= 23 keys per component); the
    //    second component starts on a multiple of 16
    if (warp == 0) {
      const int c0n = lane < K1 ? sm.count[lane] : 0;
      const int c1n = lane < K1 ? sm.count[K1 + lane] : 0;
      int i0 = c0n, i1 = c1n;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int u0 = __shfl_up_sync(0xffffffffu, i0, o), u1 = __shfl_up_sync(0xffffffffu, i1, o);
        if (lane >= o) {
          i0 += u0;
          i1 += u1;
        }
      }
      const int n0 = __shfl_sync(0xffffffffu, i0, 31), n1 = __shfl_sync(0xffffffffu, i1, 31);
      const int b1 = (n0 + 15) & ~15;
      if (lane < K1) {
        sm.base[lane] = i0 - c0n;
        sm.base[K1 + lane] = b1 + i1 - c1n;
      }
      if (lane == 0) {
        sm.n0 = n0;
        sm.b1 = b1;
        sm.n1 = n1;
      }
    }
    __syncthreads();
    // 4. the slot within the key: the binning order, or (REPRO) the order by content (cell
    //    offsets, then offsets and strength bits), so that the slots, and with them the
    //    accumulation order, follow from the record set alone; records equal in every bit may
    //    take either order
    int pos = rank;
    const uint64_t mine =
        tid < n ? ((uint64_t)(uint32_t)rec.packed << 32) | __float_as_uint(rec.dz) : 0ull;
    if (REPRO) {
      if (tid < n) {
        sm.member[sm.base[k] + rank] = tid;
        sm.order[sm.base[k] + rank] = mine;
      }
      __syncthreads();
    }
    if (REPRO && tid < n) {
      pos = 0;
      const int b = sm.base[k], cnt = sm.count[k];
      for (int q = b; q < b + cnt; ++q) {
        const uint64_t other = sm.order[q];   // one load per member; the record only on a tie
        bool before = other < mine;
        if (other == mine && q != b + rank) {
          const int o = sm.member[q];
          const RecF& u = sm.rec[o];
          const uint32_t a[3] = {__float_as_uint(u.dy), __float_as_uint(u.dx), __float_as_uint(sm.str[o])};
          const uint32_t m[3] = {__float_as_uint(rec.dy), __float_as_uint(rec.dx), __float_as_uint(sv)};
          before = a[0] != m[0] ? a[0] < m[0] : a[1] != m[1] ? a[1] < m[1] : a[2] != m[2] ? a[2] < m[2] : o < tid;
        }
        pos += before ? 1 : 0;
      }
    }
    if (REPRO) __syncthreads();
    if (tid < n) {
      const int slot = sm.base[k] + pos;
      sm.rec[slot] = rec;
      sm.str[slot] = sv;
    }
    __syncthreads();
    // 5. thread t evaluates the kernel of the record in slot t and writes its support rows
    //    (consecutive threads write consecutive columns of a row: no bank conflicts)
    {
      const int st = tid;
      const bool live = st < sm.n0 || (st >= sm.b1 && st < sm.b1 + sm.n1);
      if (live) {
        const RecF q = sm.rec[st];
        const float s = sm.str[st] * 1024.0f;
        const int lx = (q.packed & 0xff) - 64;
        const int ly = ((q.packed >> 8) & 0xff) - 64;
        const int lz = ((q.packed >> 16) & 0xff) - 64;
        // offsets d in [-W/2, -W/2 + 1) -> polynomial variable v = 2d + W - 1 in [-1, 1)
        const float vx = fmaf(2.0f, q.dx, (float)(W - 1));
        const float vy = fmaf(2.0f, q.dy, (float)(W - 1));
        const float vz = fmaf(2.0f, q.dz, (float)(W - 1));
        __half* xh = reinterpret_cast<__half*>(&sm.kxh[0][0]);
        __half* xl = reinterpret_cast<__half*>(&sm.kxl[0][0]);
#pragma unroll
        for (int i = 0; i < W; ++i) {
          const int x = lx + i, y = ly + i, z = lz + i;
          if (x >= 0 && x < 16) {
            const float v = es_cell(poly, i, vx) * 1024.0f;
            const float h = clear_low13(v);
            xh[x * 2 * kKh + st] = __float2half_rn(h);
            xl[x * 2 * kKh + st] = __float2half_rn(v - h);
          }
          if (y >= 0 && y < 16) sm.ky[y][st] = es_cell(poly, i, vy) * s;
          if (z >= 0 && z < 16) sm.kz[z][st] = es_cell(poly, i, vz);
        }
        sm.lz[st] = lz;
      }
    }
    __syncthreads();
    const int n0 = sm.n0, b1 = sm.b1, n1 = sm.n1;
    mma_region<W>(sm, 0, (n0 + 15) >> 4, n0, p0, g, t, acc_re);
    mma_region<W>(sm, b1 >> 4, (b1 + n1 + 15) >> 4, b1 + n1, p0, g, t, acc_im);
    c0 += kCap;
    kb = kb_hi;
    __syncthreads();   // another chunk reuses the staging arrays
  }
  float2* out = fine + (int64_t)(keygrid + trans) * gstride;
  const int64_t nf0 = a.nf[0], nf1 = a.nf[1];
  const float sc = 1.0f / 1048576.0f;
#pragma unroll
  for (int pi = 0; pi < 2; ++pi) {
    const int64_t zrow = ((int64_t)tz * 16 - z0 + p0 + pi) * nf1 + (int64_t)ty * 16;
#pragma unroll
    for (int nt = 0; nt < 2; ++nt) {
      const int64_t xcol = (int64_t)tx * 16 + nt * 8 + 2 * t;
#pragma unroll
      for (int hv = 0; hv < 2; ++hv) {
        const int y = g + 8 * hv;
        const float4 v = make_float4(acc_re[pi][nt][2 * hv] * sc, acc_im[pi][nt][2 * hv] * sc,
                                     acc_re[pi][nt][2 * hv + 1] * sc, acc_im[pi][nt][2 * hv + 1] * sc);
        *reinterpret_cast<float4*>(out + (zrow + y) * nf0 + xcol) = v;
      }
    }
  }
}

template <int W>
int launch_w(const SpreadArgs& a, const RecF* recs, const int* idx, const float2* cv,
             int64_t c_stride, const int* starts, int nkeys, int ntrans, float2* fine,
             cudaStream_t s, int64_t key0, int z0, int64_t gstride, bool repro) {
  static std::once_flag once;
  static cudaError_t attr = cudaSuccess;
  std::call_once(once, [] {
    attr = cudaFuncSetAttribute(spread3_pair_mma_kernel<W, false>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)sizeof(MmaSmem<W>));
    if (attr == cudaSuccess)
      attr = cudaFuncSetAttribute(spread3_pair_mma_kernel<W, true>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)sizeof(MmaSmem<W>));
  });
  if (attr != cudaSuccess) return fail(MPSQ_ERR_CUDA, "spread mma attribute: %s", cudaGetErrorString(attr));
  static std::mutex mu;
  static double cached_beta = -1.0;
  static EsPoly<W> poly;
  EsPoly<W> p;
  {
    std::lock_guard<std::mutex> lock(mu);
    if (cached_beta != a.beta) {
      poly = make_es_poly<W>(a.beta);
      cached_beta = a.beta;
    }
    p = poly;
  }
  const dim3 grid((unsigned)nkeys, (unsigned)ntrans);
  if (repro)
    spread3_pair_mma_kernel<W, true><<<grid, 256, sizeof(MmaSmem<W>), s>>>(
        a, recs, idx, cv, c_stride, starts, fine, p, key0, z0, gstride);
  else
    spread3_pair_mma_kernel<W, false><<<grid, 256, sizeof(MmaSmem<W>), s>>>(
        a, recs, idx, cv, c_stride, starts, fine, p, key0, z0, gstride);
  MPSQ_LAUNCH_CHECK();
  return MPSQ_OK;
}

}  // namespace

bool spread_pair_mma_enabled() {
  static const bool on = [] {
    const char* e = getenv("MPSQ_SPREAD");
    return !(e && strcmp(e, "fma") == 0);
  }();
  return on;
}

int launch_spread_pair_mma(const SpreadArgs& a, const RecF* recs, const int* idx,
                           const float2* cv, int64_t c_stride, const int* starts, int nkeys,
                           int ntrans, float2* fine, cudaStream_t s, int64_t key0, int z0,
                           int64_t gstride, bool repro) {
  if (a.dim != 3 || a.tile[0] != 16 || a.tile[1] != 16 || a.tile[2] != 16)
    return fail(MPSQ_ERR_ARG, "spread mma: 16^3 tiles only");
  if ((reinterpret_cast<uintptr_t>(fine) & 15) != 0 || (a.nf[0] & 1) != 0)
    return fail(MPSQ_ERR_ARG, "spread mma: grid must be 16-byte aligned with even rows");
  if (gstride <= 0) {
    key0 = 0;
    z0 = 0;
    gstride = a.n_fine;
  }
  if (nkeys <= 0) return MPSQ_OK;
#define MPSQ_W(W) \
  launch_w<W>(a, recs, idx, cv, c_stride, starts, nkeys, ntrans, fine, s, key0, z0, gstride, \
              repro)
  switch (a.w) {
    case 3: return MPSQ_W(3);
    case 4: return MPSQ_W(4);
    case 5: return MPSQ_W(5);
    case 6: return MPSQ_W(6);
    case 7: return MPSQ_W(7);
    case 8: return MPSQ_W(8);
#undef MPSQ_W
    default: return fail(MPSQ_ERR_ARG, "spread mma: kernel width %d not compiled", a.w);
  }
}

}  // namespace mpsq
