/*
 * ORACLE — test infrastructure only.  Imported by tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference arm of bench.py as the checker; never part of the product path.
 *
 * FP64 direct evaluation of the type-1 nonuniform Fourier sum, restated from its definition:
 *   fk(k1,k2[,k3]) = sum_j cj exp(i*sgn(iflag)*(k1 xj + k2 yj [+ k3 zj]))
 *   for -m/2 <= k <= (m-1)/2, modes stored k1 fastest starting at -m/2
 * — the same sum, mode range and sign rule as the direct-FT check path of the reference
 * (code/src/mp_sqom56.f90:2530-2547, selected by j_fft=0 at :1147-1152) and the FINUFFT call
 * it checks (:1148).  The code is this project's own: rows are split over OpenMP threads and
 * each point's phase factors along k1 come from an exactly recomputed base every 16 steps.
 *
 * Also: a CPU restatement of exponential-of-semicircle spreading (Barnett, Magland,
 * af Klinteberg 2019) used by the CPU NUFFT port that serves as the host-core baseline.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static void phase_row(double x, double s, int64_t kmin, int64_t m, double* re, double* im) {
  /* re[i] + i im[i] = exp(i s (kmin + i) x) */
  double cs = cos(s * x), sn = sin(s * x);
  for (int64_t i = 0; i < m; ++i) {
    if ((i & 15) == 0) {
      double a = s * (double)(kmin + i) * x;
      re[i] = cos(a);
      im[i] = sin(a);
    } else {
      re[i] = re[i - 1] * cs - im[i - 1] * sn;
      im[i] = re[i - 1] * sn + im[i - 1] * cs;
    }
  }
}

void oracle_dirft2d1(int64_t nj, const double* x, const double* y, const double* c, int iflag,
                     int64_t ms, int64_t mt, double* fk) {
  const double s = iflag >= 0 ? 1.0 : -1.0;
  memset(fk, 0, sizeof(double) * 2 * ms * mt);
#pragma omp parallel
  {
    double* er = (double*)malloc(sizeof(double) * ms);
    double* ei = (double*)malloc(sizeof(double) * ms);
#pragma omp for schedule(dynamic, 1)
    for (int64_t l = 0; l < mt; ++l) {
      const int64_t k2 = l - mt / 2;
      double* row = fk + 2 * ms * l;
      for (int64_t j = 0; j < nj; ++j) {
        const double a = s * (double)k2 * y[j];
        const double br = cos(a), bi = sin(a);
        const double cr = c[2 * j] * br - c[2 * j + 1] * bi;
        const double ci = c[2 * j] * bi + c[2 * j + 1] * br;
        phase_row(x[j], s, -ms / 2, ms, er, ei);
        for (int64_t i = 0; i < ms; ++i) {
          row[2 * i] += cr * er[i] - ci * ei[i];
          row[2 * i + 1] += cr * ei[i] + ci * er[i];
        }
      }
    }
    free(er);
    free(ei);
  }
}

void oracle_dirft3d1(int64_t nj, const double* x, const double* y, const double* z,
                     const double* c, int iflag, int64_t ms, int64_t mt, int64_t mu, double* fk) {
  const double s = iflag >= 0 ? 1.0 : -1.0;
  memset(fk, 0, sizeof(double) * 2 * ms * mt * mu);
#pragma omp parallel
  {
    double* er = (double*)malloc(sizeof(double) * ms);
    double* ei = (double*)malloc(sizeof(double) * ms);
#pragma omp for schedule(dynamic, 1)
    for (int64_t row_id = 0; row_id < mt * mu; ++row_id) {
      const int64_t l = row_id % mt, n = row_id / mt;
      const int64_t k2 = l - mt / 2, k3 = n - mu / 2;
      double* row = fk + 2 * ms * row_id;
      for (int64_t j = 0; j < nj; ++j) {
        const double a = s * ((double)k2 * y[j] + (double)k3 * z[j]);
        const double br = cos(a), bi = sin(a);
        const double cr = c[2 * j] * br - c[2 * j + 1] * bi;
        const double ci = c[2 * j] * bi + c[2 * j + 1] * br;
        phase_row(x[j], s, -ms / 2, ms, er, ei);
        for (int64_t i = 0; i < ms; ++i) {
          row[2 * i] += cr * er[i] - ci * ei[i];
          row[2 * i + 1] += cr * ei[i] + ci * er[i];
        }
      }
    }
    free(er);
    free(ei);
  }
}

/* Selected modes only: out[q] = sum_j cj exp(i s (k1 x + k2 y + k3 z)), k = kq[3q..3q+2];
 * dim 2 ignores z.  Used at full problem sizes where only a sample of modes is checked. */
void oracle_dirft_modes(int dim, int64_t nj, const double* x, const double* y, const double* z,
                        const double* c, int iflag, int64_t nq, const int64_t* kq, double* out) {
  const double s = iflag >= 0 ? 1.0 : -1.0;
#pragma omp parallel for schedule(dynamic, 4)
  for (int64_t q = 0; q < nq; ++q) {
    const double k1 = (double)kq[3 * q], k2 = (double)kq[3 * q + 1],
                 k3 = dim == 3 ? (double)kq[3 * q + 2] : 0.0;
    double sr = 0.0, si = 0.0;
    for (int64_t j = 0; j < nj; ++j) {
      double a = k1 * x[j] + k2 * y[j];
      if (dim == 3) a += k3 * z[j];
      a *= s;
      const double br = cos(a), bi = sin(a);
      sr += c[2 * j] * br - c[2 * j + 1] * bi;
      si += c[2 * j] * bi + c[2 * j + 1] * br;
    }
    out[2 * q] = sr;
    out[2 * q + 1] = si;
  }
}

/* Selected modes, for large point sets: per point, the phase factors of every mode index along
 * each axis (phase_row, recomputed exactly every 16 steps), then the product of the three axis
 * factors per selected mode.  kq holds nq triples inside [kmin[a], kmin[a] + span[a]).  Points
 * are split over threads, each accumulating its own partial sums; the partials are added in
 * thread order. */
void oracle_dirft_modes_tab(int dim, int64_t nj, const double* x, const double* y, const double* z,
                            const double* c, int iflag, int64_t nq, const int64_t* kq,
                            const int64_t* kmin, const int64_t* span, double* out) {
  const double s = iflag >= 0 ? 1.0 : -1.0;
  int nt = 1;
#ifdef _OPENMP
  nt = omp_get_max_threads();
#endif
  double* part = (double*)calloc((size_t)nt * 2 * (size_t)nq, sizeof(double));
  if (!part) return;
#pragma omp parallel
  {
    int t = 0;
#ifdef _OPENMP
    t = omp_get_thread_num();
#endif
    double* acc = part + (size_t)t * 2 * (size_t)nq;
    double* tab[3][2];
    for (int a = 0; a < 3; ++a) {
      tab[a][0] = (double*)malloc(sizeof(double) * (size_t)(span[a] > 0 ? span[a] : 1));
      tab[a][1] = (double*)malloc(sizeof(double) * (size_t)(span[a] > 0 ? span[a] : 1));
    }
#pragma omp for schedule(static)
    for (int64_t j = 0; j < nj; ++j) {
      const double pos[3] = {x[j], y[j], dim == 3 ? z[j] : 0.0};
      for (int a = 0; a < dim; ++a) phase_row(pos[a], s, kmin[a], span[a], tab[a][0], tab[a][1]);
      const double cr = c[2 * j], ci = c[2 * j + 1];
      for (int64_t q = 0; q < nq; ++q) {
        const int64_t i0 = kq[3 * q] - kmin[0], i1 = kq[3 * q + 1] - kmin[1];
        double er = tab[0][0][i0] * tab[1][0][i1] - tab[0][1][i0] * tab[1][1][i1];
        double ei = tab[0][0][i0] * tab[1][1][i1] + tab[0][1][i0] * tab[1][0][i1];
        if (dim == 3) {
          const int64_t i2 = kq[3 * q + 2] - kmin[2];
          const double fr = er * tab[2][0][i2] - ei * tab[2][1][i2];
          ei = er * tab[2][1][i2] + ei * tab[2][0][i2];
          er = fr;
        }
        acc[2 * q] += cr * er - ci * ei;
        acc[2 * q + 1] += cr * ei + ci * er;
      }
    }
    for (int a = 0; a < 3; ++a) {
      free(tab[a][0]);
      free(tab[a][1]);
    }
  }
  for (int64_t q = 0; q < 2 * nq; ++q) {
    double v = 0.0;
    for (int t = 0; t < nt; ++t) v += part[(size_t)t * 2 * (size_t)nq + q];
    out[q] = v;
  }
  free(part);
}

/* CPU exponential-of-semicircle spreading onto an n0 x n1 x n2 periodic grid (interleaved
 * complex, x fastest, zeroed by the caller).  g: 3*nj grid coordinates already folded to
 * [0, n).  Kernel phi(z) = exp(beta (sqrt(1 - z^2) - 1)) on w cells per axis.
 *
 * Organisation (the sorted, block-wise spreading of Barnett, Magland, af Klinteberg 2019, sec. 3):
 * the points are counting-sorted by the 8^dim block of their first support cell, slowest along
 * the partitioned axis (z in 3D, y in 2D); each thread owns a contiguous range of planes (rows)
 * of that axis and walks only the blocks whose support reaches them, so no two threads write
 * the same cell and consecutive points touch neighbouring grid memory.  Each point's wrapped
 * support indices are formed once; a support that does not wrap along x is one contiguous run
 * of the row.  Contributions to a cell are summed in the sorted point order. */
#define ES_BLOCK 8
#define ES_WMAX 32

static inline int64_t wrap_index(int64_t i, int64_t n) {
  int64_t r = i % n;
  return r < 0 ? r + n : r;
}

void oracle_es_spread(int dim, int64_t nj, const double* g, const double* c, int w, double beta,
                      int64_t n0, int64_t n1, int64_t n2, double* grid) {
  if (nj <= 0 || w < 1 || w > ES_WMAX) return;
  const int ax = dim == 3 ? 2 : 1;                      /* partitioned axis */
  const int64_t nslab = dim == 3 ? n2 : n1;
  const int64_t nb0 = (n0 + ES_BLOCK - 1) / ES_BLOCK, nb1 = (n1 + ES_BLOCK - 1) / ES_BLOCK;
  const int64_t nb2 = dim == 3 ? (n2 + ES_BLOCK - 1) / ES_BLOCK : 1;
  const int64_t nkeys = nb0 * nb1 * nb2;
  const int64_t nbs = dim == 3 ? nb2 : nb1;             /* blocks along the partitioned axis */
  const int64_t per_slab_block = nkeys / nbs;           /* keys per block of that axis */
  int64_t* start = (int64_t*)malloc(3 * sizeof(int64_t) * (size_t)nj);   /* wrapped first cells */
  int64_t* key = (int64_t*)malloc(sizeof(int64_t) * (size_t)nj);
  int64_t* order = (int64_t*)malloc(sizeof(int64_t) * (size_t)nj);
  int64_t* off = (int64_t*)calloc((size_t)nkeys + 1, sizeof(int64_t));
  if (!start || !key || !order || !off) {
    free(start); free(key); free(order); free(off);
    return;
  }
#pragma omp parallel for schedule(static)
  for (int64_t j = 0; j < nj; ++j) {
    const double* gj = g + 3 * j;
    int64_t s0 = wrap_index((int64_t)ceil(gj[0] - 0.5 * w), n0);
    int64_t s1 = wrap_index((int64_t)ceil(gj[1] - 0.5 * w), n1);
    int64_t s2 = dim == 3 ? wrap_index((int64_t)ceil(gj[2] - 0.5 * w), n2) : 0;
    start[3 * j] = s0; start[3 * j + 1] = s1; start[3 * j + 2] = s2;
    key[j] = ((s2 / ES_BLOCK) * nb1 + s1 / ES_BLOCK) * nb0 + s0 / ES_BLOCK;
  }
  /* stable counting sort of the points by key */
  for (int64_t j = 0; j < nj; ++j) off[key[j] + 1]++;
  for (int64_t k = 0; k < nkeys; ++k) off[k + 1] += off[k];
  {
    int64_t* cur = (int64_t*)malloc(sizeof(int64_t) * (size_t)nkeys);
    if (!cur) { free(start); free(key); free(order); free(off); return; }
    memcpy(cur, off, sizeof(int64_t) * (size_t)nkeys);
    for (int64_t j = 0; j < nj; ++j) order[cur[key[j]]++] = j;
    free(cur);
  }
#pragma omp parallel
  {
    int nt = 1, tid = 0;
#ifdef _OPENMP
    nt = omp_get_num_threads();
    tid = omp_get_thread_num();
#endif
    const int64_t lo = nslab * tid / nt, hi = nslab * (tid + 1) / nt;
    double kx[ES_WMAX], ky[ES_WMAX], kz[ES_WMAX];
    int64_t ix[ES_WMAX], iy[ES_WMAX], iz[ES_WMAX];
    const double inv = 2.0 / w;
    for (int64_t bs = 0; bs < nbs && lo < hi; ++bs) {
      /* support planes of this block: [bs*B, min(bs*B + B, nslab) + w - 1), periodically */
      const int64_t first = bs * ES_BLOCK;
      const int64_t span = (first + ES_BLOCK < nslab ? ES_BLOCK : nslab - first) + w - 1;
      int meets = 0;
      if (span >= nslab) {
        meets = 1;
      } else {
        for (int64_t p = 0; p < span && !meets; ++p) {
          const int64_t q = (first + p) % nslab;
          if (q >= lo && q < hi) meets = 1;
        }
      }
      if (!meets) continue;
      const int64_t e0 = off[bs * per_slab_block], e1 = off[(bs + 1) * per_slab_block];
      for (int64_t e = e0; e < e1; ++e) {
        const int64_t j = order[e];
        const double* gj = g + 3 * j;
        const int64_t* sj = start + 3 * j;
        /* the unwrapped first cell: the wrapped one minus a multiple of n, so the offsets to
         * the point are the same */
        const double f0 = ceil(gj[0] - 0.5 * w), f1 = ceil(gj[1] - 0.5 * w);
        const double f2 = dim == 3 ? ceil(gj[2] - 0.5 * w) : 0.0;
        for (int a = 0; a < w; ++a) {
          const double zx = (f0 + a - gj[0]) * inv, zy = (f1 + a - gj[1]) * inv;
          kx[a] = exp(beta * (sqrt(fmax(0.0, 1.0 - zx * zx)) - 1.0));
          ky[a] = exp(beta * (sqrt(fmax(0.0, 1.0 - zy * zy)) - 1.0));
          if (dim == 3) {
            const double zz = (f2 + a - gj[2]) * inv;
            kz[a] = exp(beta * (sqrt(fmax(0.0, 1.0 - zz * zz)) - 1.0));
          } else {
            kz[a] = 1.0;
          }
          int64_t t = sj[0] + a; ix[a] = t >= n0 ? t - n0 : t;
          t = sj[1] + a; iy[a] = t >= n1 ? t - n1 : t;
          t = sj[2] + a; iz[a] = dim == 3 ? (t >= n2 ? t - n2 : t) : 0;
        }
        const int contiguous = sj[0] + w <= n0;
        const double cr = c[2 * j], ci = c[2 * j + 1];
        const int wz = dim == 3 ? w : 1;
        for (int az = 0; az < wz; ++az) {
          if (dim == 3 && (iz[az] < lo || iz[az] >= hi)) continue;
          for (int ay = 0; ay < w; ++ay) {
            if (dim == 2 && (iy[ay] < lo || iy[ay] >= hi)) continue;
            const double v = kz[az] * ky[ay];
            const double vr = v * cr, vi = v * ci;
            double* row = grid + 2 * ((iz[az] * n1 + iy[ay]) * n0);
            if (contiguous) {
              double* cell = row + 2 * sj[0];
              for (int a = 0; a < w; ++a) {
                cell[2 * a] += vr * kx[a];
                cell[2 * a + 1] += vi * kx[a];
              }
            } else {
              for (int a = 0; a < w; ++a) {
                row[2 * ix[a]] += vr * kx[a];
                row[2 * ix[a] + 1] += vi * kx[a];
              }
            }
          }
        }
      }
    }
  }
  free(start); free(key); free(order); free(off);
}

/* Deconvolution and mode extraction of the type-1 NUFFT: out[k2][k1][k0] = G[(k2 - m2/2) mod n2]
 * [(k1 - m1/2) mod n1][(k0 - m0/2) mod n0] * c0[k0] c1[k1] c2[k2] (interleaved complex, k0
 * fastest; dim 2: m2 = n2 = 1 and c2 unused). */
void oracle_es_extract(int dim, const double* G, int64_t n0, int64_t n1, int64_t n2, int64_t m0,
                       int64_t m1, int64_t m2, const double* c0, const double* c1,
                       const double* c2, double* out) {
  if (dim != 3) { m2 = 1; n2 = 1; }
#pragma omp parallel for schedule(static)
  for (int64_t r = 0; r < m2 * m1; ++r) {
    const int64_t k2 = r / m1, k1 = r % m1;
    const int64_t i2 = wrap_index(k2 - m2 / 2, n2), i1 = wrap_index(k1 - m1 / 2, n1);
    const double f = c1[k1] * (dim == 3 ? c2[k2] : 1.0);
    const double* src = G + 2 * ((i2 * n1 + i1) * n0);
    double* dst = out + 2 * r * m0;
    for (int64_t k0 = 0; k0 < m0; ++k0) {
      const int64_t i0 = wrap_index(k0 - m0 / 2, n0);
      const double t = f * c0[k0];
      dst[2 * k0] = src[2 * i0] * t;
      dst[2 * k0 + 1] = src[2 * i0 + 1] * t;
    }
  }
}

/* Species weighting of one frame: cs[i] = (first ? 0 : cs[i]) + w[i] A[i] (A, cs interleaved
 * complex, w real per Q), the sum over species of code/src/mp_sqom56.f90:1338-1377. */
void oracle_weight_accumulate(int64_t n, const double* w, const double* A, double* cs, int first) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    const double re = w[i] * A[2 * i], im = w[i] * A[2 * i + 1];
    cs[2 * i] = first ? re : cs[2 * i] + re;
    cs[2 * i + 1] = first ? im : cs[2 * i + 1] + im;
  }
}

/* |F|^2 accumulation over frames: s[i] += |cs[i]|^2 (code/src/mp_sqom56.f90:1381-1387). */
void oracle_abs2_accumulate(int64_t n, const double* cs, double* s) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) s[i] += cs[2 * i] * cs[2 * i] + cs[2 * i + 1] * cs[2 * i + 1];
}

/* Parallel zeroing of n doubles (also the first touch of a fresh buffer's pages). */
void oracle_zero(double* p, int64_t n) {
#pragma omp parallel for schedule(static)
  for (int64_t b = 0; b < (n + 65535) / 65536; ++b) {
    const int64_t i0 = b * 65536, m = n - i0 < 65536 ? n - i0 : 65536;
    memset(p + i0, 0, sizeof(double) * (size_t)m);
  }
}

int oracle_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
