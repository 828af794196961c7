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

/* CPU exponential-of-semicircle spreading onto an n0 x n1 x n2 periodic grid (interleaved
 * complex, x fastest, zeroed by the caller).  g: 3*nj grid coordinates already folded to
 * [0, n).  Threads own disjoint z-planes (y-rows in 2D, n2 == 1), so no two threads write the
 * same cell.  Kernel phi(z) = exp(beta (sqrt(1 - z^2) - 1)) on w cells. */
void oracle_es_spread(int dim, int64_t nj, const double* g, const double* c, int w, double beta,
                      int64_t n0, int64_t n1, int64_t n2, double* grid) {
  const int64_t nslab = dim == 3 ? n2 : n1; /* partitioned axis */
  const int ax = dim == 3 ? 2 : 1;
#pragma omp parallel
  {
    int nt = 1, tid = 0;
#ifdef _OPENMP
    nt = omp_get_num_threads();
    tid = omp_get_thread_num();
#endif
    const int64_t lo = nslab * tid / nt, hi = nslab * (tid + 1) / nt;
    double kx[32], ky[32], kz[32];
    for (int64_t j = 0; j < nj; ++j) {
      const double* gj = g + 3 * j;
      int64_t i0[3];
      for (int d = 0; d < 3; ++d) i0[d] = (int64_t)ceil(gj[d] - 0.5 * w);
      /* does the support along the partitioned axis meet [lo, hi) (periodically)? */
      int hit = 0;
      for (int a = 0; a < w && !hit; ++a) {
        int64_t cidx = (i0[ax] + a) % nslab;
        if (cidx < 0) cidx += nslab;
        if (cidx >= lo && cidx < hi) hit = 1;
      }
      if (!hit) continue;
      for (int a = 0; a < w; ++a) {
        double zx = ((double)(i0[0] + a) - gj[0]) * 2.0 / w;
        double zy = ((double)(i0[1] + a) - gj[1]) * 2.0 / w;
        double zz = ((double)(i0[2] + a) - gj[2]) * 2.0 / w;
        kx[a] = exp(beta * (sqrt(fmax(0.0, 1.0 - zx * zx)) - 1.0));
        ky[a] = exp(beta * (sqrt(fmax(0.0, 1.0 - zy * zy)) - 1.0));
        kz[a] = dim == 3 ? exp(beta * (sqrt(fmax(0.0, 1.0 - zz * zz)) - 1.0)) : 1.0;
      }
      const int wz = dim == 3 ? w : 1;
      for (int az = 0; az < wz; ++az) {
        int64_t iz = dim == 3 ? (i0[2] + az) % n2 : 0;
        if (iz < 0) iz += n2;
        if (dim == 3 && (iz < lo || iz >= hi)) continue;
        for (int ay = 0; ay < w; ++ay) {
          int64_t iy = (i0[1] + ay) % n1;
          if (iy < 0) iy += n1;
          if (dim == 2 && (iy < lo || iy >= hi)) continue;
          const double v = kz[az] * ky[ay];
          const double vr = v * c[2 * j], vi = v * c[2 * j + 1];
          double* row = grid + 2 * ((iz * n1 + iy) * n0);
          for (int axx = 0; axx < w; ++axx) {
            int64_t ix = (i0[0] + axx) % n0;
            if (ix < 0) ix += n0;
            row[2 * ix] += vr * kx[axx];
            row[2 * ix + 1] += vi * kx[axx];
          }
        }
      }
    }
  }
}

int oracle_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
