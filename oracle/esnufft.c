/*
 * CPU exponential-of-semicircle (ES) spreader / interpolator —
 * TEST INFRASTRUCTURE ONLY (oracle and timed CPU baseline).
 *
 * mri-nufft delegates its NUFFT arithmetic to finufft (>= 2.5.0, not vendored
 * with the reference; call sites src/mrinufft/operators/interfaces/finufft.py:
 * 43-76 and 225-232).  This file restates the published algorithm of that
 * library (Barnett, Magland & af Klinteberg, SISC 2019): a sample at fine-grid
 * coordinate u receives / contributes the kernel
 *     phi(x) = exp(beta (sqrt(1 - (2x/w)^2) - 1)),  |x| < w/2,
 * on the w cells i0 .. i0 + w - 1, i0 = ceil(u - w/2), x = i - u, with
 * periodic wrap of the fine grid.  Coordinates are radians; u = k nf / (2 pi).
 *
 * Compiled twice: REAL=double (checker) and REAL=float (CPU baseline).
 * OpenMP: interpolation is parallel over samples; spreading sorts samples into
 * slabs of axis 0 (slab width >= w) and spreads even slabs, then odd slabs,
 * in parallel, so that no two threads touch the same cell.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef REAL
#define REAL double
#endif
#define CAT2(a, b) a##b
#define CAT(a, b) CAT2(a, b)
#ifdef SUFFIX
#define FN(name) CAT(name, SUFFIX)
#else
#define FN(name) name
#endif

#define MAXW 16

static inline double fold(double k, int64_t nf) {
  double u = k * (double)nf / (2.0 * M_PI);
  u = u - (double)nf * floor(u / (double)nf);
  if (!(u >= 0.0 && u <= (double)nf)) u = 0.0;
  return u;
}

static inline void weights(double u, int w, double beta, int64_t* i0, REAL* wt) {
  double s = u - 0.5 * w;
  int64_t a = (int64_t)ceil(s);
  double x0 = (double)a - u;
  for (int t = 0; t < w; ++t) {
    double z = (x0 + t) * 2.0 / w;
    double q = 1.0 - z * z;
    wt[t] = q > 0 ? (REAL)exp(beta * (sqrt(q) - 1.0)) : (REAL)0;
  }
  *i0 = a;
}

static inline int64_t wrap(int64_t i, int64_t n) {
  int64_t r = i % n;
  return r < 0 ? r + n : r;
}

/* y[j] = sum over footprint of grid * kernel; grid/y interleaved complex. */
void FN(es_interp)(int dim, const int64_t* nf, int64_t M, const REAL* k0, const REAL* k1,
                   const REAL* k2, const REAL* grid, REAL* y, int w, double beta, int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(static)
#endif
  for (int64_t j = 0; j < M; ++j) {
    REAL w0[MAXW], w1[MAXW], w2[MAXW];
    int64_t a0, a1, a2 = 0;
    weights(fold(k0[j], nf[0]), w, beta, &a0, w0);
    weights(fold(k1[j], nf[1]), w, beta, &a1, w1);
    if (dim == 3) weights(fold(k2[j], nf[2]), w, beta, &a2, w2);
    double sr = 0, si = 0;
    if (dim == 2) {
      for (int t0 = 0; t0 < w; ++t0) {
        int64_t r = wrap(a0 + t0, nf[0]) * nf[1];
        double rr = 0, ri = 0;
        for (int t1 = 0; t1 < w; ++t1) {
          int64_t c = r + wrap(a1 + t1, nf[1]);
          rr += w1[t1] * grid[2 * c];
          ri += w1[t1] * grid[2 * c + 1];
        }
        sr += w0[t0] * rr;
        si += w0[t0] * ri;
      }
    } else {
      for (int t0 = 0; t0 < w; ++t0) {
        int64_t r0 = wrap(a0 + t0, nf[0]) * nf[1];
        for (int t1 = 0; t1 < w; ++t1) {
          int64_t r1 = (r0 + wrap(a1 + t1, nf[1])) * nf[2];
          double rr = 0, ri = 0;
          for (int t2 = 0; t2 < w; ++t2) {
            int64_t c = r1 + wrap(a2 + t2, nf[2]);
            rr += w2[t2] * grid[2 * c];
            ri += w2[t2] * grid[2 * c + 1];
          }
          double k = (double)w0[t0] * w1[t1];
          sr += k * rr;
          si += k * ri;
        }
      }
    }
    y[2 * j] = (REAL)sr;
    y[2 * j + 1] = (REAL)si;
  }
}

static void spread_one(int dim, const int64_t* nf, double u0, double u1, double u2, REAL cr,
                       REAL ci, REAL* grid, int w, double beta) {
  REAL w0[MAXW], w1[MAXW], w2[MAXW];
  int64_t a0, a1, a2 = 0;
  weights(u0, w, beta, &a0, w0);
  weights(u1, w, beta, &a1, w1);
  if (dim == 3) weights(u2, w, beta, &a2, w2);
  if (dim == 2) {
    for (int t0 = 0; t0 < w; ++t0) {
      int64_t r = wrap(a0 + t0, nf[0]) * nf[1];
      REAL vr = w0[t0] * cr, vi = w0[t0] * ci;
      for (int t1 = 0; t1 < w; ++t1) {
        int64_t c = r + wrap(a1 + t1, nf[1]);
        grid[2 * c] += w1[t1] * vr;
        grid[2 * c + 1] += w1[t1] * vi;
      }
    }
  } else {
    for (int t0 = 0; t0 < w; ++t0) {
      int64_t r0 = wrap(a0 + t0, nf[0]) * nf[1];
      for (int t1 = 0; t1 < w; ++t1) {
        int64_t r1 = (r0 + wrap(a1 + t1, nf[1])) * nf[2];
        REAL k = w0[t0] * w1[t1];
        REAL vr = k * cr, vi = k * ci;
        for (int t2 = 0; t2 < w; ++t2) {
          int64_t c = r1 + wrap(a2 + t2, nf[2]);
          grid[2 * c] += w2[t2] * vr;
          grid[2 * c + 1] += w2[t2] * vi;
        }
      }
    }
  }
}

/* grid += sum_j c_j kernel (grid is not cleared). */
void FN(es_spread)(int dim, const int64_t* nf, int64_t M, const REAL* k0, const REAL* k1,
                   const REAL* k2, const REAL* c, REAL* grid, int w, double beta, int nthreads) {
  int64_t slab = w;
  int64_t nslab = nf[0] / slab;
  if (nslab < 2 || nthreads == 1) {
    for (int64_t j = 0; j < M; ++j)
      spread_one(dim, nf, fold(k0[j], nf[0]), fold(k1[j], nf[1]), dim == 3 ? fold(k2[j], nf[2]) : 0,
                 c[2 * j], c[2 * j + 1], grid, w, beta);
    return;
  }
  if (nslab % 2) nslab -= 1; /* even number of slabs; the last one absorbs the rest */
  int64_t* cnt = (int64_t*)calloc(nslab + 1, sizeof(int64_t));
  int64_t* order = (int64_t*)malloc(sizeof(int64_t) * (M > 0 ? M : 1));
  int* sl = (int*)malloc(sizeof(int) * (M > 0 ? M : 1));
  for (int64_t j = 0; j < M; ++j) {
    int64_t f = (int64_t)floor(fold(k0[j], nf[0]));
    if (f >= nf[0]) f = nf[0] - 1;
    int64_t s = f / slab;
    if (s >= nslab) s = nslab - 1;
    sl[j] = (int)s;
    cnt[s + 1]++;
  }
  for (int64_t s = 0; s < nslab; ++s) cnt[s + 1] += cnt[s];
  int64_t* pos = (int64_t*)malloc(sizeof(int64_t) * (nslab + 1));
  memcpy(pos, cnt, sizeof(int64_t) * (nslab + 1));
  for (int64_t j = 0; j < M; ++j) order[pos[sl[j]]++] = j;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
  for (int parity = 0; parity < 2; ++parity) {
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (int64_t s = parity; s < nslab; s += 2) {
      for (int64_t q = cnt[s]; q < cnt[s + 1]; ++q) {
        int64_t j = order[q];
        spread_one(dim, nf, fold(k0[j], nf[0]), fold(k1[j], nf[1]),
                   dim == 3 ? fold(k2[j], nf[2]) : 0, c[2 * j], c[2 * j + 1], grid, w, beta);
      }
    }
  }
  free(pos);
  free(sl);
  free(order);
  free(cnt);
}
