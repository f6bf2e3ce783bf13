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
 *
 * Organisation, after the same paper: the samples are counting-sorted into
 * bins of 16^3 (2D: 32^2) fine cells.  Interpolation runs over the sorted
 * order in parallel (the kernel weights are evaluated once per sample and
 * axis, and the wrapped cell indices once per axis).  Spreading runs bin by
 * bin: a bin with many samples spreads into a private padded subgrid of
 * (16 + w + 2)^3 cells, which is then added into the fine grid; a bin with
 * few samples spreads straight into the fine grid.  Bins are coloured by the
 * parity of their index along each axis; on an axis with an odd bin count or
 * a short last bin the last two bins take colours of their own (the periodic
 * wrap brings the first bin next to them).  The padded regions of bins of one
 * colour do not overlap (bin size >= w + 2), so each colour is one parallel
 * loop without atomics, and the summation order of every cell depends only
 * on the bins and the sort, not on the number of threads.
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

/* the float build (CPU baseline) evaluates the kernel in float, like the
   single-precision library; the double build (checker) in double */
#ifdef REAL_IS_FLOAT
#define EXPR expf
#define SQRTR sqrtf
#else
#define EXPR exp
#define SQRTR sqrt
#endif

#define MAXW 16
#define BIN3 16 /* bin size in cells (at least w + 2) */
#define BIN2 32
#define DENSE 64 /* samples from which a bin spreads through a subgrid */

static inline double fold(double k, int64_t nf) {
  double u = k * (double)nf / (2.0 * M_PI);
  u = u - (double)nf * floor(u / (double)nf);
  if (!(u >= 0.0 && u <= (double)nf)) u = 0.0;
  return u;
}

#ifdef REAL_IS_FLOAT
/* The float build evaluates the kernel from a piecewise polynomial, as the
 * single-precision library does: cell t of a footprint sees
 * phi(s - w/2 + t) with s = x0 + w/2 in [0, 1), which is interpolated at
 * NPOLY Chebyshev nodes of [0, 1) and stored as a power series in 2s - 1
 * (double coefficients, Horner in double).  Interior cells fit to ~1e-11,
 * the two edge cells to ~1.5e-7 (the square-root edge of the support). */
#define NPOLY(w) ((w) + 4)
typedef struct {
  int n;
  double c[MAXW][MAXW + 5];
} Poly;

static void poly_fit(int w, double beta, Poly* P) {
  const int n = NPOLY(w) > MAXW + 4 ? MAXW + 4 : NPOLY(w);
  P->n = n;
  double xk[MAXW + 5], tk[MAXW + 5][MAXW + 5];
  for (int k = 0; k < n; ++k) xk[k] = cos(M_PI * (k + 0.5) / n);
  for (int t = 0; t < w; ++t) {
    double f[MAXW + 5], ch[MAXW + 5];
    for (int k = 0; k < n; ++k) {
      const double z = ((0.5 * (xk[k] + 1.0)) - 0.5 * w + t) * 2.0 / w;
      const double q = 1.0 - z * z;
      f[k] = q > 0 ? exp(beta * (sqrt(q) - 1.0)) : 0.0;
    }
    for (int j = 0; j < n; ++j) { /* Chebyshev coefficients at the nodes */
      double a = 0;
      for (int k = 0; k < n; ++k) a += f[k] * cos(M_PI * j * (k + 0.5) / n);
      ch[j] = (j == 0 ? 1.0 : 2.0) * a / n;
    }
    /* power series: T_0 = 1, T_1 = x, T_{j+1} = 2 x T_j - T_{j-1} */
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) tk[j][i] = 0;
    tk[0][0] = 1;
    if (n > 1) tk[1][1] = 1;
    for (int j = 1; j + 1 < n; ++j)
      for (int i = 0; i < n; ++i)
        tk[j + 1][i] = (i > 0 ? 2 * tk[j][i - 1] : 0) - tk[j - 1][i];
    for (int i = 0; i < n; ++i) {
      double a = 0;
      for (int j = 0; j < n; ++j) a += ch[j] * tk[j][i];
      P->c[t][i] = a;
    }
  }
}

static inline void weights_poly(double u, int w, const Poly* P, int64_t* i0, REAL* wt) {
  const double s = u - 0.5 * w;
  const int64_t a = (int64_t)ceil(s);
  const double x = 2.0 * ((double)a - u + 0.5 * w) - 1.0;
  for (int t = 0; t < w; ++t) {
    double v = P->c[t][P->n - 1];
    for (int i = P->n - 2; i >= 0; --i) v = v * x + P->c[t][i];
    wt[t] = (REAL)v;
  }
  *i0 = a;
}
#define WEIGHTS(u, w, beta, i0, wt) weights_poly((u), (w), &poly, (i0), (wt))
#define POLY_SETUP(w, beta) \
  Poly poly;                \
  poly_fit((w), (beta), &poly)
#else
#define WEIGHTS(u, w, beta, i0, wt) weights((u), (w), (beta), (i0), (wt))
#define POLY_SETUP(w, beta) (void)0
#endif

static inline void weights(double u, int w, double beta, int64_t* i0, REAL* wt) {
  double s = u - 0.5 * w;
  int64_t a = (int64_t)ceil(s);
  const REAL x0 = (REAL)((double)a - u), inv = (REAL)(2.0 / w), b = (REAL)beta;
  for (int t = 0; t < w; ++t) {
    const REAL z = (x0 + (REAL)t) * inv;
    const REAL q = (REAL)1 - z * z;
    wt[t] = q > 0 ? EXPR(b * (SQRTR(q) - (REAL)1)) : (REAL)0;
  }
  *i0 = a;
}

static inline int64_t wrap(int64_t i, int64_t n) {
  if (i >= 0 && i < n) return i;
  int64_t r = i % n;
  return r < 0 ? r + n : r;
}

/* wrapped cell indices a .. a + w - 1 of one axis; returns 1 if contiguous */
static inline int axis_cells(int64_t a, int w, int64_t n, int64_t* out) {
  int contiguous = a >= 0 && a + w <= n;
  for (int t = 0; t < w; ++t) out[t] = contiguous ? a + t : wrap(a + t, n);
  return contiguous;
}

/* Counting sort of the samples into bins; fills order[M] and start[nbins + 1]
 * (bins numbered with axis 0 slowest), returns the bin count. */
static int64_t bin_sort(int dim, const int64_t* nf, int64_t M, const REAL* k0, const REAL* k1,
                        const REAL* k2, int64_t bs, int64_t* nb, int64_t** order_out,
                        int64_t** start_out) {
  int64_t nbins = 1;
  for (int d = 0; d < 3; ++d) {
    nb[d] = d < dim ? (nf[d] + bs - 1) / bs : 1;
    nbins *= nb[d];
  }
  int64_t* bin = (int64_t*)malloc(sizeof(int64_t) * (M > 0 ? M : 1));
  int64_t* start = (int64_t*)calloc(nbins + 1, sizeof(int64_t));
  int64_t* order = (int64_t*)malloc(sizeof(int64_t) * (M > 0 ? M : 1));
  const REAL* k[3] = {k0, k1, k2};
  for (int64_t j = 0; j < M; ++j) {
    int64_t b = 0;
    for (int d = 0; d < dim; ++d) {
      int64_t c = (int64_t)floor(fold(k[d][j], nf[d])) / bs;
      if (c >= nb[d]) c = nb[d] - 1;
      b = b * nb[d] + c;
    }
    bin[j] = b;
    start[b + 1]++;
  }
  for (int64_t b = 0; b < nbins; ++b) start[b + 1] += start[b];
  int64_t* pos = (int64_t*)malloc(sizeof(int64_t) * (nbins + 1));
  memcpy(pos, start, sizeof(int64_t) * (nbins + 1));
  for (int64_t j = 0; j < M; ++j) order[pos[bin[j]]++] = j;
  free(pos);
  free(bin);
  *order_out = order;
  *start_out = start;
  return nbins;
}

/* y[j] = sum over footprint of grid * kernel; grid/y interleaved complex. */
void FN(es_interp)(int dim, const int64_t* nf, int64_t M, const REAL* k0, const REAL* k1,
                   const REAL* k2, const REAL* grid, REAL* y, int w, double beta, int nthreads) {
  int64_t nb[3], *order, *start;
  bin_sort(dim, nf, M, k0, k1, k2, dim == 3 ? BIN3 : BIN2, nb, &order, &start);
  free(start);
  POLY_SETUP(w, beta);
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1024)
#endif
  for (int64_t q = 0; q < M; ++q) {
    const int64_t j = order[q];
    REAL w0[MAXW], w1[MAXW], w2[MAXW];
    int64_t a0, a1, a2 = 0, c0[MAXW], c1[MAXW], c2[MAXW];
    WEIGHTS(fold(k0[j], nf[0]), w, beta, &a0, w0);
    WEIGHTS(fold(k1[j], nf[1]), w, beta, &a1, w1);
    axis_cells(a0, w, nf[0], c0);
    int cont1 = axis_cells(a1, w, nf[1], c1);
    double sr = 0, si = 0;
    if (dim == 2) {
      for (int t0 = 0; t0 < w; ++t0) {
        const REAL* row = grid + 2 * c0[t0] * nf[1];
        REAL rr = 0, ri = 0;
        if (cont1) {
          const REAL* p = row + 2 * a1;
          for (int t1 = 0; t1 < w; ++t1) {
            rr += w1[t1] * p[2 * t1];
            ri += w1[t1] * p[2 * t1 + 1];
          }
        } else {
          for (int t1 = 0; t1 < w; ++t1) {
            rr += w1[t1] * row[2 * c1[t1]];
            ri += w1[t1] * row[2 * c1[t1] + 1];
          }
        }
        sr += w0[t0] * rr;
        si += w0[t0] * ri;
      }
    } else {
      WEIGHTS(fold(k2[j], nf[2]), w, beta, &a2, w2);
      int cont2 = axis_cells(a2, w, nf[2], c2);
      if (cont2) {
        /* rows of 2w contiguous values: v = sum over (t0, t1) of w0 w1 row,
           then the z weights once */
        REAL v[2 * MAXW];
        for (int i = 0; i < 2 * w; ++i) v[i] = 0;
        for (int t0 = 0; t0 < w; ++t0) {
          const int64_t r0 = c0[t0] * nf[1];
          for (int t1 = 0; t1 < w; ++t1) {
            const REAL* p = grid + 2 * ((r0 + c1[t1]) * nf[2] + a2);
            const REAL k = w0[t0] * w1[t1];
            for (int i = 0; i < 2 * w; ++i) v[i] += k * p[i];
          }
        }
        for (int t2 = 0; t2 < w; ++t2) {
          sr += (double)w2[t2] * v[2 * t2];
          si += (double)w2[t2] * v[2 * t2 + 1];
        }
      } else {
        for (int t0 = 0; t0 < w; ++t0) {
          const int64_t r0 = c0[t0] * nf[1];
          for (int t1 = 0; t1 < w; ++t1) {
            const REAL* row = grid + 2 * (r0 + c1[t1]) * nf[2];
            REAL rr = 0, ri = 0;
            for (int t2 = 0; t2 < w; ++t2) {
              rr += w2[t2] * row[2 * c2[t2]];
              ri += w2[t2] * row[2 * c2[t2] + 1];
            }
            double k = (double)w0[t0] * w1[t1];
            sr += k * rr;
            si += k * ri;
          }
        }
      }
    }
    y[2 * j] = (REAL)sr;
    y[2 * j + 1] = (REAL)si;
  }
  free(order);
}

/* One sample into a grid of extent n[0..2] (cell indices from the wrapped
 * per-axis tables c0, c1, c2; c2 unused in 2D). */
static inline void spread_cells(int dim, const int64_t* n, const int64_t* c0, const int64_t* c1,
                                const int64_t* c2, const REAL* w0, const REAL* w1, const REAL* w2,
                                REAL cr, REAL ci, REAL* g, int w) {
  if (dim == 2) {
    for (int t0 = 0; t0 < w; ++t0) {
      REAL* row = g + 2 * c0[t0] * n[1];
      REAL vr = w0[t0] * cr, vi = w0[t0] * ci;
      for (int t1 = 0; t1 < w; ++t1) {
        row[2 * c1[t1]] += w1[t1] * vr;
        row[2 * c1[t1] + 1] += w1[t1] * vi;
      }
    }
  } else if (c2[w - 1] == c2[0] + w - 1) {
    /* contiguous rows: z weights times the strength once (2w values), then
       one 2w-wide update per (t0, t1) row */
    REAL zc[2 * MAXW];
    for (int t2 = 0; t2 < w; ++t2) {
      zc[2 * t2] = w2[t2] * cr;
      zc[2 * t2 + 1] = w2[t2] * ci;
    }
    for (int t0 = 0; t0 < w; ++t0) {
      const int64_t r0 = c0[t0] * n[1];
      for (int t1 = 0; t1 < w; ++t1) {
        REAL* p = g + 2 * ((r0 + c1[t1]) * n[2] + c2[0]);
        const REAL k = w0[t0] * w1[t1];
        for (int i = 0; i < 2 * w; ++i) p[i] += k * zc[i];
      }
    }
  } else {
    for (int t0 = 0; t0 < w; ++t0) {
      const int64_t r0 = c0[t0] * n[1];
      for (int t1 = 0; t1 < w; ++t1) {
        REAL* row = g + 2 * (r0 + c1[t1]) * n[2];
        REAL k = w0[t0] * w1[t1];
        REAL vr = k * cr, vi = k * ci;
        for (int t2 = 0; t2 < w; ++t2) {
          row[2 * c2[t2]] += w2[t2] * vr;
          row[2 * c2[t2] + 1] += w2[t2] * vi;
        }
      }
    }
  }
}

/* colours along an axis of nb bins (the last one possibly short) */
static inline int colours(int64_t nb, int full) {
  if (nb == 1) return 1;
  return nb % 2 == 0 && full ? 2 : 4;
}
static inline int colour(int64_t b, int64_t nb, int ncol) {
  if (ncol == 1) return 0;
  if (ncol == 2 || b < nb - 2) return (int)(b % 2);
  return b == nb - 2 ? 2 : 3;
}

/* grid += sum_j c_j kernel (grid is not cleared). */
void FN(es_spread)(int dim, const int64_t* nf, int64_t M, const REAL* k0, const REAL* k1,
                   const REAL* k2, const REAL* c, REAL* grid, int w, double beta, int nthreads) {
  int64_t bs = dim == 3 ? BIN3 : BIN2;
  if (bs < w + 2) bs = w + 2;
  POLY_SETUP(w, beta);
  int64_t nb[3], *order, *start;
  const int64_t nbins = bin_sort(dim, nf, M, k0, k1, k2, bs, nb, &order, &start);
  /* padded subgrid: bin origin - (w + 1) / 2, extent bs + w + 2 per spread axis */
  const int64_t pad = (w + 1) / 2;
  int64_t ln[3];
  int64_t lcells = 1;
  for (int d = 0; d < 3; ++d) {
    ln[d] = d < dim ? bs + w + 2 : 1;
    lcells *= ln[d];
  }
  int ncol[3];
  for (int d = 0; d < 3; ++d) ncol[d] = d < dim ? colours(nb[d], nf[d] % bs == 0) : 1;
  int nt = 1;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
  nt = omp_get_max_threads();
#endif
  REAL** sub = (REAL**)calloc(nt, sizeof(REAL*));
  for (int col0 = 0; col0 < ncol[0]; ++col0)
    for (int col1 = 0; col1 < ncol[1]; ++col1)
      for (int col2 = 0; col2 < ncol[2]; ++col2) {
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1)
#endif
        for (int64_t b = 0; b < nbins; ++b) {
          const int64_t n = start[b + 1] - start[b];
          if (n == 0) continue;
          int64_t bi[3];
          {
            int64_t r = b;
            for (int d = 2; d >= 0; --d) {
              bi[d] = r % nb[d];
              r /= nb[d];
            }
          }
          if (colour(bi[0], nb[0], ncol[0]) != col0 || colour(bi[1], nb[1], ncol[1]) != col1 ||
              colour(bi[2], nb[2], ncol[2]) != col2)
            continue;
          int tid = 0;
#ifdef _OPENMP
          tid = omp_get_thread_num();
#endif
          REAL w0[MAXW], w1[MAXW], w2[MAXW];
          int64_t a[3] = {0, 0, 0}, c0[MAXW], c1[MAXW], c2[MAXW] = {0};
          if (n < DENSE) { /* straight into the fine grid */
            for (int64_t q = start[b]; q < start[b + 1]; ++q) {
              const int64_t j = order[q];
              WEIGHTS(fold(k0[j], nf[0]), w, beta, &a[0], w0);
              WEIGHTS(fold(k1[j], nf[1]), w, beta, &a[1], w1);
              axis_cells(a[0], w, nf[0], c0);
              axis_cells(a[1], w, nf[1], c1);
              if (dim == 3) {
                WEIGHTS(fold(k2[j], nf[2]), w, beta, &a[2], w2);
                axis_cells(a[2], w, nf[2], c2);
              }
              spread_cells(dim, nf, c0, c1, c2, w0, w1, w2, c[2 * j], c[2 * j + 1], grid, w);
            }
            continue;
          }
          /* through the padded subgrid of the bin */
          if (!sub[tid]) sub[tid] = (REAL*)malloc(sizeof(REAL) * 2 * lcells);
          REAL* s = sub[tid];
          memset(s, 0, sizeof(REAL) * 2 * lcells);
          int64_t o[3], e[3]; /* subgrid origin and the extent the bin can reach */
          for (int d = 0; d < 3; ++d) {
            o[d] = d < dim ? bi[d] * bs - pad : 0;
            const int64_t len = nf[d] - bi[d] * bs < bs ? nf[d] - bi[d] * bs : bs;
            e[d] = d < dim ? len + w + 2 : 1;
          }
          for (int64_t q = start[b]; q < start[b + 1]; ++q) {
            const int64_t j = order[q];
            WEIGHTS(fold(k0[j], nf[0]), w, beta, &a[0], w0);
            WEIGHTS(fold(k1[j], nf[1]), w, beta, &a[1], w1);
            for (int t = 0; t < w; ++t) {
              c0[t] = a[0] - o[0] + t;
              c1[t] = a[1] - o[1] + t;
            }
            if (dim == 3) {
              WEIGHTS(fold(k2[j], nf[2]), w, beta, &a[2], w2);
              for (int t = 0; t < w; ++t) c2[t] = a[2] - o[2] + t;
            }
            spread_cells(dim, ln, c0, c1, c2, w0, w1, w2, c[2 * j], c[2 * j + 1], s, w);
          }
          /* add the subgrid into the fine grid */
          for (int64_t l0 = 0; l0 < e[0]; ++l0) {
            const int64_t g0 = wrap(o[0] + l0, nf[0]);
            for (int64_t l1 = 0; l1 < e[1]; ++l1) {
              const int64_t g1 = wrap(o[1] + l1, nf[1]);
              const REAL* src = s + 2 * (l0 * ln[1] + l1) * ln[2];
              REAL* dst = grid + 2 * (g0 * nf[1] + g1) * (dim == 3 ? nf[2] : 1);
              if (dim == 2) {
                dst[0] += src[0];
                dst[1] += src[1];
                continue;
              }
              for (int64_t l2 = 0; l2 < e[2]; ++l2) {
                const int64_t g2 = wrap(o[2] + l2, nf[2]);
                dst[2 * g2] += src[2 * l2];
                dst[2 * g2 + 1] += src[2 * l2 + 1];
              }
            }
          }
        }
      }
  for (int t = 0; t < nt; ++t) free(sub[t]);
  free(sub);
  free(order);
  free(start);
}
