/*
 * FP64 CPU oracle (test infrastructure only; see oracle.h for what each
 * function restates and who may call it).
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

static int ilog2i(long n) {
  int l = 0;
  while ((1L << l) < n) ++l;
  return l;
}

/* exp(-2 pi i k / n) for k < n/2, with the angle reduced by octant symmetry
 * so every entry is accurate to ~1 ulp. */
static void make_twiddles(double *tw, int n) {
  for (int k = 0; k < n / 2; ++k) {
    double a = 2.0 * M_PI * (double)k / (double)n;
    tw[2 * k] = cos(a);
    tw[2 * k + 1] = -sin(a);
  }
  /* exact values at the quarter points */
  if (n >= 4) {
    tw[2 * (n / 4)] = 0.0;
    tw[2 * (n / 4) + 1] = -1.0;
  }
}

/* Iterative radix-2 decimation-in-time FFT on one sequence. */
static void fft_one(double *x, int n, const double *tw, const int *br, int sign) {
  for (int i = 0; i < n; ++i) {
    int j = br[i];
    if (j > i) {
      double tr = x[2 * i], ti = x[2 * i + 1];
      x[2 * i] = x[2 * j];
      x[2 * i + 1] = x[2 * j + 1];
      x[2 * j] = tr;
      x[2 * j + 1] = ti;
    }
  }
  for (int len = 2; len <= n; len <<= 1) {
    int half = len >> 1;
    int step = n / len;
    for (int base = 0; base < n; base += len) {
      for (int j = 0; j < half; ++j) {
        double wr = tw[2 * j * step];
        double wi = sign < 0 ? tw[2 * j * step + 1] : -tw[2 * j * step + 1];
        double *a = x + 2 * (base + j);
        double *b = x + 2 * (base + j + half);
        double vr = b[0] * wr - b[1] * wi;
        double vi = b[0] * wi + b[1] * wr;
        b[0] = a[0] - vr;
        b[1] = a[1] - vi;
        a[0] += vr;
        a[1] += vi;
      }
    }
  }
}

static int *make_bitrev(int n) {
  int l = ilog2i(n);
  int *br = (int *)malloc(sizeof(int) * (size_t)n);
  for (int i = 0; i < n; ++i) {
    int r = 0;
    for (int b = 0; b < l; ++b)
      if (i & (1 << b)) r |= 1 << (l - 1 - b);
    br[i] = r;
  }
  return br;
}

void orc_fft1d(double *data, int n, long batch, int sign, int nthreads) {
  if (n <= 1 || batch <= 0) return;
  double *tw = (double *)malloc(sizeof(double) * (size_t)n);
  make_twiddles(tw, n);
  int *br = make_bitrev(n);
#ifdef _OPENMP
  int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
#endif
  for (long b = 0; b < batch; ++b) fft_one(data + 2 * (size_t)n * (size_t)b, n, tw, br, sign);
  (void)nthreads;
  free(br);
  free(tw);
}

void orc_dft1d(const double *in, double *out, int n, long batch, int sign) {
  for (long b = 0; b < batch; ++b) {
    const double *x = in + 2 * (size_t)n * (size_t)b;
    double *y = out + 2 * (size_t)n * (size_t)b;
    for (int k = 0; k < n; ++k) {
      double sr = 0, si = 0;
      for (int j = 0; j < n; ++j) {
        /* reduce n*k mod N exactly before forming the angle */
        long e = ((long)j * (long)k) % n;
        double a = (double)sign * 2.0 * M_PI * (double)e / (double)n;
        double c = cos(a), s = sin(a);
        sr += x[2 * j] * c - x[2 * j + 1] * s;
        si += x[2 * j] * s + x[2 * j + 1] * c;
      }
      y[2 * k] = sr;
      y[2 * k + 1] = si;
    }
  }
}

void orc_fft2d(double *data, int nx, int ny, long batch, int sign, int nthreads) {
  /* rows (length ny, contiguous) */
  orc_fft1d(data, ny, batch * (long)nx, sign, nthreads);
  /* columns (length nx, stride ny) */
  double *tw = (double *)malloc(sizeof(double) * (size_t)nx);
  make_twiddles(tw, nx);
  int *br = make_bitrev(nx);
#ifdef _OPENMP
  int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel num_threads(nt)
#endif
  {
    double *col = (double *)malloc(sizeof(double) * 2 * (size_t)nx);
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
    for (long t = 0; t < batch * (long)ny; ++t) {
      long b = t / ny;
      int c = (int)(t % ny);
      double *base = data + 2 * (size_t)nx * (size_t)ny * (size_t)b;
      for (int r = 0; r < nx; ++r) {
        col[2 * r] = base[2 * ((size_t)r * ny + c)];
        col[2 * r + 1] = base[2 * ((size_t)r * ny + c) + 1];
      }
      fft_one(col, nx, tw, br, sign);
      for (int r = 0; r < nx; ++r) {
        base[2 * ((size_t)r * ny + c)] = col[2 * r];
        base[2 * ((size_t)r * ny + c) + 1] = col[2 * r + 1];
      }
    }
    free(col);
  }
  (void)nthreads;
  free(br);
  free(tw);
}

/* The reference builds the permutation by repeatedly transposing blocks
 * (tcfft_half.cu:1351). Closed form used here: peel the index's digits from
 * the last radix to the first; the digit peeled k-th (0-based) becomes the
 * k-th most significant digit of the storage position. */
void orc_gen_rev(int N, int *rev, const int *radices, int n_radices) {
  for (int idx = 0; idx < N; ++idx) {
    int rest = idx;
    int pos = 0;
    int span = N;
    for (int i = n_radices - 1; i >= 0; --i) {
      int r = radices[i];
      int d = rest % r;
      rest /= r;
      span /= r;
      pos += d * span;
    }
    rev[pos] = idx;
  }
}

void orc_corr2d_valid(const double *signal, const double *filter, double *out, int S, int F,
                      int sy, int sx, int fy, int fx, int nthreads) {
  int oy = sy - fy + 1, ox = sx - fx + 1;
#ifdef _OPENMP
  int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel for collapse(2) schedule(static) num_threads(nt)
#endif
  for (int f = 0; f < F; ++f)
    for (int i = 0; i < oy; ++i)
      for (int j = 0; j < ox; ++j) {
        double acc = 0.0;
        for (int s = 0; s < S; ++s) {
          const double *w = filter + ((size_t)f * S + s) * (size_t)fy * fx;
          const double *x = signal + (size_t)s * sy * sx;
          for (int k = 0; k < fy; ++k)
            for (int l = 0; l < fx; ++l) acc += w[k * fx + l] * x[(size_t)(i + k) * sx + j + l];
        }
        out[((size_t)f * oy + i) * ox + j] = acc;
      }
  (void)nthreads;
}

void orc_conv2d_same(const double *img, const double *filt, double *out, int n, int sy, int sx,
                     int fy, int fx, int nthreads) {
  int cy = (fy - 1) / 2, cx = (fx - 1) / 2;
#ifdef _OPENMP
  int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel for collapse(2) schedule(static) num_threads(nt)
#endif
  for (int b = 0; b < n; ++b)
    for (int i = 0; i < sy; ++i) {
      const double *x = img + (size_t)b * sy * sx;
      for (int j = 0; j < sx; ++j) {
        double acc = 0.0;
        for (int a = 0; a < fy; ++a) {
          int yy = i + cy - a;
          if (yy < 0 || yy >= sy) continue;
          for (int c = 0; c < fx; ++c) {
            int xx = j + cx - c;
            if (xx < 0 || xx >= sx) continue;
            acc += filt[a * fx + c] * x[(size_t)yy * sx + xx];
          }
        }
        out[((size_t)b * sy + i) * sx + j] = acc;
      }
    }
  (void)nthreads;
}

void orc_conv2d_full(const double *img, const double *kern, double *out, int kc, int ny, int nx,
                     int ky, int kx, int nthreads) {
  int oy = ny + ky - 1, ox = nx + kx - 1;
#ifdef _OPENMP
  int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel for collapse(2) schedule(static) num_threads(nt)
#endif
  for (int k = 0; k < kc; ++k)
    for (int y = 0; y < oy; ++y) {
      const double *w = kern + (size_t)k * ky * kx;
      for (int x = 0; x < ox; ++x) {
        double acc = 0.0;
        for (int a = 0; a < ky; ++a) {
          int yy = y - a;
          if (yy < 0 || yy >= ny) continue;
          for (int b = 0; b < kx; ++b) {
            int xx = x - b;
            if (xx < 0 || xx >= nx) continue;
            acc += w[a * kx + b] * img[(size_t)yy * nx + xx];
          }
        }
        out[((size_t)k * oy + y) * ox + x] = acc;
      }
    }
  (void)nthreads;
}

double orc_clipped_error(const double *tested, const double *standard, long count) {
  double err = 0.0;
  for (long i = 0; i < count; ++i) {
    double d = fabs((tested[i] - standard[i]) / standard[i]);
    /* 0/0 is NaN; the reference's std::min(1.0, NaN) returns 1.0 */
    err += (d < 1.0) ? d : 1.0;
  }
  return count > 0 ? err / (double)count : 0.0;
}

double orc_rel_l2(const double *tested, const double *standard, long count) {
  double num = 0.0, den = 0.0;
  for (long i = 0; i < count; ++i) {
    double d = tested[i] - standard[i];
    num += d * d;
    den += standard[i] * standard[i];
  }
  return den > 0.0 ? sqrt(num / den) : sqrt(num);
}

double orc_max_abs(const double *tested, const double *standard, long count) {
  double m = 0.0;
  for (long i = 0; i < count; ++i) {
    double d = fabs(tested[i] - standard[i]);
    if (d > m) m = d;
  }
  return m;
}

/* Line-projection 2D DFT of n x n complex planes whose non-zeros lie in the
 * top-left box_rows x box_cols box, as the reference computes filter spectra
 * in fast_fft (fftconvolve2d.cu:1011-1260; find_input_index :155,
 * qdVector_construct :884, scatter qdVectorReconstruct fft_utils.cu:587):
 * directions (p, s) = (1, i) for i < n and (2(i - n), 1) for n <= i < 3n/2;
 * projection v[t] = sum of the box entries with p x + s y = t (mod n); its
 * 1D DFT (sign) is written to frequency (t p mod n, t s mod n), in the
 * reference's order (direction-major, later lines overwrite earlier ones). */
void orc_qd_fft2d(const double *planes, double *out, int n, long count, int box_rows, int box_cols, int sign) {
  const int ndir = n + n / 2;
  double *v = (double *)malloc(sizeof(double) * 2 * (size_t)n);
  double *w = (double *)malloc(sizeof(double) * 2 * (size_t)n);
  for (long g = 0; g < count; ++g) {
    const double *pl = planes + (size_t)g * 2 * n * n;
    double *o = out + (size_t)g * 2 * n * n;
    for (int i = 0; i < ndir; ++i) {
      const long p = i < n ? 1 : 2L * (i - n), s = i < n ? i : 1;
      for (int t = 0; t < 2 * n; ++t) v[t] = 0.0;
      for (int x = 0; x < box_rows; ++x)
        for (int y = 0; y < box_cols; ++y) {
          const long t = (p * x + s * y) % n;
          v[2 * t] += pl[2 * ((size_t)x * n + y)];
          v[2 * t + 1] += pl[2 * ((size_t)x * n + y) + 1];
        }
      for (int t = 0; t < 2 * n; ++t) w[t] = v[t];
      orc_fft1d(w, n, 1, sign, 1);
      for (int t = 0; t < n; ++t) {
        const long u = (t * p) % n, vv = (t * s) % n;
        o[2 * (u * n + vv)] = w[2 * t];
        o[2 * (u * n + vv) + 1] = w[2 * t + 1];
      }
    }
  }
  free(v);
  free(w);
}
