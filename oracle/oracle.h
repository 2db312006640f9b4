/*
 * FP64 CPU oracle for the tensor-core FFT / FFT-convolution path.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the checker and the timed CPU
 * baseline. Only tests/, __graft_entry__.smoke() and bench.py (its
 * cpu_baseline leg and its --impl reference arm) may load it. The product
 * library (libtcfft_gb300.so) never links or calls it.
 *
 * What each function restates (file:line in yuelingfan/fft_demo):
 *   orc_fft1d / orc_dft1d  - the transform tcfftExec computes
 *                            (tcfft_half.cu:1177; checked there by FFTW,
 *                            main.cpp:68-80): unnormalised C2C,
 *                            X[k] = sum_n x[n] exp(sign * 2 pi i n k / N).
 *   orc_fft2d              - tcfftExec_2d (tcfft_half_2d.cu:1128; FFTW 2D
 *                            main.cpp:82-95): row-major [nx][ny], ny fastest.
 *   orc_gen_rev            - gen_rev digit-reversal permutation
 *                            (tcfft_half.cu:1351, tcfft_half_2d.cu:1227).
 *   orc_corr2d_valid       - naive_fft_conv2d_ss_sf_valid (main.cpp:97),
 *                            extended over S input channels and F filters as
 *                            fft_conv2d_half::conv2d_forward computes
 *                            (tensorcore_fft_conv2d.cpp:283).
 *   orc_conv2d_same        - 'same'-mode true 2D convolution (odd filters).
 *   orc_conv2d_full        - full linear 2D convolution, one image with
 *                            kernelCount filters (convolve_direct_fft,
 *                            fftconvolve2d.cu:184: its 1/fftSize
 *                            cancels the unnormalised C2R inverse).
 *   orc_qd_fft2d           - fast_fft's line-projection 2D DFT of box-limited
 *                            planes (fftconvolve2d.cu:1011, :884, :155).
 *   orc_clipped_error      - get_error (main.cpp:118).
 *
 * Parity pins: the FFT against the direct DFT and known-answer vectors; the
 * permutation against the reference's own gen_rev compiled from its source
 * (oracle/ref_build.sh) and the rev_256/rev_512 tables of
 * tensorcore_fft_conv2d.h:72,96.
 */
#ifndef TCFFT_ORACLE_H
#define TCFFT_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

/* In-place batched complex FFT; data = interleaved (re, im) doubles, batch
 * sequences of n points back to back. n must be a power of two. sign = -1
 * forward, +1 inverse. No normalisation. nthreads <= 0: all cores. */
void orc_fft1d(double *data, int n, long batch, int sign, int nthreads);
/* Direct O(n^2) DFT (any n), out-of-place. */
void orc_dft1d(const double *in, double *out, int n, long batch, int sign);
/* 2D FFT of batch [nx][ny] arrays (ny fastest), in place. */
void orc_fft2d(double *data, int nx, int ny, long batch, int sign, int nthreads);

/* Digit-reversal permutation for the radix list radices[0..n_radices-1]
 * (product == N): rev[i] = natural index stored at position i. */
void orc_gen_rev(int N, int *rev, const int *radices, int n_radices);

/* Valid cross-correlation: signal [S][sy][sx], filter [F][S][fy][fx],
 * out [F][sy-fy+1][sx-fx+1]. */
void orc_corr2d_valid(const double *signal, const double *filter, double *out, int S, int F,
                      int sy, int sx, int fy, int fx, int nthreads);
/* 'same' true convolution of image [n][sy][sx] with one filter [fy][fx]
 * (fy, fx odd); out [n][sy][sx], centred (offset (fy-1)/2, (fx-1)/2). */
void orc_conv2d_same(const double *img, const double *filt, double *out, int n, int sy, int sx,
                     int fy, int fx, int nthreads);
/* Full linear convolution: image [ny][nx], kernels [kc][ky][kx];
 * out [kc][ny+ky-1][nx+kx-1]. */
void orc_conv2d_full(const double *img, const double *kern, double *out, int kc, int ny, int nx,
                     int ky, int kx, int nthreads);

/* Mean over all components of min(1, |t - s| / |s|). */
/* Line-projection ("qdFFT") 2D DFT of box-limited planes (fast_fft,
 * fftconvolve2d.cu:1011): interleaved complex [count][n][n] in and out. */
void orc_qd_fft2d(const double *planes, double *out, int n, long count, int box_rows, int box_cols, int sign);

double orc_clipped_error(const double *tested, const double *standard, long count);
/* ||t - s||_2 / ||s||_2 and max |t - s| over count doubles. */
double orc_rel_l2(const double *tested, const double *standard, long count);
double orc_max_abs(const double *tested, const double *standard, long count);

int orc_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
