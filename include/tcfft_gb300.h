/*
 * tcfft_gb300 -- tensor-core FFT and FFT convolution for one GB300 (sm_103a).
 *
 * Thin C ABI: plain pointers, sizes and integer enums; no CUDA or C++ types.
 * Device buffers are raw device pointers; `stream` is a cudaStream_t passed as
 * void* (NULL = legacy default stream). Every call returns a tcfftStatus.
 *
 * Data formats
 *   TCFFT_FP16        interleaved complex half (re, im) = 4 bytes / element,
 *                     the format of the reference's half2 buffers.
 *   TCFFT_SPLIT_FP32  interleaved complex float (re, im) = 8 bytes / element,
 *                     computed with hi+lo FP16 operands on the tensor cores.
 *
 * Transforms are unnormalised (as the reference's); tcfft_exec's `scale`
 * multiplies every output (pass 1.0f/N for a normalised inverse).
 *
 * Entry points replace (file:line in yuelingfan/fft_demo):
 *   tcfft_plan_1d   tcfftCreate       tcfft_half.cu:1235  (plan + tables)
 *   tcfft_exec      tcfftExec         tcfft_half.cu:1177  (launch chain)
 *   tcfft_destroy   (none: the reference leaks its plans, tcfft_half.cu:1340)
 *   tcfft_plan_2d   tcfftCreate_2d    tcfft_half_2d.cu:1151
 *                   TensorCoreFFTCreate tensorcore_fft_conv2d_kernel.cu:1557
 *   tcfft_exec      tcfftExec_2d      tcfft_half_2d.cu:1128
 *                   TensorCoreFFTExec tensorcore_fft_conv2d_kernel.cu:1495,1526
 *   tcfft_exec_digitrev  tcfftExec on the digit-reversed input that setup()
 *                   prepares (tcfft_half.cu:1376-1394, gen_rev :1351)
 *   tcfft_exec_digitrev_2d  tcfftExec_2d on setup_2d()'s input
 *                   (tcfft_half_2d.cu:1128, :1253)
 */
#ifndef TCFFT_GB300_H
#define TCFFT_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum tcfftStatus {
  TCFFT_OK = 0,
  TCFFT_INVALID_SIZE = 1,   /* size not a supported power of two / too large */
  TCFFT_UNSUPPORTED = 2,    /* valid request this build cannot do */
  TCFFT_ALLOC_FAILED = 3,   /* device allocation failed */
  TCFFT_LAUNCH_FAILED = 4,  /* a CUDA launch or call failed */
  TCFFT_TIMEOUT = 5,        /* a bounded device wait gave up */
  TCFFT_CAPACITY = 6,       /* request exceeds an admission / memory cap */
  TCFFT_INVALID_VALUE = 7,  /* null pointer, bad enum, misaligned buffer */
  TCFFT_NO_DEVICE = 8       /* no usable sm_103 device */
} tcfftStatus;

typedef enum tcfftPrecision { TCFFT_FP16 = 0, TCFFT_SPLIT_FP32 = 1 } tcfftPrecision;

typedef enum tcfftDirection { TCFFT_FORWARD = -1, TCFFT_INVERSE = 1 } tcfftDirection;

typedef struct tcfftPlanImpl *tcfftPlan;

/* Batched 1D C2C plan: `batch` sequences of n points, back to back.
 * n = 2^k, 16 <= n <= 2^24. */
tcfftStatus tcfft_plan_1d(tcfftPlan *plan, long long n, long long batch, int precision);

/* Batched 2D C2C plan over [batch][nx][ny] arrays (ny contiguous).
 * nx, ny = 2^k in [16, 4096]. */
tcfftStatus tcfft_plan_2d(tcfftPlan *plan, int nx, int ny, long long batch, int precision);

/* 1D FP16 plans with 2^15 <= n <= 2^24 can run both four-step passes in
 * one persistent launch that keeps the intermediate in a small L2-resident
 * workspace ring (enable = 1; the ring is allocated on first use). The
 * default, enable = 0, is two pass launches through the plan's full-size
 * workspace. Both forms give bit-identical results. */
tcfftStatus tcfft_plan_set_fused(tcfftPlan plan, int enable);

/* Bytes of device workspace the plan holds (allocated at plan time). */
tcfftStatus tcfft_workspace_bytes(tcfftPlan plan, size_t *bytes);

/* out = scale * FFT_direction(in). in == out is allowed. Buffers must be
 * 16-byte aligned device memory. Asynchronous on `stream`. */
tcfftStatus tcfft_exec(tcfftPlan plan, const void *in, void *out, int direction, float scale,
                       void *stream);

/* Forward transform of input stored in the digit-reversed order of the
 * reference's setup() for a radix list `radices[0..n_radices-1]`
 * (product == n; n_radices == 0 means natural order). Output natural order,
 * in place allowed. 1D FP16 plans only. */
tcfftStatus tcfft_exec_digitrev(tcfftPlan plan, const void *in, void *out, const int *radices,
                                int n_radices, void *stream);

/* 2D transform (direction TCFFT_FORWARD / TCFFT_INVERSE, unnormalised) of
 * input whose rows are stored in the digit-reversed order of radices_x and
 * whose elements within a row follow radices_y, as the reference's
 * setup_2d() (tcfft_half_2d.cu:1253-1273) and fft_conv2d_half's rev tables
 * (tensorcore_fft_conv2d.h:72,96) prepare. 2D FP16 plans. */
tcfftStatus tcfft_exec_digitrev_2d(tcfftPlan plan, const void *in, void *out, const int *radices_x,
                                   int n_radices_x, const int *radices_y, int n_radices_y,
                                   int direction, void *stream);

/* Synchronise `stream` and report any error a kernel of this plan flagged
 * (e.g. TCFFT_TIMEOUT from a bounded wait). Clears the flag. */
tcfftStatus tcfft_check(tcfftPlan plan, void *stream);

tcfftStatus tcfft_destroy(tcfftPlan plan);

/* No counterpart in the reference. 1D FP16 transform without a plan and
 * without any device allocation, for callers that cannot allocate: the
 * fused four-step kernel of tcfft_exec runs with its workspace ring,
 * counters, error word and tables in one file-scope device array of 17 MiB
 * (see "First call" below). out = scale * FFT_direction(in), in == out allowed, 16-byte
 * aligned device buffers of n * batch interleaved complex halves.
 * Limits: n = 2^k with 2^15 <= n <= 2^21 (TCFFT_INVALID_SIZE below the
 * range or for other n, TCFFT_CAPACITY above it) and
 * ceil(batch / (2^21 / n)) <= 8159 (TCFFT_CAPACITY beyond that).
 * Every call on a device shares the array, so calls that overlap on the GPU
 * (other streams, unordered host threads) race; calls on one stream do not.
 * wait != 0: synchronise `stream` and report a kernel error flagged by this
 * call or by earlier calls made with wait == 0 (TCFFT_TIMEOUT), then clear
 * it; wait == 0: asynchronous, a flagged error stays recorded for the next
 * call that waits.
 * First call on each device: it sets the array up -- the CUDA runtime loads
 * the library's device code onto the device (lazy module loading, the
 * default; CUDA_MODULE_LOADING=EAGER does it at context creation instead),
 * which gives the array its device memory, then the tables are written on
 * `stream` and `stream` is synchronised once. Make that first call before
 * any stream capture and outside latency-critical code; during a capture it
 * returns TCFFT_UNSUPPORTED. A failed set-up is retried by the next call. */
tcfftStatus tcfft_exec_static(const void *in, void *out, long long n, long long batch, int direction,
                              float scale, void *stream, int wait);

/* ------------------------------------------------------------------------
 * 2D FFT convolution
 *   images  [batch][S][sy][sx] real (half for TCFFT_FP16, float for split)
 *   filters [F][S][fy][fx] float, transformed once and kept on the device
 *   out     [batch][F][oy][ox] real (same type as images)
 * Modes:
 *   TCFFT_CONV_VALID_CORR  out[f] = sum_s valid cross-correlation of image s
 *                          with filter (f, s); oy = sy-fy+1, ox = sx-fx+1.
 *                          This is fft_conv2d_half::conv2d_forward
 *                          (tensorcore_fft_conv2d.cpp:283) and
 *                          naive_fft_conv2d_ss_sf_valid (main.cpp:97).
 *   TCFFT_CONV_SAME        true convolution, centred (fy, fx odd); oy = sy,
 *                          ox = sx; S must be 1 or the channels are summed.
 *   TCFFT_CONV_FULL        full linear convolution; oy = sy+fy-1,
 *                          ox = sx+fx-1 (convolve_direct_fft family,
 *                          fftconvolve2d.cu:184, whose 1/fftSize cancels
 *                          its unnormalised C2R inverse).
 * The padded transform size P is the smallest power of two without
 * wrap-around inside the output window (P <= 4096 FP16, <= 2048 split).
 * ------------------------------------------------------------------------ */
typedef enum tcfftConvMode {
  TCFFT_CONV_VALID_CORR = 0,
  TCFFT_CONV_SAME = 1,
  TCFFT_CONV_FULL = 2
} tcfftConvMode;

typedef struct tcfftConvImpl *tcfftConv;

/* Plan for batches of up to max_batch images (device buffers are sized for it). */
tcfftStatus tcfft_conv2d_plan(tcfftConv *conv, int S, int F, int sy, int sx, int fy, int fx, int mode,
                              int precision, long long max_batch);
/* Transform and keep the filters (device float [F][S][fy][fx]). Replaces the
 * filter FFT of the fft_conv2d_half constructor (tensorcore_fft_conv2d.cpp:46-57). */
tcfftStatus tcfft_conv2d_set_filters(tcfftConv conv, const float *filters, void *stream);
/* out = conv(images) for `batch` <= max_batch images (device buffers). */
tcfftStatus tcfft_conv2d_exec(tcfftConv conv, const void *images, void *out, long long batch, void *stream);
/* Same contract as tcfft_conv2d_set_filters, with the filter spectra made by
 * line projections (tcfft_qd_* below) instead of the masked row and column
 * passes: the route convolve_turbo_fft_v3 (fftconvolve2d.cu:1263) takes to
 * its filter spectra. Results agree with tcfft_conv2d_set_filters to the
 * plan's precision. */
tcfftStatus tcfft_conv2d_set_filters_qd(tcfftConv conv, const float *filters, void *stream);
/* Output window and padded transform size of the plan. */
tcfftStatus tcfft_conv2d_shape(tcfftConv conv, int *out_rows, int *out_cols, int *padded);
/* Synchronise `stream`, report a flagged device error. */
tcfftStatus tcfft_conv2d_check(tcfftConv conv, void *stream);
tcfftStatus tcfft_conv2d_destroy(tcfftConv conv);

/* ------------------------------------------------------------------------
 * Line-projection 2D DFT ("qdFFT"; replaces fast_fft's projection, batched
 * 1D FFT and scatter, fftconvolve2d.cu:884,1011, fft_utils.cu:161-700).
 * Input: `planes` complex float planes [planes][n][n] (device) whose
 * non-zeros lie in the top-left box_rows x box_cols box (only the box is
 * read). Output: their unnormalised 2D DFTs (direction), [planes][n][n]
 * complex float, out != planes. For each of the 3n/2 directions (1, s),
 * (2q, 1) the box is projected onto lines p x + s y = t (mod n); a 1D DFT of
 * each projection gives the spectrum along one line through the origin.
 * 16 <= n <= 4096, n a power of two; FP32 data, split-precision transforms.
 * ------------------------------------------------------------------------ */
typedef struct tcfftQdImpl *tcfftQd;
tcfftStatus tcfft_qd_plan(tcfftQd *qd, int n, long long planes, int box_rows, int box_cols);
tcfftStatus tcfft_qd_exec(tcfftQd qd, const void *planes, void *out, int direction, void *stream);
/* Synchronise `stream`, report a flagged device error of the transforms. */
tcfftStatus tcfft_qd_check(tcfftQd qd, void *stream);
tcfftStatus tcfft_qd_destroy(tcfftQd qd);

/* ------------------------------------------------------------------------
 * Uneven batches: many 1D transforms of different power-of-two sizes
 * (64 <= n <= 2^20) anywhere in one input and one output buffer, run by one
 * persistent launch fed from a device work queue. No counterpart in the
 * reference, whose plans hold one size and one contiguous batch
 * (tcfft_half.cu:1235); its per-size form is TCFFT_BATCH_PER_SIZE below.
 * n[i], in_off[i], out_off[i]: size and element offsets of transform i;
 * scale: per-transform output scale (NULL = 1). Offsets must keep every
 * transform 16-byte aligned.
 * ------------------------------------------------------------------------ */
typedef struct tcfftBatchImpl *tcfftBatch;
typedef enum tcfftBatchMode {
  TCFFT_BATCH_PERSISTENT = 0,  /* one persistent launch (default) */
  TCFFT_BATCH_PER_SIZE = 1     /* plain path: one tcfft_exec per run of adjacent same-size transforms */
} tcfftBatchMode;
tcfftStatus tcfft_batch_plan(tcfftBatch *batch, int count, const long long *n, const long long *in_off,
                             const long long *out_off, const float *scale, int precision, int direction);
/* 2D convolutions in the same persistent launch (forward plans only): one
 * real sy x sx image (half for TCFFT_FP16, float for split) convolved with
 * one fy x fx float filter, tcfftConvMode semantics of tcfft_conv2d_plan,
 * padded size P <= 2048. Offsets are in elements of the conv input / output
 * buffers and of `filters` (device or host floats, filter_floats in total;
 * copied, and the spectra made, at plan time). */
typedef struct tcfftBatchConv {
  int sy, sx, fy, fx, mode;
  long long img_off, out_off, filt_off;
} tcfftBatchConv;
tcfftStatus tcfft_batch_plan_mixed(tcfftBatch *batch, int count, const long long *n, const long long *in_off,
                                   const long long *out_off, const float *scale, int nconv,
                                   const tcfftBatchConv *convs, const float *filters, long long filter_floats,
                                   int precision, int direction);
tcfftStatus tcfft_batch_set_mode(tcfftBatch batch, int mode);
/* enable != 0: tcfft_batch_exec replays a CUDA graph of its launches,
 * captured on the first call for these buffers (re-captured when they change). */
tcfftStatus tcfft_batch_set_graph(tcfftBatch batch, int enable);
tcfftStatus tcfft_batch_exec(tcfftBatch batch, const void *in, void *out, void *stream);
tcfftStatus tcfft_batch_exec_mixed(tcfftBatch batch, const void *in, void *out, const void *conv_in,
                                   void *conv_out, void *stream);
/* Work items of the persistent launch, workspace bytes, persistent CTAs. */
tcfftStatus tcfft_batch_info(tcfftBatch batch, int *items, size_t *workspace_bytes, int *ctas);
tcfftStatus tcfft_batch_check(tcfftBatch batch, void *stream);
tcfftStatus tcfft_batch_destroy(tcfftBatch batch);

/* ------------------------------------------------------------------------
 * Serving queue (no counterpart in the reference): continuous batching of
 * forward 1D FFTs (64 <= n <= 2^20) and 2D convolutions (filters from a
 * resident pool) into the persistent batch kernel.
 * Tables, the filter pool and its spectra (made per padded size on first
 * use), a workspace arena of workspace_bytes and four staging slots of
 * staging_bytes stay resident; a submit builds the work list on the host,
 * copies it with one async copy and launches once (twice when a filter
 * spectrum is new). A convolution whose own padded size would be 2048 or
 * more (an image side above ~1000) runs as overlap-add: its image is cut
 * into square blocks of side 512 - (f - 1) for an f x f filter (1024 or 2048
 * minus f - 1 when f > 129 or > 257), whose full convolutions are items of the
 * same launch padded to 512 (1024, 2048), written to workspace scratch, and
 * one more launch sums them into the requested window.
 * Submits share the workspace: one stream per queue.
 * TCFFT_CAPACITY: the submit needs more workspace or staging; split it.
 * ------------------------------------------------------------------------ */
typedef struct tcfftQueueImpl *tcfftQueue;
typedef struct tcfftQueueConv {
  int sy, sx, filter_id, mode;
  long long img_off, out_off; /* real elements in conv_in / conv_out */
} tcfftQueueConv;
tcfftStatus tcfft_queue_create(tcfftQueue *queue, int precision, size_t workspace_bytes, size_t staging_bytes);
/* Adds filter `id` (fy x fx floats, host or device; copied). */
tcfftStatus tcfft_queue_set_filter(tcfftQueue queue, int id, const float *filter, int fy, int fx);
tcfftStatus tcfft_queue_submit(tcfftQueue queue, int count, const long long *n, const long long *in_off,
                               const long long *out_off, const float *scale, int nconv,
                               const tcfftQueueConv *convs, const void *in, void *out, const void *conv_in,
                               void *conv_out, void *stream);
tcfftStatus tcfft_queue_check(tcfftQueue queue, void *stream);
tcfftStatus tcfft_queue_destroy(tcfftQueue queue);
/* Request inputs from the host: copies src[i] (bytes[i] bytes of host
 * memory, page-locked for the copy to be asynchronous) to
 * dst_base + dst_off[i] (bytes) on the device, one cudaMemcpyAsync per input
 * on `stream`, so a submit on the same stream reads them. */
tcfftStatus tcfft_copy_inputs(int count, const void *const *src, const size_t *bytes, void *dst_base,
                              const size_t *dst_off, void *stream);

/* Bound of the dependency waits inside the persistent kernels (the fused
 * four-step launch, tcfft_exec_static, the uneven-batch and serving
 * kernels): a work item waits at most `polls` polls for the items it depends
 * on, then gives up, skips its work and flags TCFFT_TIMEOUT, which the
 * plan's check call reports. Applies to launches made after the call (a CUDA
 * graph captured earlier keeps its bound). polls < 0 restores the default,
 * 2^24 (seconds); 0 makes every such wait give up at once, a deterministic
 * way to exercise the timeout path. Waits on the tensor cores and on copies
 * keep their own bound. No counterpart in the reference, whose kernels never
 * wait on one another. */
tcfftStatus tcfft_set_wait_limit(long long polls);

/* Last status returned on this thread, and a readable name for a status. */
tcfftStatus tcfft_get_last_error(void);
const char *tcfft_status_string(tcfftStatus status);

/* Number of kernel launches the last tcfft_exec* call on this thread made. */
int tcfft_last_launch_count(void);

/* ------------------------------------------------------------------------
 * Tuning (used by the autotuner, fft_demo_gb300/autotune.py)
 * A transform is a chain of passes; each pass kind has several tile
 * variants (lines per CTA tile, CTAs per SM). The tuned variant per
 * (precision, pass kind, log2 of the pass length) is process-wide state.
 * ------------------------------------------------------------------------ */
typedef enum tcfftPassKind { TCFFT_PASS_ROW = 0, TCFFT_PASS_COL = 1, TCFFT_PASS_ROWT = 2 } tcfftPassKind;
typedef enum tcfftTile {
  TCFFT_TILE_SMALL = 0,  /* 128 MMA rows per tile */
  TCFFT_TILE_BIG = 1,    /* FP16 1024 rows; split precision 512 rows */
  TCFFT_TILE_MID = 2,    /* FP16 512 rows, next tile prefetched, 3 CTAs/SM;
                            split precision 256 rows on 128 threads, 4 CTAs/SM */
  TCFFT_TILE_NARROW = 3  /* FP16 256 rows, next tile prefetched, 128 threads,
                            6 CTAs/SM */
} tcfftTile;
/* tile = -1 restores the built-in choice. tcfft_tune_set: every launch of
 * the pass uses that variant. tcfft_tune_prefer (a tuning file's choice,
 * measured on batches that fill the GPU): the same, except that an FP16
 * batch the variant would spread over fewer than two tiles per SM takes
 * the smaller narrow tiles. */
tcfftStatus tcfft_tune_set(int precision, int pass_kind, int log2_len, int tile);
tcfftStatus tcfft_tune_prefer(int precision, int pass_kind, int log2_len, int tile);
tcfftStatus tcfft_tune_get(int precision, int pass_kind, int log2_len, int *tile);
/* Four-step split for 1D plans of 2^log2_n points made after this call:
 * column passes of 2^log2_n1 points, then transposing passes of
 * 2^(log2_n - log2_n1); -1 restores the built-in choice. TCFFT_UNSUPPORTED
 * when either pass length has no kernel. */
tcfftStatus tcfft_tune_split(int precision, int log2_n, int log2_n1);
/* Geometry of a pass variant: lines per tile, co-resident CTAs per SM, SMs. */
tcfftStatus tcfft_pass_info(int precision, int pass_kind, int log2_len, int tile, int *lines_per_tile,
                            int *ctas_per_sm, int *num_sms);

#ifdef __cplusplus
}
#endif
#endif /* TCFFT_GB300_H */
