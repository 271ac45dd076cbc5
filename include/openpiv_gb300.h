/* openpiv_gb300.h -- C ABI of the GB300 (sm_103a) PIV window-correlation path.
 *
 * Drop-in for the per-window hot loop of OpenPIV-c++ (examples/process/
 * main.cpp:189-237): every interrogation window of an image pair is
 * extracted, correlated (FFT::cross_correlate or FFT::cross_correlate_real),
 * peak-searched (core::find_peaks, 2 peaks, radius 1), Gaussian-fitted
 * (core::fit_simple_gaussian) and turned into a vector {x, y, u, v, sn}
 * exactly as that loop does, by hand-written CUDA kernels on one GPU.
 *
 * Plain C: pointers, sizes and status codes only.  The caller owns every
 * buffer passed in; a plan owns its device scratch.  No function keeps a
 * pointer passed to it after it returns, except where a stream is given
 * (the device-buffer calls are asynchronous on that stream).
 *
 * Status codes mirror the exceptions the reference throws; the message of
 * the last failure on the calling thread is returned by opiv_last_error().
 */
#ifndef OPENPIV_GB300_H
#define OPENPIV_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------- */
enum {
    OPIV_OK = 0,
    OPIV_ERR_OFFSET_RANGE = -1,   /* "offsets must be between 0.0 and 1.0"      grid.impl.h:14-15 */
    OPIV_ERR_IMAGE_EMPTY = -2,    /* "image size must be non-zero"              grid.impl.h:29-30 */
    OPIV_ERR_IA_EMPTY = -3,       /* "interrogation size must be non-zero"      grid.impl.h:32-33 */
    OPIV_ERR_OFFSET_ZERO = -4,    /* "offsets must be non-zero"                 grid.impl.h:35-36 */
    OPIV_ERR_IA_TOO_BIG = -5,     /* "interrogation size is bigger than image"  grid.impl.h:38-40 */
    OPIV_ERR_NOT_POW2 = -6,       /* "dimensions must be power of 2"            fft.h:81-83 */
    OPIV_ERR_CAPACITY = -7,       /* output buffer too small */
    OPIV_ERR_RECT_OUTSIDE = -8,   /* "extract: rectangle to extract is too large for image"
                                     image_utils.impl.h:396-401 */
    OPIV_ERR_ARG = -9,            /* invalid argument (null pointer, bad enum) */
    OPIV_ERR_SIZE_MISMATCH = -10, /* "image size is different from expected"    fft.h:94-98, :136-141 */
    OPIV_ERR_UNSUPPORTED = -11,   /* window size this build has no kernel for */
    OPIV_ERR_CUDA = -12,          /* a CUDA runtime call failed */
    OPIV_ERR_NO_DEVICE = -13,     /* no CUDA device */
    OPIV_ERR_TIMEOUT = -14        /* a tensor-core kernel gave up waiting for its MMAs */
};

/* ---- enums -------------------------------------------------------------- */
enum { OPIV_U8 = 0, OPIV_U16 = 1, OPIV_F32 = 2 };           /* pixel type of the frames */
enum { OPIV_CORR_REAL = 0,      /* FFT::cross_correlate_real, fft.h:208-227 (spectrum row 0,
                                   row H/2 and column 0 left at zero, as the reference does) */
       OPIV_CORR_COMPLEX = 1,   /* FFT::cross_correlate, fft.h:188-206 (circular correlation) */
       OPIV_CORR_POCKET = 2,    /* PocketFFT::cross_correlate, pocket_fft.h:236-253: c2c both
                                   ways with fct 1.0 -- the same circular correlation */
       OPIV_CORR_POCKET_REAL = 3 }; /* PocketFFT::cross_correlate_real, pocket_fft.h:255-272:
                                   r2c / c2r with fct 1.0 -- the same circular correlation
                                   (no partial unpack); both pocket modes run the COMPLEX
                                   kernels */

/* Per-window result, as the reference's point_vector (main.cpp:144-149):
 * x, y   window midpoint, y measured from the image top (H - y, main.cpp:230)
 * u, v   midpoint - (bottom-left + fitted peak)        (main.cpp:227)
 * sn     first peak / second peak if the second is > 0 (main.cpp:233-234)
 * All five are 0 when fewer than two peaks were found (main.cpp:214-218). */
typedef struct { float x, y, u, v, sn; } opiv_vector;

/* peak code per window: py * W + px of the first peak in the quadrant-
 * swapped plane (zero lag at (W/2, W/2)), or -1 when fewer than two peaks;
 * OPIV_PEAK_EXACT is or-ed in when the window was decided by the exact
 * double-precision pass rather than the FP32 pass. */
#define OPIV_PEAK_EXACT 0x40000000
#define OPIV_PEAK_MASK 0x0000FFFF

typedef struct opiv_plan opiv_plan;

/* ---- library ------------------------------------------------------------ */
const char* opiv_last_error(void);
const char* opiv_status_string(int status);
int opiv_version(void);
/* number of GPU kernel launches issued by this thread's calls so far */
int64_t opiv_kernel_launch_count(void);

/* ---- grid (host; bit-exact with the reference) --------------------------- */
/* core::generate_cartesian_grid(size, size, double)  grid.h:88-91, grid.impl.h:9-22.
 * Writes (x, y) bottom-left corners, y outer / x inner.  out_xy may be NULL
 * to query the count.  Returns the window count or a negative status. */
int64_t opiv_grid(uint32_t img_w, uint32_t img_h, uint32_t ia_w, uint32_t ia_h,
                  double step_fraction, int32_t* out_xy, int64_t cap);
/* core::generate_cartesian_grid(size, size, array<uint32_t,2>)  grid.h:104-107,
 * grid.impl.h:24-61. */
int64_t opiv_grid_offsets(uint32_t img_w, uint32_t img_h, uint32_t ia_w, uint32_t ia_h,
                          uint32_t dx, uint32_t dy, int32_t* out_xy, int64_t cap);

/* ---- plans -------------------------------------------------------------- */
/* A plan fixes image size, pixel type, window size, grid step and mode, and
 * owns the device scratch for one pair at a time.  ia must be a power of two
 * the build has a kernel for (16, 32 or 64): fft.h:76-84 throws for non-powers
 * of two (OPIV_ERR_NOT_POW2); other powers of two give OPIV_ERR_UNSUPPORTED.
 * dx, dy: grid step in pixels (generate_cartesian_grid's offsets).
 * limit_search: search peaks only in the centre rect().dilate(0.5) of the
 * plane (main.cpp:204-208).  A grid of more than 2^31 - 1 windows gives
 * OPIV_ERR_CAPACITY (the kernels index a pass's windows in 32 bits). */
int opiv_plan_create(opiv_plan** plan, uint32_t img_w, uint32_t img_h, int dtype, uint32_t ia,
                     uint32_t dx, uint32_t dy, int mode, int limit_search, int device);
int opiv_plan_destroy(opiv_plan* plan);
int64_t opiv_plan_window_count(const opiv_plan* plan);
/* copies the plan's grid (bottom-left corners) to out_xy (2 * count int32) */
int opiv_plan_grid(const opiv_plan* plan, int32_t* out_xy, int64_t cap);

/* Whole pass over one image pair, host buffers in and out (synchronous).
 * frame_a, frame_b: img_h rows of pitch_bytes each.  out_vec: count
 * entries.  out_peak: count int32 or NULL.  Replaces the grid loop of
 * main.cpp:239-302 (with the processor of :189-237). */
int opiv_process_pair(opiv_plan* plan, const void* frame_a, const void* frame_b, size_t pitch_bytes,
                      opiv_vector* out_vec, int32_t* out_peak);

/* Same, all buffers on the device, asynchronous on `stream` (a cudaStream_t;
 * NULL = legacy default stream).  d_out_peak may be NULL. */
int opiv_process_pair_device(opiv_plan* plan, const void* d_frame_a, const void* d_frame_b,
                             size_t pitch_bytes, opiv_vector* d_out_vec, int32_t* d_out_peak,
                             void* stream);

/* number of windows the last pass sent to the exact double-precision
 * re-evaluation (synchronises with the plan's last pass) */
int64_t opiv_plan_exact_count(opiv_plan* plan);

/* Many image pairs of the plan's size through opiv_process_pair's pass,
 * pipelined: the upload of pair i+1 and the download of pair i-1 overlap
 * the pass over pair i (three device slots, two compute streams, an upload
 * and a download stream; frames in pinned host memory are needed for the
 * overlap).  No
 * counterpart in the reference (its loop handles one pair).  Returns when
 * every pair's vectors (and peak codes if out_peak is not null) are in host
 * memory. */
int opiv_process_pairs(opiv_plan* plan, int64_t n_pairs, const void* const* frames_a,
                       const void* const* frames_b, size_t pitch_bytes, opiv_vector* const* out_vec,
                       int32_t* const* out_peak);

/* Kernel timing, the GPU counterpart of the reference's "processing time"
 * log (main.cpp:239, :304-309).  When enabled, every pass records CUDA
 * events around its two kernels on the pass's stream; opiv_plan_last_timing
 * waits for the last pass and returns the FP32 kernel's and the exact
 * pass's durations in milliseconds. */
int opiv_plan_set_timing(opiv_plan* plan, int enable);
int opiv_plan_last_timing(opiv_plan* plan, float* fp32_ms, float* exact_ms);

/* ---- precision of a plan's passes ---------------------------------------------
 * No counterpart in the reference (it computes in double only).
 * OPIV_PREC_FP32 (default): the FP32 kernels plus the exact re-decision
 *   pass; integer peaks identical to the reference, u, v within 1e-4 px.
 * OPIV_PREC_TC_SPLIT_BF16: 16, 32, 48 or 64 px windows as four DFT matrix
 *   products on the tensor cores, BF16 operands split into hi + lo parts,
 *   FP32 accumulation; no exact pass (a window whose top two plane values
 *   lie within the rounding may pick the other peak).  Needs u8/u16 frames
 *   and 16-byte aligned rows; 32 px windows also window x positions and x
 *   step multiples of 8 pixels; OPIV_ERR_UNSUPPORTED otherwise.  48 px windows need a plan from
 *   opiv_plan_create_tc (the FFT path takes powers of 2 only) and run a
 *   kernel with one window per tile on any regular grid.  16 px grids
 *   with row steps of 1..6 pixels and window x positions and x step on
 *   multiples of 4 pixels run a kernel that stacks eight windows of a grid
 *   column per tile (each image row transformed once); other 16 px grids a
 *   generic kernel (about half as fast).  64 px grids with window x
 *   positions and x step on multiples of 8 pixels run a kernel with one
 *   window per tile (about three times the generic kernel's speed).
 * OPIV_PREC_TC_BF16: the same with plain BF16 operands (one MMA per product).
 * OPIV_PREC_TC_SPLIT_FP16 / OPIV_PREC_TC_FP16: the same with FP16 operands
 *   (11-bit significand), kept inside FP16's range by powers of two (a
 *   fixed one per stage, one per window for the product), undone exactly.
 * OPIV_PREC_TC_SPLIT2_FP16: FP16 operands with the data
 *   split into hi + lo and the constant matrices single FP16 (hi*C + lo*C,
 *   two MMAs per product instead of three): the data carries ~22 bits, the
 *   DFT constants 11, so the error is set by the constants' rounding.
 * OPIV_PREC_FP64: every window through the exact FP64 kernel (the
 *   reference's arithmetic, bit-identical planes): the oracle pass that the
 *   other precisions are measured against.
 * The last timing's "fp32_ms" is the main kernel of whichever precision. */
enum {
    OPIV_PREC_FP32 = 0,
    OPIV_PREC_TC_SPLIT_BF16 = 1,
    OPIV_PREC_TC_BF16 = 2,
    OPIV_PREC_FP64 = 3,
    OPIV_PREC_TC_SPLIT_FP16 = 4,
    OPIV_PREC_TC_FP16 = 5,
    OPIV_PREC_TC_SPLIT2_FP16 = 6
};
int opiv_plan_set_precision(opiv_plan* plan, int precision);

/* A plan of the tensor-core path alone, created with one of the
 * OPIV_PREC_TC_* precisions: 16, 32, 48 or 64 px windows.  A DFT matrix
 * needs no power of 2, so 48 px windows, which FFT::FFT rejects
 * (fft.h:76-84, OPIV_ERR_NOT_POW2 from opiv_plan_create), are taken here;
 * such a plan refuses OPIV_PREC_FP32 / OPIV_PREC_FP64 and the adjoint with
 * OPIV_ERR_NOT_POW2.  Other arguments as opiv_plan_create. */
int opiv_plan_create_tc(opiv_plan** plan, uint32_t img_w, uint32_t img_h, int dtype, uint32_t ia,
                        uint32_t dx, uint32_t dy, int mode, int limit_search, int precision,
                        int device);
/* Tile shape of the 32 px tensor-core kernel (no reference counterpart):
 * a CTA takes four windows stacked in a grid column (OPIV_TILE_VERTICAL:
 * the 56 image rows of the four are transformed once; row steps of at most
 * 8 px) or side by side in a grid row (OPIV_TILE_HORIZONTAL); AUTO stacks
 * them where the step allows.  opiv_plan_get_tile returns the shape a pass
 * of the plan uses (AUTO for plans without a choice: FFT path, 16/48/64 px).
 * opiv_plan_autotune times both shapes on the given device frames (fastest
 * of three passes after a warm-up, CUDA events on `stream`, outputs into the
 * plan's own buffers) and keeps the faster; synchronous; a no-op for plans
 * without a choice. */
enum { OPIV_TILE_AUTO = 0, OPIV_TILE_VERTICAL = 1, OPIV_TILE_HORIZONTAL = 2 };
int opiv_plan_set_tile(opiv_plan* plan, int tile);
int opiv_plan_get_tile(const opiv_plan* plan);
int opiv_plan_autotune(opiv_plan* plan, const void* d_frame_a, const void* d_frame_b,
                       size_t pitch_bytes, void* stream);
/* Test of the failure path (no counterpart in the reference).  With on = 1
 * the 32 px tensor-core kernel of this plan issues no MMAs, so every CTA's
 * first wait for them runs out after its bounded poll limit (about a
 * second), the CTA stops, frees its tensor memory and flags the plan's
 * status: the pass returns OPIV_ERR_TIMEOUT (its outputs are not valid) and
 * the device stays usable.  on = 0 restores normal passes.
 * OPIV_ERR_UNSUPPORTED for other plans. */
int opiv_plan_test_mma_timeout(opiv_plan* plan, int on);
/* OPIV_OK, or OPIV_ERR_TIMEOUT if a tensor-core pass of this plan gave up
 * waiting for its MMAs since the last call (waits for the plan's work). */
int opiv_plan_status(opiv_plan* plan);
/* Tensor-core precisions only: where the next passes also write every
 * window's correlation plane after swap_quadrants, minus its pedestal
 * sum(a) * sum(b) (n_win x 32 x 32 floats, device memory), and the
 * pedestals (n_win doubles).  Null pointers switch the output off. */
int opiv_plan_set_plane_output(opiv_plan* plan, float* d_planes, double* d_pedestals);

/* ---- adjoint: d(u, v) / d(pixels) --------------------------------------------
 * No counterpart in the reference.  For a pair and the peak codes of a
 * pass over it (the d_out_peak of opiv_process_pair_device; any
 * correlation mode, single-pass plans), the vector u = W/2 - px - fx,
 * v = W/2 - py - fy depends on the pixels only through the 3-point fit of
 * five plane values, each a direct correlation sum (REAL mode: of the
 * windows with each row's mean and each column's mean and alternating
 * mean removed, which is what its zeroed spectrum column 0 and rows 0,
 * H/2 amount to); the adjoint recomputes them (no plane is stored) and
 *  - with d_cotangent (n_win x 2 floats: dL/du, dL/dv per window) adds the
 *    vector-Jacobian product into d_grad_a / d_grad_b (float images of the
 *    frames' size, grad_pitch_bytes per row; accumulated, not cleared);
 *  - with d_sigma (n_win x 2 floats) writes the propagated standard
 *    deviation of u and v for independent pixel noise of variance var_a
 *    (frame A) and var_b (frame B); NaN where the fit takes the log of a
 *    non-positive value, 0 for windows without two peaks.
 * Integer peaks are held fixed (their derivative is zero almost everywhere).
 * Asynchronous on `stream`. */
int opiv_plan_adjoint(opiv_plan* plan, const void* d_fa, const void* d_fb, size_t pitch_bytes,
                      const int32_t* d_peak, const float* d_cotangent, float* d_grad_a,
                      float* d_grad_b, size_t grad_pitch_bytes, float var_a, float var_b,
                      float* d_sigma, void* stream);

/* ---- multi-pass window offsetting ------------------------------------------
 * No counterpart in the reference (its README lists multi-pass as to do,
 * README.md:280); composed from the reference's per-window steps.  Pass 0 is
 * the single pass above.  Pass k > 0 (window ia[k], step step[k]) moves every
 * frame-B window by the integer displacement of the previous pass's window
 * whose centre is nearest, clamped to keep the window inside the image, then
 * correlates, searches and fits as usual; its vector is the residual vector
 * minus that offset, so it is the total displacement in the reference's
 * sign convention.  The integer displacement a window hands on is its
 * offset plus (px - W/2, py - W/2) of its first peak, or its offset when it
 * has fewer than two peaks; packed (dy << 16) | (dx & 0xffff). */
typedef struct opiv_multipass opiv_multipass;
int opiv_multipass_create(opiv_multipass** mp, uint32_t img_w, uint32_t img_h, int dtype,
                          int n_passes, const uint32_t* ia, const uint32_t* step, int mode,
                          int limit_search, int device);
int opiv_multipass_destroy(opiv_multipass* mp);
int64_t opiv_multipass_window_count(const opiv_multipass* mp, int pass);
int opiv_multipass_grid(const opiv_multipass* mp, int pass, int32_t* out_xy, int64_t cap);
/* host frames in; the last pass's vectors / peak codes / displacements out
 * (each may be NULL); every pass's results stay readable with _results */
int opiv_multipass_process(opiv_multipass* mp, const void* frame_a, const void* frame_b,
                           size_t pitch_bytes, opiv_vector* out_vec, int32_t* out_peak,
                           int32_t* out_disp);
/* device frames, asynchronous on `stream`; results stay on the device */
int opiv_multipass_process_device(opiv_multipass* mp, const void* d_frame_a, const void* d_frame_b,
                                  size_t pitch_bytes, void* stream);
/* copies pass `pass`'s results to host buffers (synchronises the device) */
int opiv_multipass_results(opiv_multipass* mp, int pass, opiv_vector* out_vec, int32_t* out_peak,
                           int32_t* out_disp);

/* ---- batches of image pairs ------------------------------------------------
 * No counterpart in the reference.  Many image pairs (each its own size)
 * through the same multi-pass schedule.  The batch owns device frames
 * (fill them with opiv_batch_upload or through opiv_batch_frames).
 * opiv_batch_run enqueues every pair's passes on forked streams; with
 * use_graph = 1 the first call records that whole submission into a CUDA
 * graph (after one eager run) and every call replays the graph with one
 * launch.  A null `stream` means the batch's own stream (used by
 * opiv_batch_upload too).  Two kernel launches per pair and pass are added
 * to opiv_kernel_launch_count for every run, replayed or not. */
typedef struct opiv_batch opiv_batch;
int opiv_batch_create(opiv_batch** batch, int n_pairs, const uint32_t* widths,
                      const uint32_t* heights, int dtype, int n_passes, const uint32_t* ia,
                      const uint32_t* step, int mode, int limit_search, int device);
int opiv_batch_destroy(opiv_batch* batch);
int opiv_batch_frames(opiv_batch* batch, int pair, void** d_frame_a, void** d_frame_b,
                      size_t* pitch_bytes);
int opiv_batch_upload(opiv_batch* batch, int pair, const void* frame_a, const void* frame_b,
                      size_t pitch_bytes, void* stream);
int opiv_batch_run(opiv_batch* batch, int use_graph, void* stream);
int64_t opiv_batch_window_count(const opiv_batch* batch, int pair, int pass);
int opiv_batch_results(opiv_batch* batch, int pair, int pass, opiv_vector* out_vec,
                       int32_t* out_peak, int32_t* out_disp);
/* Host frames in, every pair's final-pass vectors out, pipelined: pair i's
 * frames go up on an upload stream, its pass chain starts on a fork stream
 * as soon as they are in, and its vectors (and peak codes when out_peak is
 * not null) come back on a download stream as soon as its last pass ends,
 * so copies overlap the other pairs' passes (frames and outputs in pinned
 * host memory are needed for the overlap).  pitch_bytes: one row pitch per
 * pair.  Returns when every pair's results are in host memory. */
int opiv_batch_process(opiv_batch* batch, const void* const* frames_a, const void* const* frames_b,
                       const size_t* pitch_bytes, opiv_vector* const* out_vec,
                       int32_t* const* out_peak);

/* Schedules of a batch (no counterpart in the reference).
 * OPIV_BATCH_STREAMS (the default): every pair's pass chain on a fork
 *   stream, two launches per pair and pass.
 * OPIV_BATCH_QUEUE: per pass and group of up to 64 pairs, one launch over
 *   a device work list that holds the group's windows (a persistent grid
 *   whose CTAs take tasks from an atomic counter, or one CTA per task group;
 *   see the tuning), then one exact re-decision launch over the group's
 *   flagged windows; the groups form lanes on fork streams (see
 *   opiv_batch_set_lanes).  Results are identical to the
 *   streams schedule.  Window sizes 16, 32 and 64 (the FP32 kernels);
 *   OPIV_ERR_UNSUPPORTED otherwise, and when a group's combined window
 *   count exceeds 2^31 - 1.  opiv_batch_process under this schedule uploads
 *   every pair, runs the passes, then downloads (no copy / pass overlap).
 * Changing the schedule or the tuning drops a recorded graph; the next
 * opiv_batch_run with use_graph = 1 records a new one. */
enum { OPIV_BATCH_STREAMS = 0, OPIV_BATCH_QUEUE = 1 };
int opiv_batch_set_schedule(opiv_batch* batch, int schedule);
/* Queue tuning of pass `pass`: the persistent grid has ctas_per_sm CTAs per
 * SM (1 .. 32; above the kernel's resident limit the extra CTAs simply run
 * later) and each warp of a CTA takes `chunk` tasks (1 .. 1024) per dequeue
 * (16, 32 px: a CTA takes 4 * chunk consecutive tasks, its warps
 * interleaved; 64 px: a CTA runs one task at a time).  ctas_per_sm = 0
 * launches the same work list with one CTA per task group instead (the
 * hardware's block scheduler hands them out; no persistent loop, chunk
 * unused).  Untuned passes use the persistent grid at the resident limit
 * and chunk 1. */
int opiv_batch_set_tuning(opiv_batch* batch, int pass, int ctas_per_sm, int chunk);
/* Current tuning of pass `pass`; *max_ctas_per_sm (may be null) receives the
 * queue kernel's resident CTAs per SM (0 before the queue's first use) and
 * *tuned_ms (may be null) the autotuner's fastest time of the pass in ms (0
 * when the pass's tuning did not come from the autotuner). */
int opiv_batch_get_tuning(const opiv_batch* batch, int pass, int* ctas_per_sm, int* chunk,
                          int* max_ctas_per_sm, float* tuned_ms);
/* Lanes of the queue schedule (1 .. 8, default 2, at most the number of
 * pairs): the pairs are split into `lanes` sets of about equal image area,
 * each running its pass chain on its own fork stream, so that one lane's
 * exact re-decision (a few hundred microseconds of FP64 latency per pass)
 * overlaps another lane's FP32 kernel.  Two launches per pass and group;
 * a group holds up to 64 pairs of one lane.  opiv_batch_get_lanes returns
 * the lanes in use (or a negative status). */
int opiv_batch_set_lanes(opiv_batch* batch, int lanes);
int opiv_batch_get_lanes(const opiv_batch* batch);
/* Autotuner: selects the queue schedule and, pass after pass, times every
 * candidate (the hardware-dispatched list; persistent grids of 1 .. resident
 * limit (at most 4) CTAs per SM with chunk 1, 2, 4, 8; fastest of
 * two timed runs after one warm-up, CUDA events on `stream`) on the frames
 * the batch holds now, and keeps the fastest per pass.  The pass chain runs
 * in order, so each pass is tuned on the real offsets of the one before.
 * Then the whole chain is timed with 1 and 2 lanes and the faster kept.
 * The batch's results afterwards are those of a normal run.  Synchronous. */
int opiv_batch_autotune(opiv_batch* batch, void* stream);

/* ---- allocation-free pass ------------------------------------------------ */
/* No counterpart in the reference.  The same pass as opiv_process_pair_device
 * for callers that must not allocate device memory once they are running
 * (fixed-budget acquisition loops, hosts that own the device allocator): no
 * plan, no cudaMalloc / cudaFree.  Its scratch lives in one fixed device
 * array of about 4 MiB that every GPU using the library holds until exit.
 * Limits: 16 or 32 px windows only (64 px: OPIV_ERR_UNSUPPORTED); grids of
 * more than 1,048,576 windows are rejected (OPIV_ERR_CAPACITY); the
 * PocketFFT modes run the COMPLEX kernels, as opiv_plan_create does.
 * The first call on a device does a one-time set-up (address lookup and a
 * synchronous table upload): make it before any stream capture.  The set-up
 * is not repeated, so the call is not usable after a cudaDeviceReset.  All
 * calls share the scratch; calls that overlap on the GPU race, so order them
 * on one stream.  Uses the current device; asynchronous on `stream`. */
int opiv_process_pair_device_noalloc(const void* d_frame_a, const void* d_frame_b,
                                     size_t pitch_bytes, uint32_t img_w, uint32_t img_h, int dtype,
                                     uint32_t ia, uint32_t dx, uint32_t dy, int mode,
                                     int limit_search, opiv_vector* d_out_vec, int32_t* d_out_peak,
                                     void* stream);

/* ---- per-window correlation (FFT::cross_correlate[_real] on a batch) ------ */
/* n window pairs of w x w doubles (a, b: n*w*w each, row-major), planes out:
 * n*w*w doubles, quadrant-swapped as the reference returns them.
 * exact = 0: FP32 kernels + exact pedestal (within 1e-5 of the plane peak);
 * exact = 1: double-precision kernels that repeat the reference's arithmetic
 * operation for operation (bit-identical planes).  Host buffers, synchronous.
 * At most (2^31 - 1) / w windows per call (OPIV_ERR_CAPACITY beyond).
 * FFT::cross_correlate / cross_correlate_real: fft.h:188-227. */
int opiv_cross_correlate_batch(const double* a, const double* b, uint32_t w, int64_t n, int mode,
                               int exact, double* out_planes, int device);

/* ---- per-window spectra (FFT::transform, transform_real, auto_correlate) -- */
/* algos::direction (fft_common.h:9-12) */
enum { OPIV_FORWARD = 0, OPIV_REVERSE = 1 };
/* n windows of w x w, row-major, complex values interleaved (re, im).
 * All three run the exact double kernel (the reference's butterflies,
 * twiddle tables and complex products, bit-identical results) on the GPU;
 * host buffers, synchronous.  w: a power of 2 from 4 to 64.
 * FFT::transform(input, d), fft.h:87-119: unnormalised 2-D transform of
 *   `in` (2 n w^2 doubles) into `out`. */
int opiv_transform_batch(const double* in, uint32_t w, int64_t n, int direction, double* out,
                         int device);
/* FFT::transform_real(a, b, d), fft.h:123-186: a, b real (n w^2 doubles
 * each); out_a, out_b the two spectra of the two-for-one transform with the
 * reference's partial unpack (rows [1, H/2) x columns [1, W) and their
 * mirrors; row 0, row H/2 and column 0 zero). */
int opiv_transform_real_batch(const double* a, const double* b, uint32_t w, int64_t n, int direction,
                              double* out_a, double* out_b, int device);
/* FFT::auto_correlate(a), fft.h:229-242: real(IFFT(|FFT(a)|^2)) after
 * swap_quadrants, as a complex image with zero imaginary parts. */
int opiv_auto_correlate_batch(const double* in, uint32_t w, int64_t n, double* out, int device);

/* ---- image ingest and vector output (host) ------------------------------- */
/* The reference's loaders (loaders/pnm_image_loader.cpp:199-226, PNM P5/P6,
 * 8- or 16-bit big-endian samples; loaders/tiff_image_loader.cpp:190-226,
 * TIFF through libtiff) deliver 8/16-bit grey samples (RGB -> grey with
 * (218 r + 732 g + 74 b) >> 10, pixel_types.h:390-400).  These read PNM and
 * baseline uncompressed TIFF (8/16-bit, 1 or 3 samples, first image) without
 * external libraries.  dtype: OPIV_U8 for 8-bit files, OPIV_U16 for 16-bit. */
int opiv_image_info(const char* path, uint32_t* width, uint32_t* height, int* dtype);
int opiv_image_load(const char* path, void* out, size_t pitch_bytes, uint32_t width,
                    uint32_t height, int dtype);
/* One "x, y, u, v, sn" line per window, as main.cpp:312-313 prints them
 * (6 significant digits); path NULL or "-" writes to stdout. */
int opiv_vectors_write(const char* path, const opiv_vector* vectors, int64_t n);

/* ---- host helpers of the same path (no GPU) ------------------------------ */
/* core::find_peaks(im, num_peaks, radius): image_utils.impl.h:42-74.  Writes
 * up to num_peaks centres (x, y) and values, highest first; returns count. */
int opiv_find_peaks(const double* im, uint32_t w, uint32_t h, uint16_t num_peaks, uint32_t radius,
                    int32_t* out_xy, double* out_value);
/* The two offsets fit_simple_gaussian adds to a 3x3 view's midpoint
 * (image_utils.impl.h:86-98): v9 row-major, out_fxfy = (fx, fy). */
int opiv_gaussian_offsets(const double* v9, double* out_fxfy);
/* core::fit_simple_gaussian on the 3x3 around (px, py): image_utils.impl.h:77-101 */
int opiv_fit_simple_gaussian(const double* plane, uint32_t w, uint32_t h, int32_t px, int32_t py,
                             double* out_xy);

#ifdef __cplusplus
}
#endif

#endif /* OPENPIV_GB300_H */
