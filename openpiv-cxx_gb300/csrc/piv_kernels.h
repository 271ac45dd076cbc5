// piv_kernels.h -- launch interface between the C ABI layer and the kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "openpiv_gb300.h"

namespace opiv {

enum { kModeReal = OPIV_CORR_REAL, kModeComplex = OPIV_CORR_COMPLEX };
enum { kU8 = OPIV_U8, kU16 = OPIV_U16, kF32 = OPIV_F32, kF64 = 3 /* internal: batch API */ };

// Everything one pass over an image pair needs on the device.
struct PivParams {
    const void* fa = nullptr;          // frame A (device), img_h rows of `pitch` bytes
    const void* fb = nullptr;          // frame B
    size_t pitch = 0;                  // bytes per row
    int img_w = 0, img_h = 0;
    // regular grid: window k at (gx0 + (k % gnx) * gdx, gy0 + (k / gnx) * gdy)
    int gx0 = 0, gy0 = 0, gdx = 0, gdy = 0, gnx = 1;
    // 32 px tensor-core kernel: tiles of four windows stacked in a grid
    // column (1, rows transformed once; row steps <= 8 only) or side by side
    // in a grid row (2); 0: stacked where allowed
    int tc_tile = 0;
    const int32_t* win_xy = nullptr;   // explicit (x, y) list overrides the grid
    int64_t n_win = 0;
    opiv_vector* out_vec = nullptr;
    int32_t* out_peak = nullptr;       // may be null
    // windows whose FP32 decisions are not certain (see piv_fp32.cu)
    unsigned int* flag_count = nullptr;
    int32_t* flag_list = nullptr;
    int32_t flag_base = 0;             // added to a flagged window's index (a queue's list)
    float kappa = 16.f;                // FP32 error-bound factor
    // debug / per-window API outputs
    float* planes = nullptr;           // FP32 kernel: n_win * W * W (mean-free part)
    double* peds = nullptr;            // FP32 kernel: per-window pedestal
    double* planes64 = nullptr;        // exact kernel: n_win * W * W full planes
    // exact pass
    const double2* tw_fwd = nullptr;   // reference twiddle tables for length W
    const double2* tw_rev = nullptr;
    // window offsetting (multi-pass): integer displacement of every window
    // of the previous pass, packed (dy << 16) | (dx & 0xffff), and that
    // pass's grid; frame B's window is moved by the displacement of the
    // previous window nearest to this window's centre.  Null: no offset.
    const int32_t* prev_disp = nullptr;
    int pgx0 = 0, pgy0 = 0, pgdx = 1, pgdy = 1, pgnx = 1, pgny = 1, pw = 0;
    // test of the failure path: the 32 px tensor-core kernel issues no MMAs,
    // so its bounded waits run out and it reports through `status`
    int mma_skip = 0;
    int32_t* out_disp = nullptr;       // this pass's integer displacements (may be null)
    int* status = nullptr;             // tensor-core kernel: set to 1 if an MMA wait gave up
};

// Tensor-core DFT-GEMM kernels (piv_tc.cu): 16, 32, 48 and 64 px windows
// (32: piv_tc_kernel.cuh; the others: piv_tcg_kernel.cuh), u8/u16 frames,
// window x positions and steps multiples of 8 pixels.  Constant matrices,
// each W x W 16-bit in the K-major no-swizzle operand layout, all hi parts
// then all lo parts; -S, C, S adjacent so that [C; S] and [-S; C] are
// 2W-row operands.
enum { kTcG1 = 0, kTcNS = 1, kTcC = 2, kTcS = 3, kTcC4 = 4, kTcNumMat = 5 };
bool tc_supports(int w, int dtype);
size_t tc_constant_bytes(int w);
void tc_constants(int w, unsigned char* out);
// Adjoint of a pass (piv_adjoint.cu): complex or REAL mode planes, peaks
// from the forward pass, cotangents (n_win x 2) pulled back into float image
// gradients (accumulated, gpitch floats per row) and/or the propagated
// standard deviation of u, v (n_win x 2) for pixel noise variances var_a, var_b.
cudaError_t launch_piv_adjoint(const PivParams& p, int w, int dtype, int mode, const int32_t* peaks,
                               const float* cot, float* grad_a, float* grad_b, size_t gpitch,
                               float var_a, float var_b, float* sigma, cudaStream_t s);

// consts: tc_constant_bytes(w) bytes from tc_constants (BF16 set, FP16 set);
// passes: MMAs per product, 3 (hi*hi + hi*lo + lo*hi), 2 (data split,
// constants single; 32 px windows) or 1
cudaError_t launch_piv_tc(const PivParams& p, int w, int dtype, int mode, int limit, int passes,
                          bool fp16, const void* consts, cudaStream_t s);

// Fused FP32 kernels, one entry per window size (piv_fp32_w*.cu; 64 x 64
// windows use the shared-memory kernel of piv_fp32_w64.cu).  Frames
// (u8/u16/f32) without plane output; double windows (kF64) with planes.
cudaError_t launch_piv_fp32_w16(const PivParams& p, int dtype, int mode, int limit, bool planes,
                                cudaStream_t s);
cudaError_t launch_piv_fp32_w32(const PivParams& p, int dtype, int mode, int limit, bool planes,
                                cudaStream_t s);
cudaError_t launch_piv_fp32_w64(const PivParams& p, int dtype, int mode, int limit, bool planes,
                                cudaStream_t s);
inline bool fp32_supports(int w) { return w == 16 || w == 32 || w == 64; }
inline cudaError_t launch_piv_fp32(const PivParams& p, int w, int dtype, int mode, int limit,
                                   bool planes, cudaStream_t s)
{
    if (w == 16) return launch_piv_fp32_w16(p, dtype, mode, limit, planes, s);
    if (w == 32) return launch_piv_fp32_w32(p, dtype, mode, limit, planes, s);
    if (w == 64) return launch_piv_fp32_w64(p, dtype, mode, limit, planes, s);
    return cudaErrorInvalidValue;
}

// Exact double-precision re-evaluation.  When `list_count` is non-null the
// kernel processes the windows listed in flag_list[0 .. *list_count);
// otherwise all n_win windows.  `blocks` CTAs stride over the work.
bool exact_supports(int w);
cudaError_t launch_piv_exact(const PivParams& p, int w, int dtype, int mode, int limit,
                             bool use_list, int blocks, cudaStream_t s);

// The per-window spectral API (FFT::transform, transform_real,
// auto_correlate; fft.h:87-186, :229-242) on n windows of w x w, in the
// exact kernel's double arithmetic (piv_exact.cu).  All device pointers:
//  kSpectralTransform  in_c (complex) -> out_a, with tw = the forward or
//                      the reverse table;
//  kSpectralReal       in_ra, in_rb (real) -> out_a, out_b (the partial
//                      unpack), tw = one direction's table;
//  kSpectralAuto       in_c -> out_a (real part, quadrant-swapped, zero
//                      imaginary parts), tw = forward table then reverse.
enum { kSpectralTransform = 0, kSpectralReal = 1, kSpectralAuto = 2 };
struct SpectralParams {
    int w = 0;
    int64_t n = 0;
    const double2* in_c = nullptr;
    const double* in_ra = nullptr;
    const double* in_rb = nullptr;
    double2* out_a = nullptr;
    double2* out_b = nullptr;
    const double2* tw = nullptr;
};
cudaError_t launch_spectral_exact(const SpectralParams& q, int op, int blocks, cudaStream_t s);

// Device work queue of one pass over up to kQueueMaxItems image pairs (one
// window size), passed by value in the kernel's parameter space (read
// through the constant cache): pair j is items[j]; its tasks are numbered
// first_task[j] .. first_task[j + 1] - 1 and its windows first_win[j] ..
// first_win[j + 1] - 1 in the queue's combined numbering.  A task is what
// one warp (16, 32 px: 2 * 32 / W windows) or one CTA (64 px: two windows)
// of the single-pair kernel does.  Two launch shapes run the tasks: a
// persistent grid whose CTAs take them from *head (zero before the launch),
// or the list kernels, one CTA per task group handed out by the hardware
// (the exact kernel reads items[]; the FP32 kernels copy items_g[task_item[t]]
// into shared memory per task).  Every item flags its uncertain windows into
// one list (flag_count / flag_list, combined window numbers), which the
// exact queue kernel then re-decides for all the queue's pairs at once.
constexpr int kQueueMaxItems = 64;
struct PivQueue {
    PivParams items[kQueueMaxItems];
    int first_task[kQueueMaxItems + 1] = {};
    int first_win[kQueueMaxItems + 1] = {};
    int n_items = 0;
    // the same descriptors in global memory (a task copies its pair's into
    // shared memory) and the pair of every task, one byte each
    const PivParams* items_g = nullptr;
    const uint8_t* task_item = nullptr;
    unsigned int* head = nullptr;
    int chunk = 1;
    const unsigned int* flag_count = nullptr;
    const int32_t* flag_list = nullptr;
};
static_assert(kQueueMaxItems <= 256, "task_item holds pair numbers in one byte");
static_assert(sizeof(PivParams) == 208, "descriptor size (queue parameter space)");
static_assert(sizeof(PivParams) % 16 == 0, "descriptors are copied in 16-byte words");
// tasks of a pair of n_win windows in the queue of window size w
inline int fp32_queue_tasks(int w, int64_t n_win)
{
    const int per = w == 64 ? 2 : 2 * (32 / w);
    return (int)((n_win + per - 1) / per);
}
// Queue kernels per window size (piv_fp32_w*.cu).  `vec`: every item's A
// rows start on 16-byte boundaries (128-bit loads); `blocks` CTAs of the
// persistent grid.  With max_ctas non-null nothing is launched and
// *max_ctas receives the kernel's resident CTAs per SM.
cudaError_t queue_piv_fp32_w16(const PivQueue& q, int dtype, int mode, int limit, bool vec, int blocks,
                               int* max_ctas, cudaStream_t s);
cudaError_t queue_piv_fp32_w32(const PivQueue& q, int dtype, int mode, int limit, bool vec, int blocks,
                               int* max_ctas, cudaStream_t s);
cudaError_t queue_piv_fp32_w64(const PivQueue& q, int dtype, int mode, int limit, bool vec, int blocks,
                               int* max_ctas, cudaStream_t s);
inline cudaError_t queue_piv_fp32(const PivQueue& q, int w, int dtype, int mode, int limit, bool vec,
                                  int blocks, int* max_ctas, cudaStream_t s)
{
    if (w == 16) return queue_piv_fp32_w16(q, dtype, mode, limit, vec, blocks, max_ctas, s);
    if (w == 32) return queue_piv_fp32_w32(q, dtype, mode, limit, vec, blocks, max_ctas, s);
    if (w == 64) return queue_piv_fp32_w64(q, dtype, mode, limit, vec, blocks, max_ctas, s);
    return cudaErrorInvalidValue;
}
// The exact pass over a queue's combined flag list (piv_exact.cu), and the
// resident CTAs per SM of that kernel for window size w.
cudaError_t launch_piv_exact_queue(const PivQueue& q, int w, int dtype, int mode, int limit,
                                   int blocks, cudaStream_t s);
int exact_queue_max_ctas_per_sm(int w);

// Records `message` as the calling thread's last error (opiv_last_error)
// and returns `status`.
int record_error(int status, const char* message);

// Streaming multiprocessors of `device` (queried once per device, then
// cached); 1 if the query fails, so that grid sizes stay positive.
int device_sm_count(int device);

}  // namespace opiv
