// opiv_api.cpp -- the C ABI (include/openpiv_gb300.h): validation, grids,
// plans, device buffers and kernel launches.  Host C++17; the kernels are in
// piv_fp32_w*.cu and piv_exact.cu.
//
// Errors: every entry point returns a status code; the message of the last
// failure on the calling thread is kept for opiv_last_error().  Messages
// start with the same text as the exceptions the reference throws.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "openpiv_gb300.h"
#include "piv_kernels.h"

using namespace opiv;

namespace {

thread_local std::string g_last_error;
thread_local int64_t g_launches = 0;

int fail(int status, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return status;
}

int cuda_fail(cudaError_t e, const char* what)
{
    return fail(OPIV_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define CUDA_TRY(call)                                          \
    do {                                                        \
        cudaError_t e_ = (call);                                \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call);     \
    } while (0)

// the same inside functions that restore the caller's device through `done`
#define CUDA_TRY_D(call)                                              \
    do {                                                              \
        cudaError_t e_ = (call);                                      \
        if (e_ != cudaSuccess) return done(cuda_fail(e_, #call));     \
    } while (0)

// openpiv/core/util.h:67-70
bool is_pow2(uint64_t v) { return v && (v == (v & (~v + 1))); }

size_t px_bytes(int dtype)
{
    switch (dtype) {
    case OPIV_U8: return 1;
    case OPIV_U16: return 2;
    case OPIV_F32: return 4;
    default: return 0;
    }
}

struct grid_geom {
    int64_t xc = 0, yc = 0;
    int64_t xs = 0, ys = 0;
};

// generate_cartesian_grid(size, size, array<uint32_t,2>) argument checks and
// geometry: openpiv/core/detail/grid.impl.h:29-48 (same unsigned arithmetic).
int grid_geometry(uint32_t img_w, uint32_t img_h, uint32_t ia_w, uint32_t ia_h, uint32_t dx,
                  uint32_t dy, grid_geom& g)
{
    if ((uint64_t)img_w * img_h == 0) return fail(OPIV_ERR_IMAGE_EMPTY, "image size must be non-zero");
    if ((uint64_t)ia_w * ia_h == 0)
        return fail(OPIV_ERR_IA_EMPTY, "interrogation size must be non-zero");
    if (dx == 0 || dy == 0) return fail(OPIV_ERR_OFFSET_ZERO, "offsets must be non-zero");
    if (ia_w > img_w || ia_h > img_h)
        return fail(OPIV_ERR_IA_TOO_BIG, "interrogation size is bigger than image");
    const uint32_t xc = 1 + (img_w - ia_w) / dx;
    const uint32_t yc = 1 + (img_h - ia_h) / dy;
    g.xc = xc;
    g.yc = yc;
    g.xs = (img_w - ia_w - (dx * (xc - 1))) / 2;
    g.ys = (img_h - ia_h - (dy * (yc - 1))) / 2;
    return OPIV_OK;
}

// Twiddle table exactly as the reference builds it (fft.h:274-294):
// entry i = (cos t, sin t), t = (s * M_PI * i) / n, s = -1 forward, +1 reverse.
std::vector<double2> reference_twiddles(uint32_t n, int dir)
{
    std::vector<double2> t(n);
    const double s = dir < 0 ? -1.0 : 1.0;
    for (uint32_t i = 0; i < n; ++i) {
        const double theta = (s * M_PI * (double)(int)i) / (double)n;
        t[i] = make_double2(std::cos(theta), std::sin(theta));
    }
    return t;
}

// CTAs of the exact pass: two per SM for a flagged list, eight per SM when
// every window takes the exact kernel
int exact_blocks(int device) { return 2 * device_sm_count(device); }
int exact_all_blocks(int device) { return 8 * device_sm_count(device); }

bool is_tc(int precision)
{
    return precision == OPIV_PREC_TC_SPLIT_BF16 || precision == OPIV_PREC_TC_BF16 ||
           precision == OPIV_PREC_TC_SPLIT_FP16 || precision == OPIV_PREC_TC_FP16 ||
           precision == OPIV_PREC_TC_SPLIT2_FP16;
}

// MMAs per product of a tensor-core precision: 3 (hi*hi + hi*lo + lo*hi),
// 2 (data split, constants single) or 1
int tc_passes(int precision)
{
    if (precision == OPIV_PREC_TC_SPLIT_BF16 || precision == OPIV_PREC_TC_SPLIT_FP16) return 3;
    return precision == OPIV_PREC_TC_SPLIT2_FP16 ? 2 : 1;
}

// The PocketFFT modes compute the true circular correlation, as
// FFT::cross_correlate does: they run the COMPLEX kernels.
int kernel_mode(int mode)
{
    return (mode == OPIV_CORR_POCKET || mode == OPIV_CORR_POCKET_REAL) ? OPIV_CORR_COMPLEX : mode;
}
// Error-bound factor of the FP32 kernel: the largest error measured on 68k
// windows of particle images (W = 16, 32; both modes) was 3.15 * 2^-24 * 2N *
// (E_1 + E_2) (E = window energy of the pair sharing an inverse transform);
// 8 leaves a 2.5x margin.
constexpr float kKappa = 8.0f;

}  // namespace

int opiv::record_error(int status, const char* message)
{
    g_last_error = message;
    return status;
}

int opiv::device_sm_count(int device)
{
    static std::atomic<int> cache[64];
    if (device < 0 || device >= 64) return 1;
    int n = cache[device].load();
    if (n > 0) return n;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || n <= 0) return 1;
    cache[device].store(n);
    return n;
}

struct opiv_plan {
    int device = 0;
    uint32_t img_w = 0, img_h = 0, ia = 0, dx = 0, dy = 0;
    int dtype = 0, mode = 0, limit = 0;
    grid_geom g;
    int64_t n_win = 0;
    cudaStream_t stream = nullptr;      // used by the host-buffer calls
    void* d_fa = nullptr;               // frames for the host-buffer calls
    void* d_fb = nullptr;
    size_t d_pitch = 0;
    opiv_vector* d_vec = nullptr;
    int32_t* d_peak = nullptr;
    unsigned int* d_flag_count = nullptr;
    int32_t* d_flag_list = nullptr;
    double2* d_tw = nullptr;            // forward then reverse, ia entries each
    unsigned int* h_flag_count = nullptr;   // pinned copy of the last count
    bool timing = false;
    cudaEvent_t ev[3] = { nullptr, nullptr, nullptr };   // fp32 start, fp32 end, exact end
    int32_t* d_disp = nullptr;          // integer displacements (multi-pass plans)
    int precision = OPIV_PREC_FP32;
    int tc_tile = OPIV_TILE_AUTO;       // 32 px tensor-core tile shape
    int mma_skip = 0;                   // failure-path test: no MMAs issued
    void* d_tc = nullptr;               // tensor-core constant matrices
    int* d_status = nullptr;            // tensor-core wait status
    float* d_planes = nullptr;          // optional plane output (tensor-core precisions)
    double* d_peds = nullptr;
    // opiv_process_pairs: kPipeSlots slots of device frames, outputs and
    // exact-pass scratch, an upload and a download stream, a second compute
    // stream, and the events that order them with the passes
    static constexpr int kPipeSlots = 3;
    bool pipe = false;
    cudaStream_t up = nullptr, down = nullptr;
    cudaStream_t cs2 = nullptr;                 // compute stream of odd pairs
    unsigned int* p_flag_count[kPipeSlots] = {};
    int32_t* p_flag_list[kPipeSlots] = {};
    void* p_fa[kPipeSlots] = {};
    void* p_fb[kPipeSlots] = {};
    opiv_vector* p_vec[kPipeSlots] = {};
    int32_t* p_peak[kPipeSlots] = {};
    cudaEvent_t ev_up[kPipeSlots] = {}, ev_done[kPipeSlots] = {}, ev_down[kPipeSlots] = {};
};

// A chain of plans over the same image pair: pass k's frame-B windows are
// offset by pass k-1's integer displacements (offsets.cuh).
struct opiv_multipass {
    std::vector<opiv_plan*> passes;
    void* d_fa = nullptr;
    void* d_fb = nullptr;
    size_t d_pitch = 0;
};

namespace {

void plan_free(opiv_plan* p)
{
    if (!p) return;
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(p->device);
    if (p->stream) cudaStreamSynchronize(p->stream);
    cudaFree(p->d_fa);
    cudaFree(p->d_fb);
    cudaFree(p->d_vec);
    cudaFree(p->d_peak);
    cudaFree(p->d_flag_count);
    cudaFree(p->d_flag_list);
    cudaFree(p->d_tw);
    cudaFree(p->d_disp);
    cudaFree(p->d_tc);
    cudaFree(p->d_status);
    if (p->up) cudaStreamSynchronize(p->up);
    if (p->down) cudaStreamSynchronize(p->down);
    for (int k = 0; k < opiv_plan::kPipeSlots; ++k) {
        cudaFree(p->p_fa[k]);
        cudaFree(p->p_fb[k]);
        cudaFree(p->p_vec[k]);
        cudaFree(p->p_peak[k]);
        if (p->ev_up[k]) cudaEventDestroy(p->ev_up[k]);
        if (p->ev_done[k]) cudaEventDestroy(p->ev_done[k]);
        if (p->ev_down[k]) cudaEventDestroy(p->ev_down[k]);
    }
    if (p->cs2) cudaStreamSynchronize(p->cs2);
    for (int k = 0; k < opiv_plan::kPipeSlots; ++k) {
        cudaFree(p->p_flag_count[k]);
        cudaFree(p->p_flag_list[k]);
    }
    if (p->up) cudaStreamDestroy(p->up);
    if (p->down) cudaStreamDestroy(p->down);
    if (p->cs2) cudaStreamDestroy(p->cs2);
    if (p->h_flag_count) cudaFreeHost(p->h_flag_count);
    for (cudaEvent_t& e : p->ev)
        if (e) cudaEventDestroy(e);
    if (p->stream) cudaStreamDestroy(p->stream);
    cudaSetDevice(prev);
    delete p;
}

PivParams base_params(const opiv_plan* p)
{
    PivParams k;
    k.img_w = (int)p->img_w;
    k.img_h = (int)p->img_h;
    k.gx0 = (int)p->g.xs;
    k.gy0 = (int)p->g.ys;
    k.gdx = (int)p->dx;
    k.gdy = (int)p->dy;
    k.gnx = (int)p->g.xc;
    k.n_win = p->n_win;
    k.kappa = kKappa;
    k.flag_count = p->d_flag_count;
    k.flag_list = p->d_flag_list;
    k.tw_fwd = p->d_tw;
    k.tw_rev = p->d_tw + p->ia;
    return k;
}

// One pass: FP32 kernel over all windows, then the exact pass over the
// flagged ones.  Two kernel launches.  `prev` (may be null): the previous
// pass of a multi-pass chain, whose integer displacements offset frame B.
// flag_count / flag_list: the exact pass's scratch (null: the plan's own;
// passes that may run concurrently need their own).
// The parameters of one pass of plan p over frames fa, fb; `prev`: the
// previous pass of a multi-pass chain (window offsetting) or null.
PivParams pass_params(const opiv_plan* p, const void* fa, const void* fb, size_t pitch,
                      opiv_vector* vec, int32_t* peak, const opiv_plan* prev)
{
    PivParams k = base_params(p);
    k.fa = fa;
    k.fb = fb;
    k.pitch = pitch;
    k.out_vec = vec;
    k.out_peak = peak;
    k.out_disp = p->d_disp;
    if (prev != nullptr) {
        k.prev_disp = prev->d_disp;
        k.pgx0 = (int)prev->g.xs;
        k.pgy0 = (int)prev->g.ys;
        k.pgdx = (int)prev->dx;
        k.pgdy = (int)prev->dy;
        k.pgnx = (int)prev->g.xc;
        k.pgny = (int)prev->g.yc;
        k.pw = (int)prev->ia;
    }
    return k;
}

int run_pass(opiv_plan* p, const void* fa, const void* fb, size_t pitch, opiv_vector* vec,
             int32_t* peak, cudaStream_t s, const opiv_plan* prev = nullptr,
             unsigned int* flag_count = nullptr, int32_t* flag_list = nullptr)
{
    PivParams k = pass_params(p, fa, fb, pitch, vec, peak, prev);
    if (flag_count) {
        k.flag_count = flag_count;
        k.flag_list = flag_list;
    }
    CUDA_TRY(cudaMemsetAsync(k.flag_count, 0, sizeof(unsigned int), s));
    if (is_tc(p->precision)) {
        if (((uintptr_t)fa | (uintptr_t)fb | (uintptr_t)pitch) % 16 != 0)
            return fail(OPIV_ERR_ARG, "the tensor-core path needs 16-byte aligned frame rows");
        k.status = p->d_status;
        k.planes = p->d_planes;
        k.peds = p->d_peds;
        k.tc_tile = p->tc_tile;
        k.mma_skip = p->mma_skip;
        if (p->timing) CUDA_TRY(cudaEventRecord(p->ev[0], s));
        CUDA_TRY(launch_piv_tc(k, (int)p->ia, p->dtype, p->mode, p->limit, tc_passes(p->precision),
                               p->precision == OPIV_PREC_TC_SPLIT_FP16 || p->precision == OPIV_PREC_TC_FP16 ||
                                   p->precision == OPIV_PREC_TC_SPLIT2_FP16,
                               p->d_tc, s));
        ++g_launches;
        if (p->timing) {
            CUDA_TRY(cudaEventRecord(p->ev[1], s));
            CUDA_TRY(cudaEventRecord(p->ev[2], s));
        }
        return OPIV_OK;
    }
    if (p->precision == OPIV_PREC_FP64) {
        if (p->timing) CUDA_TRY(cudaEventRecord(p->ev[0], s));
        CUDA_TRY(launch_piv_exact(k, (int)p->ia, p->dtype, p->mode, p->limit, false, exact_all_blocks(p->device), s));
        ++g_launches;
        if (p->timing) {
            CUDA_TRY(cudaEventRecord(p->ev[1], s));
            CUDA_TRY(cudaEventRecord(p->ev[2], s));
        }
        return OPIV_OK;
    }
    if (p->timing) CUDA_TRY(cudaEventRecord(p->ev[0], s));
    CUDA_TRY(launch_piv_fp32(k, (int)p->ia, p->dtype, p->mode, p->limit, false, s));
    ++g_launches;
    if (p->timing) CUDA_TRY(cudaEventRecord(p->ev[1], s));
    CUDA_TRY(launch_piv_exact(k, (int)p->ia, p->dtype, p->mode, p->limit, true, exact_blocks(p->device), s));
    ++g_launches;
    if (p->timing) CUDA_TRY(cudaEventRecord(p->ev[2], s));
    return OPIV_OK;
}

}  // namespace

extern "C" {

const char* opiv_last_error(void) { return g_last_error.c_str(); }

const char* opiv_status_string(int s)
{
    switch (s) {
    case OPIV_OK: return "ok";
    case OPIV_ERR_OFFSET_RANGE: return "offsets must be between 0.0 and 1.0";
    case OPIV_ERR_IMAGE_EMPTY: return "image size must be non-zero";
    case OPIV_ERR_IA_EMPTY: return "interrogation size must be non-zero";
    case OPIV_ERR_OFFSET_ZERO: return "offsets must be non-zero";
    case OPIV_ERR_IA_TOO_BIG: return "interrogation size is bigger than image";
    case OPIV_ERR_NOT_POW2: return "dimensions must be power of 2";
    case OPIV_ERR_CAPACITY: return "output buffer too small";
    case OPIV_ERR_RECT_OUTSIDE: return "extract: rectangle to extract is too large for image";
    case OPIV_ERR_ARG: return "invalid argument";
    case OPIV_ERR_SIZE_MISMATCH: return "image size is different from expected";
    case OPIV_ERR_UNSUPPORTED: return "unsupported window size";
    case OPIV_ERR_CUDA: return "CUDA error";
    case OPIV_ERR_NO_DEVICE: return "no CUDA device";
    case OPIV_ERR_TIMEOUT: return "a tensor-core kernel gave up waiting for its MMAs";
    default: return "unknown status";
    }
}

int opiv_version(void) { return 100; }

int64_t opiv_kernel_launch_count(void) { return g_launches; }

int64_t opiv_grid_offsets(uint32_t img_w, uint32_t img_h, uint32_t ia_w, uint32_t ia_h,
                          uint32_t dx, uint32_t dy, int32_t* out_xy, int64_t cap)
{
    grid_geom g;
    const int rc = grid_geometry(img_w, img_h, ia_w, ia_h, dx, dy, g);
    if (rc != OPIV_OK) return rc;
    const int64_t n = g.xc * g.yc;
    if (out_xy == nullptr) return n;
    if (cap < n) return fail(OPIV_ERR_CAPACITY, "grid needs %lld entries, buffer has %lld",
                             (long long)n, (long long)cap);
    int64_t k = 0;
    for (int64_t y = 0; y < g.yc; ++y)
        for (int64_t x = 0; x < g.xc; ++x, ++k) {
            out_xy[2 * k] = (int32_t)(g.xs + x * dx);
            out_xy[2 * k + 1] = (int32_t)(g.ys + y * dy);
        }
    return n;
}

int64_t opiv_grid(uint32_t img_w, uint32_t img_h, uint32_t ia_w, uint32_t ia_h,
                  double step_fraction, int32_t* out_xy, int64_t cap)
{
    // grid.impl.h:14-21
    if (step_fraction < 0.0 || step_fraction > 1.0)
        return fail(OPIV_ERR_OFFSET_RANGE, "offsets must be between 0.0 and 1.0");
    return opiv_grid_offsets(img_w, img_h, ia_w, ia_h, (uint32_t)(ia_w * step_fraction),
                             (uint32_t)(ia_h * step_fraction), out_xy, cap);
}

namespace {

// tc_only: a plan of the tensor-core path alone (any window size that path
// takes, powers of 2 or not); otherwise the FFT path's rules
int plan_create(opiv_plan** out, uint32_t img_w, uint32_t img_h, int dtype, uint32_t ia, uint32_t dx,
                uint32_t dy, int mode, int limit_search, int device, bool tc_only)
{
    if (out == nullptr) return fail(OPIV_ERR_ARG, "plan pointer is null");
    *out = nullptr;
    if (px_bytes(dtype) == 0) return fail(OPIV_ERR_ARG, "unknown pixel type %d", dtype);
    if (mode < OPIV_CORR_REAL || mode > OPIV_CORR_POCKET_REAL)
        return fail(OPIV_ERR_ARG, "unknown correlation mode %d", mode);
    mode = kernel_mode(mode);
    grid_geom g;
    int rc = grid_geometry(img_w, img_h, ia, ia, dx, dy, g);
    if (rc != OPIV_OK) return rc;
    if (tc_only) {
        if (!tc_supports((int)ia, dtype))
            return fail(OPIV_ERR_UNSUPPORTED,
                        "the tensor-core path takes 16, 32, 48 or 64 px windows of u8/u16 frames");
    } else {
        if (!is_pow2(ia)) return fail(OPIV_ERR_NOT_POW2, "dimensions must be power of 2: %ux%u", ia, ia);
        if (!fp32_supports((int)ia) || !exact_supports((int)ia))
            return fail(OPIV_ERR_UNSUPPORTED, "no kernel for %ux%u windows", ia, ia);
    }
    if (g.xs + (int64_t)dx * (g.xc - 1) + ia > (int64_t)img_w || g.ys + (int64_t)dy * (g.yc - 1) + ia > (int64_t)img_h)
        return fail(OPIV_ERR_RECT_OUTSIDE, "extract: rectangle to extract is too large for image");
    // the kernels index a pass's windows with 32-bit integers
    if ((int64_t)g.xc * g.yc > (int64_t)INT32_MAX)
        return fail(OPIV_ERR_CAPACITY, "grid of %lld windows: a plan takes at most 2^31 - 1",
                    (long long)((int64_t)g.xc * g.yc));

    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return fail(OPIV_ERR_NO_DEVICE, "no CUDA device");
    if (device < 0 || device >= ndev) return fail(OPIV_ERR_ARG, "device %d out of range", device);

    opiv_plan* p = new (std::nothrow) opiv_plan;
    if (!p) return fail(OPIV_ERR_ARG, "out of host memory");
    p->device = device;
    p->img_w = img_w;
    p->img_h = img_h;
    p->ia = ia;
    p->dx = dx;
    p->dy = dy;
    p->dtype = dtype;
    p->mode = mode;
    p->limit = limit_search ? 1 : 0;
    p->g = g;
    p->n_win = g.xc * g.yc;

    int prev = 0;
    cudaGetDevice(&prev);
    auto done = [&](int status) {
        cudaSetDevice(prev);
        if (status != OPIV_OK) plan_free(p);
        else *out = p;
        return status;
    };
    cudaError_t e;
    if ((e = cudaSetDevice(device)) != cudaSuccess) return done(cuda_fail(e, "cudaSetDevice"));
    if ((e = cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking)) != cudaSuccess)
        return done(cuda_fail(e, "cudaStreamCreate"));
    if ((e = cudaMalloc(&p->d_vec, sizeof(opiv_vector) * p->n_win)) != cudaSuccess)
        return done(cuda_fail(e, "cudaMalloc(vectors)"));
    if ((e = cudaMalloc(&p->d_peak, sizeof(int32_t) * p->n_win)) != cudaSuccess)
        return done(cuda_fail(e, "cudaMalloc(peaks)"));
    if ((e = cudaMalloc(&p->d_flag_count, sizeof(unsigned int))) != cudaSuccess)
        return done(cuda_fail(e, "cudaMalloc(flag count)"));
    if ((e = cudaMalloc(&p->d_flag_list, sizeof(int32_t) * p->n_win)) != cudaSuccess)
        return done(cuda_fail(e, "cudaMalloc(flag list)"));
    if ((e = cudaMemset(p->d_flag_count, 0, sizeof(unsigned int))) != cudaSuccess)
        return done(cuda_fail(e, "cudaMemset"));
    if ((e = cudaMallocHost(&p->h_flag_count, sizeof(unsigned int))) != cudaSuccess)
        return done(cuda_fail(e, "cudaMallocHost"));
    *p->h_flag_count = 0;
    if (is_pow2(ia)) {   // the exact kernel's twiddles (FFT path)
        std::vector<double2> tw = reference_twiddles(ia, -1), tr = reference_twiddles(ia, +1);
        tw.insert(tw.end(), tr.begin(), tr.end());
        if ((e = cudaMalloc(&p->d_tw, sizeof(double2) * tw.size())) != cudaSuccess)
            return done(cuda_fail(e, "cudaMalloc(twiddles)"));
        if ((e = cudaMemcpy(p->d_tw, tw.data(), sizeof(double2) * tw.size(), cudaMemcpyHostToDevice)) !=
            cudaSuccess)
            return done(cuda_fail(e, "cudaMemcpy(twiddles)"));
    }
    return done(OPIV_OK);
}

}  // namespace

int opiv_plan_create(opiv_plan** out, uint32_t img_w, uint32_t img_h, int dtype, uint32_t ia,
                     uint32_t dx, uint32_t dy, int mode, int limit_search, int device)
{
    return plan_create(out, img_w, img_h, dtype, ia, dx, dy, mode, limit_search, device, false);
}

int opiv_plan_create_tc(opiv_plan** out, uint32_t img_w, uint32_t img_h, int dtype, uint32_t ia,
                        uint32_t dx, uint32_t dy, int mode, int limit_search, int precision, int device)
{
    if (precision < OPIV_PREC_FP32 || precision > OPIV_PREC_TC_SPLIT2_FP16)
        return fail(OPIV_ERR_ARG, "unknown precision %d", precision);
    if (!is_tc(precision)) return fail(OPIV_ERR_ARG, "precision %d is not a tensor-core precision", precision);
    int rc = plan_create(out, img_w, img_h, dtype, ia, dx, dy, mode, limit_search, device, true);
    if (rc != OPIV_OK) return rc;
    rc = opiv_plan_set_precision(*out, precision);
    if (rc != OPIV_OK) {
        const std::string msg = opiv_last_error();
        opiv_plan_destroy(*out);
        *out = nullptr;
        return fail(rc, "%s", msg.c_str());
    }
    return OPIV_OK;
}

int opiv_plan_destroy(opiv_plan* plan)
{
    plan_free(plan);
    return OPIV_OK;
}

int64_t opiv_plan_window_count(const opiv_plan* plan)
{
    if (!plan) return fail(OPIV_ERR_ARG, "plan is null");
    return plan->n_win;
}

int opiv_plan_grid(const opiv_plan* plan, int32_t* out_xy, int64_t cap)
{
    if (!plan || !out_xy) return fail(OPIV_ERR_ARG, "null argument");
    const int64_t n = opiv_grid_offsets(plan->img_w, plan->img_h, plan->ia, plan->ia, plan->dx,
                                        plan->dy, out_xy, cap);
    return n < 0 ? (int)n : OPIV_OK;
}

int opiv_process_pair_device(opiv_plan* plan, const void* d_fa, const void* d_fb,
                             size_t pitch_bytes, opiv_vector* d_out_vec, int32_t* d_out_peak,
                             void* stream)
{
    if (!plan || !d_fa || !d_fb || !d_out_vec) return fail(OPIV_ERR_ARG, "null argument");
    if (pitch_bytes < (size_t)plan->img_w * px_bytes(plan->dtype) ||
        pitch_bytes % px_bytes(plan->dtype) != 0)
        return fail(OPIV_ERR_ARG, "pitch %zu too small or not a multiple of the pixel size",
                    pitch_bytes);
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(plan->device);
    const int rc = run_pass(plan, d_fa, d_fb, pitch_bytes, d_out_vec, d_out_peak,
                            (cudaStream_t)stream);
    if (rc == OPIV_OK)
        cudaMemcpyAsync(plan->h_flag_count, plan->d_flag_count, sizeof(unsigned int),
                        cudaMemcpyDeviceToHost, (cudaStream_t)stream);
    cudaSetDevice(prev);
    return rc;
}

int opiv_process_pair(opiv_plan* plan, const void* frame_a, const void* frame_b, size_t pitch_bytes,
                      opiv_vector* out_vec, int32_t* out_peak)
{
    if (!plan || !frame_a || !frame_b || !out_vec) return fail(OPIV_ERR_ARG, "null argument");
    const size_t row = (size_t)plan->img_w * px_bytes(plan->dtype);
    if (pitch_bytes < row) return fail(OPIV_ERR_ARG, "pitch %zu smaller than a row", pitch_bytes);
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(plan->device);
    auto done = [&](int s) { cudaSetDevice(prev); return s; };
    cudaError_t e;
    if (!plan->d_fa) {
        if ((e = cudaMalloc(&plan->d_fa, row * plan->img_h)) != cudaSuccess)
            return done(cuda_fail(e, "cudaMalloc(frame)"));
        if ((e = cudaMalloc(&plan->d_fb, row * plan->img_h)) != cudaSuccess)
            return done(cuda_fail(e, "cudaMalloc(frame)"));
        plan->d_pitch = row;
    }
    cudaStream_t s = plan->stream;
    if ((e = cudaMemcpy2DAsync(plan->d_fa, plan->d_pitch, frame_a, pitch_bytes, row, plan->img_h,
                               cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return done(cuda_fail(e, "cudaMemcpy2DAsync(frame a)"));
    if ((e = cudaMemcpy2DAsync(plan->d_fb, plan->d_pitch, frame_b, pitch_bytes, row, plan->img_h,
                               cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return done(cuda_fail(e, "cudaMemcpy2DAsync(frame b)"));
    int rc = run_pass(plan, plan->d_fa, plan->d_fb, plan->d_pitch, plan->d_vec,
                      out_peak ? plan->d_peak : nullptr, s);
    if (rc != OPIV_OK) return done(rc);
    if ((e = cudaMemcpyAsync(out_vec, plan->d_vec, sizeof(opiv_vector) * plan->n_win,
                             cudaMemcpyDeviceToHost, s)) != cudaSuccess)
        return done(cuda_fail(e, "cudaMemcpyAsync(vectors)"));
    if (out_peak &&
        (e = cudaMemcpyAsync(out_peak, plan->d_peak, sizeof(int32_t) * plan->n_win,
                             cudaMemcpyDeviceToHost, s)) != cudaSuccess)
        return done(cuda_fail(e, "cudaMemcpyAsync(peaks)"));
    cudaMemcpyAsync(plan->h_flag_count, plan->d_flag_count, sizeof(unsigned int),
                    cudaMemcpyDeviceToHost, s);
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess)
        return done(cuda_fail(e, "cudaStreamSynchronize"));
    if (plan->d_status) return done(opiv_plan_status(plan));
    return done(OPIV_OK);
}

int opiv_process_pairs(opiv_plan* plan, int64_t n_pairs, const void* const* frames_a,
                       const void* const* frames_b, size_t pitch_bytes, opiv_vector* const* out_vec,
                       int32_t* const* out_peak)
{
    if (!plan || n_pairs < 0 || (n_pairs > 0 && (!frames_a || !frames_b || !out_vec)))
        return fail(OPIV_ERR_ARG, "null argument");
    if (n_pairs == 0) return OPIV_OK;
    const size_t row = (size_t)plan->img_w * px_bytes(plan->dtype);
    if (pitch_bytes < row) return fail(OPIV_ERR_ARG, "pitch %zu smaller than a row", pitch_bytes);
    for (int64_t i = 0; i < n_pairs; ++i)
        if (!frames_a[i] || !frames_b[i] || !out_vec[i] || (out_peak && !out_peak[i]))
            return fail(OPIV_ERR_ARG, "null buffer for pair %lld", (long long)i);
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(plan->device);
    auto done = [&](int st) { cudaSetDevice(prev); return st; };
    cudaError_t e = cudaSuccess;
    if (!plan->pipe) {
        for (int k = 0; k < opiv_plan::kPipeSlots && e == cudaSuccess; ++k) {
            if ((e = cudaMalloc(&plan->p_fa[k], row * plan->img_h)) != cudaSuccess) break;
            if ((e = cudaMalloc(&plan->p_fb[k], row * plan->img_h)) != cudaSuccess) break;
            if ((e = cudaMalloc(&plan->p_vec[k], sizeof(opiv_vector) * plan->n_win)) != cudaSuccess) break;
            if ((e = cudaMalloc(&plan->p_peak[k], sizeof(int32_t) * plan->n_win)) != cudaSuccess) break;
            if ((e = cudaEventCreateWithFlags(&plan->ev_up[k], cudaEventDisableTiming)) != cudaSuccess) break;
            if ((e = cudaEventCreateWithFlags(&plan->ev_done[k], cudaEventDisableTiming)) != cudaSuccess) break;
            if ((e = cudaEventCreateWithFlags(&plan->ev_down[k], cudaEventDisableTiming)) != cudaSuccess) break;
            if ((e = cudaMalloc(&plan->p_flag_count[k], sizeof(unsigned int))) != cudaSuccess) break;
            e = cudaMalloc(&plan->p_flag_list[k], sizeof(int32_t) * plan->n_win);
        }
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&plan->up, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&plan->down, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&plan->cs2, cudaStreamNonBlocking);
        if (e != cudaSuccess) return done(cuda_fail(e, "opiv_process_pairs set-up"));
        plan->pipe = true;
    }
    // the plan's timing events cannot follow two streams: off meanwhile
    const bool timing = plan->timing;
    plan->timing = false;
    struct restore_timing {
        opiv_plan* p;
        bool t;
        ~restore_timing() { p->timing = t; }
    } restore{ plan, timing };
    // pair i uses slot k = i % 3 and compute stream i % 2: its upload
    // waits until pass i-3 has read the slot's frames, its pass until the
    // download of pair i-3 has read the slot's outputs; uploads, passes and
    // downloads of neighbouring pairs overlap, and so do the exact pass of
    // one pair (a few SMs) and the FP32 kernel of the next.  Three slots:
    // a slot's upload does not wait for the pass just before it.
    constexpr int S = opiv_plan::kPipeSlots;
    for (int64_t i = 0; i < n_pairs; ++i) {
        const int k = (int)(i % S);
        cudaStream_t cs = (i & 1) ? plan->cs2 : plan->stream;
        if (i >= S) CUDA_TRY(cudaStreamWaitEvent(plan->up, plan->ev_done[k], 0));
        if ((e = cudaMemcpy2DAsync(plan->p_fa[k], row, frames_a[i], pitch_bytes, row, plan->img_h,
                                   cudaMemcpyHostToDevice, plan->up)) != cudaSuccess ||
            (e = cudaMemcpy2DAsync(plan->p_fb[k], row, frames_b[i], pitch_bytes, row, plan->img_h,
                                   cudaMemcpyHostToDevice, plan->up)) != cudaSuccess)
            return done(cuda_fail(e, "cudaMemcpy2DAsync(frames)"));
        CUDA_TRY(cudaEventRecord(plan->ev_up[k], plan->up));
        CUDA_TRY(cudaStreamWaitEvent(cs, plan->ev_up[k], 0));
        if (i >= S) CUDA_TRY(cudaStreamWaitEvent(cs, plan->ev_down[k], 0));
        const int rc = run_pass(plan, plan->p_fa[k], plan->p_fb[k], row, plan->p_vec[k],
                                out_peak ? plan->p_peak[k] : nullptr, cs, nullptr,
                                plan->p_flag_count[k], plan->p_flag_list[k]);
        if (rc != OPIV_OK) return done(rc);
        CUDA_TRY(cudaEventRecord(plan->ev_done[k], cs));
        CUDA_TRY(cudaStreamWaitEvent(plan->down, plan->ev_done[k], 0));
        if ((e = cudaMemcpyAsync(out_vec[i], plan->p_vec[k], sizeof(opiv_vector) * plan->n_win,
                                 cudaMemcpyDeviceToHost, plan->down)) != cudaSuccess)
            return done(cuda_fail(e, "cudaMemcpyAsync(vectors)"));
        if (out_peak && (e = cudaMemcpyAsync(out_peak[i], plan->p_peak[k], sizeof(int32_t) * plan->n_win,
                                             cudaMemcpyDeviceToHost, plan->down)) != cudaSuccess)
            return done(cuda_fail(e, "cudaMemcpyAsync(peaks)"));
        CUDA_TRY(cudaEventRecord(plan->ev_down[k], plan->down));
    }
    if ((e = cudaStreamSynchronize(plan->down)) != cudaSuccess ||
        (e = cudaStreamSynchronize(plan->stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(plan->cs2)) != cudaSuccess)
        return done(cuda_fail(e, "cudaStreamSynchronize"));
    if (plan->d_status) return done(opiv_plan_status(plan));
    return done(OPIV_OK);
}

int64_t opiv_plan_exact_count(opiv_plan* plan)
{
    if (!plan) return fail(OPIV_ERR_ARG, "plan is null");
    cudaDeviceSynchronize();
    return (int64_t)*plan->h_flag_count;
}

int opiv_multipass_create(opiv_multipass** out, uint32_t img_w, uint32_t img_h, int dtype,
                          int n_passes, const uint32_t* ia, const uint32_t* step, int mode,
                          int limit_search, int device)
{
    if (!out || !ia || !step || n_passes < 1) return fail(OPIV_ERR_ARG, "invalid multi-pass arguments");
    *out = nullptr;
    opiv_multipass* mp = new (std::nothrow) opiv_multipass;
    if (!mp) return fail(OPIV_ERR_ARG, "out of host memory");
    for (int k = 0; k < n_passes; ++k) {
        opiv_plan* p = nullptr;
        int rc = opiv_plan_create(&p, img_w, img_h, dtype, ia[k], step[k], step[k], mode,
                                  limit_search, device);
        if (rc == OPIV_OK) {
            int prev = 0;
            cudaGetDevice(&prev);
            cudaSetDevice(device);
            const cudaError_t e = cudaMalloc(&p->d_disp, sizeof(int32_t) * p->n_win);
            cudaSetDevice(prev);
            if (e != cudaSuccess) {
                plan_free(p);
                rc = cuda_fail(e, "cudaMalloc(displacements)");
            }
        }
        if (rc != OPIV_OK) {
            opiv_multipass_destroy(mp);
            return rc;
        }
        mp->passes.push_back(p);
    }
    *out = mp;
    return OPIV_OK;
}

int opiv_multipass_destroy(opiv_multipass* mp)
{
    if (!mp) return OPIV_OK;
    if (!mp->passes.empty()) {
        int prev = 0;
        cudaGetDevice(&prev);
        cudaSetDevice(mp->passes[0]->device);
        cudaFree(mp->d_fa);
        cudaFree(mp->d_fb);
        cudaSetDevice(prev);
    }
    for (opiv_plan* p : mp->passes) plan_free(p);
    delete mp;
    return OPIV_OK;
}

int64_t opiv_multipass_window_count(const opiv_multipass* mp, int pass)
{
    if (!mp || pass < 0 || pass >= (int)mp->passes.size()) return fail(OPIV_ERR_ARG, "no such pass");
    return mp->passes[pass]->n_win;
}

int opiv_multipass_grid(const opiv_multipass* mp, int pass, int32_t* out_xy, int64_t cap)
{
    if (!mp || pass < 0 || pass >= (int)mp->passes.size()) return fail(OPIV_ERR_ARG, "no such pass");
    return opiv_plan_grid(mp->passes[pass], out_xy, cap);
}

int opiv_multipass_process_device(opiv_multipass* mp, const void* d_fa, const void* d_fb,
                                  size_t pitch_bytes, void* stream)
{
    if (!mp || !d_fa || !d_fb) return fail(OPIV_ERR_ARG, "null argument");
    opiv_plan* first = mp->passes[0];
    if (pitch_bytes < (size_t)first->img_w * px_bytes(first->dtype))
        return fail(OPIV_ERR_ARG, "pitch %zu smaller than a row", pitch_bytes);
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(first->device);
    int rc = OPIV_OK;
    for (size_t k = 0; k < mp->passes.size() && rc == OPIV_OK; ++k) {
        opiv_plan* p = mp->passes[k];
        rc = run_pass(p, d_fa, d_fb, pitch_bytes, p->d_vec, p->d_peak, (cudaStream_t)stream,
                      k ? mp->passes[k - 1] : nullptr);
    }
    cudaSetDevice(prev);
    return rc;
}

int opiv_multipass_process(opiv_multipass* mp, const void* frame_a, const void* frame_b,
                           size_t pitch_bytes, opiv_vector* out_vec, int32_t* out_peak,
                           int32_t* out_disp)
{
    if (!mp || !frame_a || !frame_b) return fail(OPIV_ERR_ARG, "null argument");
    opiv_plan* first = mp->passes[0];
    const size_t row = (size_t)first->img_w * px_bytes(first->dtype);
    if (pitch_bytes < row) return fail(OPIV_ERR_ARG, "pitch %zu smaller than a row", pitch_bytes);
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(first->device);
    auto done = [&](int st) { cudaSetDevice(prev); return st; };
    cudaError_t e;
    if (!mp->d_fa) {
        if ((e = cudaMalloc(&mp->d_fa, row * first->img_h)) != cudaSuccess) return done(cuda_fail(e, "cudaMalloc(frame)"));
        if ((e = cudaMalloc(&mp->d_fb, row * first->img_h)) != cudaSuccess) return done(cuda_fail(e, "cudaMalloc(frame)"));
        mp->d_pitch = row;
    }
    cudaStream_t s = first->stream;
    if ((e = cudaMemcpy2DAsync(mp->d_fa, mp->d_pitch, frame_a, pitch_bytes, row, first->img_h,
                               cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return done(cuda_fail(e, "cudaMemcpy2DAsync(frame a)"));
    if ((e = cudaMemcpy2DAsync(mp->d_fb, mp->d_pitch, frame_b, pitch_bytes, row, first->img_h,
                               cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return done(cuda_fail(e, "cudaMemcpy2DAsync(frame b)"));
    const int rc = opiv_multipass_process_device(mp, mp->d_fa, mp->d_fb, mp->d_pitch, s);
    if (rc != OPIV_OK) return done(rc);
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return done(cuda_fail(e, "cudaStreamSynchronize"));
    cudaSetDevice(prev);
    return opiv_multipass_results(mp, (int)mp->passes.size() - 1, out_vec, out_peak, out_disp);
}

int opiv_multipass_results(opiv_multipass* mp, int pass, opiv_vector* out_vec, int32_t* out_peak,
                           int32_t* out_disp)
{
    if (!mp || pass < 0 || pass >= (int)mp->passes.size()) return fail(OPIV_ERR_ARG, "no such pass");
    opiv_plan* p = mp->passes[pass];
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(p->device);
    auto done = [&](int st) { cudaSetDevice(prev); return st; };
    cudaError_t e;
    if ((e = cudaDeviceSynchronize()) != cudaSuccess) return done(cuda_fail(e, "cudaDeviceSynchronize"));
    if (out_vec && (e = cudaMemcpy(out_vec, p->d_vec, sizeof(opiv_vector) * p->n_win,
                                   cudaMemcpyDeviceToHost)) != cudaSuccess)
        return done(cuda_fail(e, "cudaMemcpy(vectors)"));
    if (out_peak && (e = cudaMemcpy(out_peak, p->d_peak, sizeof(int32_t) * p->n_win,
                                    cudaMemcpyDeviceToHost)) != cudaSuccess)
        return done(cuda_fail(e, "cudaMemcpy(peaks)"));
    if (out_disp && (e = cudaMemcpy(out_disp, p->d_disp, sizeof(int32_t) * p->n_win,
                                    cudaMemcpyDeviceToHost)) != cudaSuccess)
        return done(cuda_fail(e, "cudaMemcpy(displacements)"));
    return done(OPIV_OK);
}

// ---- batches of image pairs ----------------------------------------------------
// Device work queues of one pass of a batch (OPIV_BATCH_QUEUE): the pairs
// in groups of up to kQueueMaxItems, one queue (two launches) per group.
struct batch_queue_pass {
    std::vector<PivQueue> groups;       // host copies, passed by value at launch
    unsigned int* d_ctr = nullptr;      // per group: dequeue head, flagged windows
    int32_t* d_flags = nullptr;         // per group: its flag list (combined window numbers)
    PivParams* d_items = nullptr;       // per group: its descriptors (kQueueMaxItems slots)
    uint8_t* d_task_item = nullptr;     // per group: the pair of every task
    int ia = 0, dtype = 0, mode = 0, limit = 0;
    bool vec = true;                    // every pair's A rows 16-byte aligned
    int max_ctas = 0;                   // resident CTAs per SM of the queue kernel
    int exact_blocks = 0;               // CTAs of the exact launch: every resident slot
    int ctas_per_sm = -1;               // tuning: -1 untuned (the resident limit), 0 hardware dispatch
    int chunk = 1;                      // tuning: tasks per dequeue
    float tuned_ms = 0.f;               // the autotuner's fastest pass time
};

struct opiv_batch {
    std::vector<opiv_multipass*> pairs;
    std::vector<void*> d_fa, d_fb;
    std::vector<size_t> pitch;
    cudaStream_t main = nullptr;         // used when the caller passes no stream
    std::vector<cudaStream_t> streams;   // fork streams of the captured graph
    std::vector<cudaEvent_t> events;     // fork / join events
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int device = 0;
    // opiv_batch_process: copy streams and one upload / done event per pair
    cudaStream_t up = nullptr, down = nullptr;
    std::vector<cudaEvent_t> ev_up, ev_done;
    // OPIV_BATCH_QUEUE: one work queue per pass, built on first use; the
    // tuning of a pass may be set before that (kept in tune_*)
    int schedule = OPIV_BATCH_STREAMS;
    std::vector<batch_queue_pass> qp;
    std::vector<int> tune_ctas, tune_chunk;
    std::vector<float> tune_ms;
    int sms = 0;
    // lanes of the queue schedule: the pairs split into `lanes` sets of about
    // equal area, each running its pass chain on its own fork stream; groups
    // are ordered lane by lane, lane l owning groups lane_first[l] ..
    // lane_first[l + 1] - 1
    int lanes = 2;
    std::vector<int> lane_first;
};

namespace {

void batch_drop_graph(opiv_batch* b)
{
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
}

void batch_free_queue(opiv_batch* b)
{
    for (batch_queue_pass& q : b->qp) {
        cudaFree(q.d_ctr);
        cudaFree(q.d_flags);
        cudaFree(q.d_items);
        cudaFree(q.d_task_item);
    }
    b->qp.clear();
}

// Builds every pass's work queues (descriptors of all pairs, counters and
// flag lists on the device); the batch's device is current.
int batch_queue_setup(opiv_batch* b)
{
    if (!b->qp.empty()) return OPIV_OK;
    const int n = (int)b->pairs.size();
    const int n_pass = (int)b->pairs[0]->passes.size();
    if (b->sms == 0) CUDA_TRY(cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->device));
    // pairs to lanes, largest image first to the lane with the least area;
    // each lane's pairs (in index order) in groups of up to kQueueMaxItems
    const int L = std::max(1, std::min({ b->lanes, n, (int)b->streams.size() }));
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    auto area = [&](int i) { return (int64_t)b->pairs[i]->passes[0]->img_w * b->pairs[i]->passes[0]->img_h; };
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return area(x) > area(y); });
    std::vector<std::vector<int>> lane_pairs(L);
    std::vector<int64_t> load(L, 0);
    for (int i : order) {
        const int l = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        lane_pairs[l].push_back(i);
        load[l] += area(i);
    }
    std::vector<std::vector<int>> group_pairs;
    b->lane_first.assign(1, 0);
    for (int l = 0; l < L; ++l) {
        std::sort(lane_pairs[l].begin(), lane_pairs[l].end());
        for (size_t i0 = 0; i0 < lane_pairs[l].size(); i0 += kQueueMaxItems)
            group_pairs.emplace_back(lane_pairs[l].begin() + i0,
                                     lane_pairs[l].begin() + std::min(lane_pairs[l].size(), i0 + kQueueMaxItems));
        b->lane_first.push_back((int)group_pairs.size());
    }
    const int n_groups = (int)group_pairs.size();
    std::vector<batch_queue_pass> qs(n_pass);
    int rc = OPIV_OK;
    for (int k = 0; k < n_pass && rc == OPIV_OK; ++k) {
        batch_queue_pass& q = qs[k];
        const opiv_plan* p0 = b->pairs[0]->passes[k];
        q.ia = (int)p0->ia;
        q.dtype = p0->dtype;
        q.mode = kernel_mode(p0->mode);
        q.limit = p0->limit;
        if (!fp32_supports(q.ia) || p0->precision != OPIV_PREC_FP32) {
            rc = fail(OPIV_ERR_UNSUPPORTED, "the queue schedule runs 16, 32 and 64 px FP32 passes only");
            break;
        }
        q.groups.resize(n_groups);
        std::vector<int64_t> flag_off(n_groups + 1, 0);   // each group's flag list in d_flags
        std::vector<int64_t> task_off(n_groups + 1, 0);   // each group's task pairs in d_task_item
        std::vector<uint8_t> task_item;
        const size_t px = px_bytes(q.dtype);
        for (int g = 0; g < n_groups && rc == OPIV_OK; ++g) {
            PivQueue& pq = q.groups[g];
            pq.n_items = (int)group_pairs[g].size();
            int64_t tasks = 0, wins = 0;
            for (int j = 0; j < pq.n_items; ++j) {
                const int i = group_pairs[g][j];
                const opiv_plan* p = b->pairs[i]->passes[k];
                const opiv_plan* prev = k ? b->pairs[i]->passes[k - 1] : nullptr;
                PivParams it = pass_params(p, b->d_fa[i], b->d_fb[i], b->pitch[i], p->d_vec, p->d_peak, prev);
                pq.first_task[j] = (int)tasks;
                pq.first_win[j] = (int)wins;
                it.flag_base = (int32_t)wins;
                const int nt = fp32_queue_tasks(q.ia, p->n_win);
                task_item.insert(task_item.end(), (size_t)nt, (uint8_t)j);
                tasks += nt;
                wins += p->n_win;
                if (tasks > INT32_MAX || wins > INT32_MAX) {
                    rc = fail(OPIV_ERR_UNSUPPORTED, "a queue of %d pairs holds more than 2^31 - 1 windows",
                              kQueueMaxItems);
                    break;
                }
                // the condition of the single-pair kernel's 128-bit row loads
                q.vec = q.vec && ((uintptr_t)it.fa % 16 == 0) && ((uintptr_t)it.fb % 16 == 0) &&
                        (it.pitch % 16 == 0) && (((size_t)it.gx0 * px) % 16 == 0) &&
                        (((size_t)it.gdx * px) % 16 == 0) && (((size_t)q.ia * px) % 16 == 0);
                pq.items[j] = it;
            }
            pq.first_task[pq.n_items] = (int)tasks;
            pq.first_win[pq.n_items] = (int)wins;
            flag_off[g + 1] = flag_off[g] + (wins > 0 ? wins : 1);
            task_off[g + 1] = task_off[g] + tasks;
        }
        if (rc != OPIV_OK) break;
        cudaError_t e;
        if ((e = cudaMalloc(&q.d_ctr, 2 * sizeof(unsigned int) * n_groups)) != cudaSuccess ||
            (e = cudaMalloc(&q.d_flags, sizeof(int32_t) * flag_off[n_groups])) != cudaSuccess ||
            (e = cudaMalloc(&q.d_items, sizeof(PivParams) * kQueueMaxItems * n_groups)) != cudaSuccess ||
            (e = cudaMalloc(&q.d_task_item, task_item.size() + 1)) != cudaSuccess) {
            rc = cuda_fail(e, "cudaMalloc(work queue)");
            break;
        }
        for (int g = 0; g < n_groups && rc == OPIV_OK; ++g) {
            PivQueue& pq = q.groups[g];
            pq.head = q.d_ctr + 2 * g;
            pq.flag_count = q.d_ctr + 2 * g + 1;
            pq.flag_list = q.d_flags + flag_off[g];
            for (int j = 0; j < pq.n_items; ++j) {   // the group's one flag list
                pq.items[j].flag_count = q.d_ctr + 2 * g + 1;
                pq.items[j].flag_list = q.d_flags + flag_off[g];
            }
            pq.items_g = q.d_items + (size_t)kQueueMaxItems * g;
            pq.task_item = q.d_task_item + task_off[g];
            if ((e = cudaMemcpy(q.d_items + (size_t)kQueueMaxItems * g, pq.items, sizeof(PivParams) * pq.n_items,
                                cudaMemcpyHostToDevice)) != cudaSuccess)
                rc = cuda_fail(e, "cudaMemcpy(work queue)");
        }
        if (rc != OPIV_OK) break;
        if (!task_item.empty() &&
            (e = cudaMemcpy(q.d_task_item, task_item.data(), task_item.size(), cudaMemcpyHostToDevice)) !=
                cudaSuccess) {
            rc = cuda_fail(e, "cudaMemcpy(work queue)");
            break;
        }
        const cudaError_t oe =
            queue_piv_fp32(q.groups[0], q.ia, q.dtype, q.mode, q.limit, q.vec, 0, &q.max_ctas, nullptr);
        if (oe != cudaSuccess) {
            rc = cuda_fail(oe, "queue kernel occupancy");
            break;
        }
        if (q.max_ctas < 1) q.max_ctas = 1;
        // flagged windows are few but each costs ~0.1 ms of FP64 latency in one
        // CTA; as many run at once as fit, so the pass waits about one round
        q.exact_blocks = exact_queue_max_ctas_per_sm(q.ia) * b->sms;
        q.ctas_per_sm = b->tune_ctas[k];
        q.chunk = b->tune_chunk[k];
        q.tuned_ms = b->tune_ms[k];
    }
    b->qp.swap(qs);
    if (rc != OPIV_OK) batch_free_queue(b);   // a failed set-up's partial buffers
    return rc;
}

// Pass k of the queue schedule on stream s: counters reset, then per group
// of pairs the persistent FP32 kernel and the exact re-decision of the
// group's flagged windows.
int batch_queue_pass_enqueue(opiv_batch* b, int k, cudaStream_t s, int g0 = 0, int g1 = -1)
{
    batch_queue_pass& q = b->qp[k];
    if (g1 < 0) g1 = (int)q.groups.size();
    // CTAs of the persistent grid; 0: the hardware-dispatched list kernel
    const int ctas = q.ctas_per_sm >= 0 ? q.ctas_per_sm : q.max_ctas;
    CUDA_TRY(cudaMemsetAsync(q.d_ctr + 2 * g0, 0, 2 * sizeof(unsigned int) * (g1 - g0), s));
    for (int g = g0; g < g1; ++g) {
        PivQueue& pq = q.groups[g];
        pq.chunk = q.chunk;
        CUDA_TRY(queue_piv_fp32(pq, q.ia, q.dtype, q.mode, q.limit, q.vec, ctas * b->sms, nullptr, s));
        ++g_launches;
        CUDA_TRY(launch_piv_exact_queue(pq, q.ia, q.dtype, q.mode, q.limit, q.exact_blocks, s));
        ++g_launches;
    }
    return OPIV_OK;
}

// The whole chain: one lane on s; several lanes forked from s onto the
// batch's streams, each running all passes of its pairs, joined back into s
// (one lane's exact pass overlaps another lane's FP32 kernel).
int batch_queue_enqueue(opiv_batch* b, cudaStream_t s)
{
    int rc = batch_queue_setup(b);
    if (rc != OPIV_OK) return rc;
    const int L = (int)b->lane_first.size() - 1;
    if (L <= 1) {
        for (int k = 0; k < (int)b->qp.size() && rc == OPIV_OK; ++k) rc = batch_queue_pass_enqueue(b, k, s);
        return rc;
    }
    const int ns = (int)b->streams.size();
    CUDA_TRY(cudaEventRecord(b->events[ns], s));
    for (int l = 0; l < L; ++l) CUDA_TRY(cudaStreamWaitEvent(b->streams[l], b->events[ns], 0));
    for (int k = 0; k < (int)b->qp.size() && rc == OPIV_OK; ++k)
        for (int l = 0; l < L && rc == OPIV_OK; ++l)
            rc = batch_queue_pass_enqueue(b, k, b->streams[l], b->lane_first[l], b->lane_first[l + 1]);
    for (int l = 0; l < L; ++l) {
        CUDA_TRY(cudaEventRecord(b->events[l], b->streams[l]));
        CUDA_TRY(cudaStreamWaitEvent(s, b->events[l], 0));
    }
    return rc;
}

int64_t batch_queue_launches(const opiv_batch* b)
{
    if (b->qp.empty()) return 0;
    return 2 * (int64_t)b->qp[0].groups.size() * (int64_t)b->qp.size();
}

}  // namespace

int opiv_batch_destroy(opiv_batch* b)
{
    if (!b) return OPIV_OK;
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(b->device);
    if (b->main) cudaStreamSynchronize(b->main);
    batch_drop_graph(b);
    batch_free_queue(b);
    for (cudaStream_t st : b->streams) cudaStreamDestroy(st);
    if (b->main) cudaStreamDestroy(b->main);
    if (b->up) cudaStreamDestroy(b->up);
    if (b->down) cudaStreamDestroy(b->down);
    for (cudaEvent_t ev : b->events) cudaEventDestroy(ev);
    for (cudaEvent_t ev : b->ev_up) cudaEventDestroy(ev);
    for (cudaEvent_t ev : b->ev_done) cudaEventDestroy(ev);
    for (void* f : b->d_fa) cudaFree(f);
    for (void* f : b->d_fb) cudaFree(f);
    cudaSetDevice(prev);
    for (opiv_multipass* mp : b->pairs) opiv_multipass_destroy(mp);
    delete b;
    return OPIV_OK;
}

int opiv_batch_create(opiv_batch** out, int n_pairs, const uint32_t* widths, const uint32_t* heights,
                      int dtype, int n_passes, const uint32_t* ia, const uint32_t* step, int mode,
                      int limit_search, int device)
{
    if (!out || n_pairs < 1 || !widths || !heights) return fail(OPIV_ERR_ARG, "invalid batch arguments");
    *out = nullptr;
    opiv_batch* b = new (std::nothrow) opiv_batch;
    if (!b) return fail(OPIV_ERR_ARG, "out of host memory");
    b->device = device;
    for (int i = 0; i < n_pairs; ++i) {
        opiv_multipass* mp = nullptr;
        const int rc = opiv_multipass_create(&mp, widths[i], heights[i], dtype, n_passes, ia, step,
                                             mode, limit_search, device);
        if (rc != OPIV_OK) {
            opiv_batch_destroy(b);
            return rc;
        }
        b->pairs.push_back(mp);
    }
    b->tune_ctas.assign(n_passes, -1);
    b->tune_chunk.assign(n_passes, 1);
    b->tune_ms.assign(n_passes, 0.f);
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(device);
    cudaError_t e = cudaSuccess;
    const int n_streams = n_pairs < 8 ? n_pairs : 8;
    for (int i = 0; i < n_pairs && e == cudaSuccess; ++i) {
        const size_t row = (size_t)widths[i] * px_bytes(dtype);
        void *fa = nullptr, *fb = nullptr;
        if ((e = cudaMalloc(&fa, row * heights[i])) != cudaSuccess) break;
        b->d_fa.push_back(fa);
        if ((e = cudaMalloc(&fb, row * heights[i])) != cudaSuccess) break;
        b->d_fb.push_back(fb);
        b->pitch.push_back(row);
    }
    if (e == cudaSuccess) e = cudaStreamCreate(&b->main);
    for (int i = 0; i < n_streams && e == cudaSuccess; ++i) {
        cudaStream_t st;
        if ((e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking)) != cudaSuccess) break;
        b->streams.push_back(st);
    }
    for (int i = 0; i < n_streams + 1 && e == cudaSuccess; ++i) {
        cudaEvent_t ev;
        if ((e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming)) != cudaSuccess) break;
        b->events.push_back(ev);
    }
    cudaSetDevice(prev);
    if (e != cudaSuccess) {
        opiv_batch_destroy(b);
        return cuda_fail(e, "opiv_batch_create");
    }
    *out = b;
    return OPIV_OK;
}

int opiv_batch_frames(opiv_batch* b, int pair, void** d_frame_a, void** d_frame_b, size_t* pitch_bytes)
{
    if (!b || pair < 0 || pair >= (int)b->pairs.size() || !d_frame_a || !d_frame_b || !pitch_bytes)
        return fail(OPIV_ERR_ARG, "no such pair");
    *d_frame_a = b->d_fa[pair];
    *d_frame_b = b->d_fb[pair];
    *pitch_bytes = b->pitch[pair];
    return OPIV_OK;
}

int opiv_batch_upload(opiv_batch* b, int pair, const void* frame_a, const void* frame_b,
                      size_t pitch_bytes, void* stream)
{
    if (!b || pair < 0 || pair >= (int)b->pairs.size() || !frame_a || !frame_b)
        return fail(OPIV_ERR_ARG, "no such pair");
    const opiv_plan* p0 = b->pairs[pair]->passes[0];
    const size_t row = (size_t)p0->img_w * px_bytes(p0->dtype);
    if (pitch_bytes < row) return fail(OPIV_ERR_ARG, "pitch %zu smaller than a row", pitch_bytes);
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(b->device);
    cudaStream_t s = stream ? (cudaStream_t)stream : b->main;
    cudaError_t e = cudaMemcpy2DAsync(b->d_fa[pair], b->pitch[pair], frame_a, pitch_bytes, row,
                                      p0->img_h, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpy2DAsync(b->d_fb[pair], b->pitch[pair], frame_b, pitch_bytes, row, p0->img_h,
                              cudaMemcpyHostToDevice, s);
    cudaSetDevice(prev);
    return e == cudaSuccess ? OPIV_OK : cuda_fail(e, "opiv_batch_upload");
}

namespace {

// Every pair's pass chain, pairs spread over the fork streams.
int batch_enqueue(opiv_batch* b, cudaStream_t s)
{
    const int ns = (int)b->streams.size();
    CUDA_TRY(cudaEventRecord(b->events[ns], s));
    for (int i = 0; i < ns; ++i) CUDA_TRY(cudaStreamWaitEvent(b->streams[i], b->events[ns], 0));
    for (size_t i = 0; i < b->pairs.size(); ++i) {
        const int rc = opiv_multipass_process_device(b->pairs[i], b->d_fa[i], b->d_fb[i], b->pitch[i],
                                                     b->streams[i % ns]);
        if (rc != OPIV_OK) return rc;
    }
    for (int i = 0; i < ns; ++i) {
        CUDA_TRY(cudaEventRecord(b->events[i], b->streams[i]));
        CUDA_TRY(cudaStreamWaitEvent(s, b->events[i], 0));
    }
    return OPIV_OK;
}

}  // namespace

int opiv_batch_run(opiv_batch* b, int use_graph, void* stream)
{
    if (!b) return fail(OPIV_ERR_ARG, "batch is null");
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(b->device);
    auto done = [&](int st) { cudaSetDevice(prev); return st; };
    cudaStream_t s = stream ? (cudaStream_t)stream : b->main;
    const bool queue = b->schedule == OPIV_BATCH_QUEUE;
    auto enqueue = [&](cudaStream_t st) { return queue ? batch_queue_enqueue(b, st) : batch_enqueue(b, st); };
    if (!use_graph) return done(enqueue(s));
    cudaError_t e;
    if (!b->exec) {
        // one eager run first: one-time kernel attribute set-up happens
        // outside the capture
        int rc = enqueue(s);
        if (rc != OPIV_OK) return done(rc);
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return done(cuda_fail(e, "cudaStreamSynchronize"));
        if ((e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
            return done(cuda_fail(e, "cudaStreamBeginCapture"));
        const int64_t counted = g_launches;   // a capture launches nothing
        rc = enqueue(s);
        g_launches = counted;
        cudaGraph_t g = nullptr;
        e = cudaStreamEndCapture(s, &g);
        if (rc != OPIV_OK) {
            if (g) cudaGraphDestroy(g);
            return done(rc);
        }
        if (e != cudaSuccess) return done(cuda_fail(e, "cudaStreamEndCapture"));
        b->graph = g;
        if ((e = cudaGraphInstantiate(&b->exec, g, 0)) != cudaSuccess)
            return done(cuda_fail(e, "cudaGraphInstantiate"));
        return done(OPIV_OK);   // the eager run has produced this call's results
    }
    if ((e = cudaGraphLaunch(b->exec, s)) != cudaSuccess) return done(cuda_fail(e, "cudaGraphLaunch"));
    g_launches += queue ? batch_queue_launches(b)
                        : 2 * (int64_t)b->pairs.size() * (int64_t)b->pairs[0]->passes.size();
    return done(OPIV_OK);
}

int opiv_batch_set_schedule(opiv_batch* b, int schedule)
{
    if (!b) return fail(OPIV_ERR_ARG, "batch is null");
    if (schedule != OPIV_BATCH_STREAMS && schedule != OPIV_BATCH_QUEUE)
        return fail(OPIV_ERR_ARG, "unknown batch schedule %d", schedule);
    if (schedule == b->schedule) return OPIV_OK;
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(b->device);
    cudaStreamSynchronize(b->main);
    batch_drop_graph(b);
    cudaSetDevice(prev);
    b->schedule = schedule;
    return OPIV_OK;
}

int opiv_batch_set_tuning(opiv_batch* b, int pass, int ctas_per_sm, int chunk)
{
    if (!b) return fail(OPIV_ERR_ARG, "batch is null");
    if (pass < 0 || pass >= (int)b->tune_ctas.size()) return fail(OPIV_ERR_ARG, "no such pass");
    if (ctas_per_sm < 0 || ctas_per_sm > 32) return fail(OPIV_ERR_ARG, "ctas_per_sm %d outside 0 .. 32", ctas_per_sm);
    if (chunk < 1 || chunk > 1024) return fail(OPIV_ERR_ARG, "chunk %d outside 1 .. 1024", chunk);
    b->tune_ctas[pass] = ctas_per_sm;
    b->tune_chunk[pass] = chunk;
    b->tune_ms[pass] = 0.f;
    if (!b->qp.empty()) {
        b->qp[pass].ctas_per_sm = ctas_per_sm;
        b->qp[pass].chunk = chunk;
        b->qp[pass].tuned_ms = 0.f;
    }
    if (b->exec) {
        int prev = 0;
        cudaGetDevice(&prev);
        cudaSetDevice(b->device);
        cudaStreamSynchronize(b->main);
        batch_drop_graph(b);
        cudaSetDevice(prev);
    }
    return OPIV_OK;
}

int opiv_batch_get_tuning(const opiv_batch* b, int pass, int* ctas_per_sm, int* chunk, int* max_ctas_per_sm,
                          float* tuned_ms)
{
    if (!b || !ctas_per_sm || !chunk) return fail(OPIV_ERR_ARG, "null argument");
    if (pass < 0 || pass >= (int)b->tune_ctas.size()) return fail(OPIV_ERR_ARG, "no such pass");
    const int mx = b->qp.empty() ? 0 : b->qp[pass].max_ctas;
    *ctas_per_sm = b->tune_ctas[pass] >= 0 ? b->tune_ctas[pass] : mx;
    *chunk = b->tune_chunk[pass];
    if (max_ctas_per_sm) *max_ctas_per_sm = mx;
    if (tuned_ms) *tuned_ms = b->tune_ms[pass];
    return OPIV_OK;
}

int opiv_batch_set_lanes(opiv_batch* b, int lanes)
{
    if (!b) return fail(OPIV_ERR_ARG, "batch is null");
    if (lanes < 1 || lanes > 8) return fail(OPIV_ERR_ARG, "lanes %d outside 1 .. 8", lanes);
    if (lanes == b->lanes) return OPIV_OK;
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(b->device);
    cudaStreamSynchronize(b->main);
    batch_drop_graph(b);
    batch_free_queue(b);
    cudaSetDevice(prev);
    b->lanes = lanes;
    return OPIV_OK;
}

int opiv_batch_get_lanes(const opiv_batch* b)
{
    if (!b) return fail(OPIV_ERR_ARG, "batch is null");
    const int n = (int)b->pairs.size();
    return std::max(1, std::min({ b->lanes, n, (int)b->streams.size() }));
}

int opiv_batch_autotune(opiv_batch* b, void* stream)
{
    if (!b) return fail(OPIV_ERR_ARG, "batch is null");
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(b->device);
    auto done = [&](int st) { cudaSetDevice(prev); return st; };
    cudaStream_t s = stream ? (cudaStream_t)stream : b->main;
    CUDA_TRY_D(cudaStreamSynchronize(s));
    batch_drop_graph(b);
    b->schedule = OPIV_BATCH_QUEUE;
    int rc = batch_queue_setup(b);
    if (rc != OPIV_OK) return done(rc);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    CUDA_TRY_D(cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return done(fail(OPIV_ERR_CUDA, "cudaEventCreate"));
    }
    static const int kChunks[] = { 1, 2, 4, 8 };
    for (int k = 0; k < (int)b->qp.size() && rc == OPIV_OK; ++k) {
        batch_queue_pass& q = b->qp[k];
        float best = 3.4e38f;
        int best_c = q.max_ctas, best_k = 1;
        const int max_c = q.max_ctas < 4 ? q.max_ctas : 4;
        for (int c = 0; c <= max_c && rc == OPIV_OK; ++c)
            for (int ch : kChunks) {
                if (c == 0 && ch != 1) continue;   // the list kernel has no chunk
                q.ctas_per_sm = c;
                q.chunk = ch;
                float t_min = 3.4e38f;
                for (int r = 0; r < 3 && rc == OPIV_OK; ++r) {   // one warm-up, two timed
                    cudaEventRecord(e0, s);
                    rc = batch_queue_pass_enqueue(b, k, s);
                    cudaEventRecord(e1, s);
                    if (rc != OPIV_OK) break;
                    cudaError_t e = cudaEventSynchronize(e1);
                    if (e != cudaSuccess) {
                        rc = cuda_fail(e, "autotune run");
                        break;
                    }
                    float ms = 0.f;
                    cudaEventElapsedTime(&ms, e0, e1);
                    if (r > 0 && ms < t_min) t_min = ms;
                }
                if (rc != OPIV_OK) break;
                if (t_min < best) {
                    best = t_min;
                    best_c = c;
                    best_k = ch;
                }
            }
        if (rc != OPIV_OK) break;
        q.ctas_per_sm = best_c;
        q.chunk = best_k;
        q.tuned_ms = best;
        b->tune_ctas[k] = best_c;
        b->tune_chunk[k] = best_k;
        b->tune_ms[k] = best;
        // the pass once more with its choice: the next pass reads its offsets
        rc = batch_queue_pass_enqueue(b, k, s);
    }
    // lanes: the whole chain with 1 and 2 lanes (fastest of two timed runs)
    if (rc == OPIV_OK && b->pairs.size() > 1) {
        float best = 3.4e38f;
        int best_l = 1;
        for (int L = 1; L <= 2 && rc == OPIV_OK; ++L) {
            b->lanes = L;
            batch_free_queue(b);
            float t_min = 3.4e38f;
            for (int r = 0; r < 3 && rc == OPIV_OK; ++r) {
                cudaEventRecord(e0, s);
                rc = batch_queue_enqueue(b, s);
                cudaEventRecord(e1, s);
                if (rc != OPIV_OK) break;
                cudaError_t e = cudaEventSynchronize(e1);
                if (e != cudaSuccess) {
                    rc = cuda_fail(e, "autotune run");
                    break;
                }
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                if (r > 0 && ms < t_min) t_min = ms;
            }
            if (t_min < best) {
                best = t_min;
                best_l = L;
            }
        }
        if (rc == OPIV_OK && b->lanes != best_l) {
            b->lanes = best_l;
            batch_free_queue(b);
            rc = batch_queue_enqueue(b, s);   // leaves a normal run's results
        }
    }
    cudaError_t e = cudaStreamSynchronize(s);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc == OPIV_OK && e != cudaSuccess) rc = cuda_fail(e, "cudaStreamSynchronize");
    return done(rc);
}

int opiv_batch_process(opiv_batch* b, const void* const* frames_a, const void* const* frames_b,
                       const size_t* pitch_bytes, opiv_vector* const* out_vec, int32_t* const* out_peak)
{
    if (!b || !frames_a || !frames_b || !pitch_bytes || !out_vec) return fail(OPIV_ERR_ARG, "null argument");
    const int n = (int)b->pairs.size();
    for (int i = 0; i < n; ++i) {
        const opiv_plan* p0 = b->pairs[i]->passes[0];
        if (!frames_a[i] || !frames_b[i] || !out_vec[i] || (out_peak && !out_peak[i]))
            return fail(OPIV_ERR_ARG, "null buffer for pair %d", i);
        if (pitch_bytes[i] < (size_t)p0->img_w * px_bytes(p0->dtype))
            return fail(OPIV_ERR_ARG, "pitch %zu of pair %d smaller than a row", pitch_bytes[i], i);
    }
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(b->device);
    auto done = [&](int st) { cudaSetDevice(prev); return st; };
    cudaError_t e = cudaSuccess;
    if (!b->up) {
        if ((e = cudaStreamCreateWithFlags(&b->up, cudaStreamNonBlocking)) != cudaSuccess ||
            (e = cudaStreamCreateWithFlags(&b->down, cudaStreamNonBlocking)) != cudaSuccess)
            return done(cuda_fail(e, "cudaStreamCreateWithFlags"));
        for (int i = 0; i < n; ++i) {
            cudaEvent_t eu, ed;
            if ((e = cudaEventCreateWithFlags(&eu, cudaEventDisableTiming)) != cudaSuccess)
                return done(cuda_fail(e, "cudaEventCreateWithFlags"));
            b->ev_up.push_back(eu);
            if ((e = cudaEventCreateWithFlags(&ed, cudaEventDisableTiming)) != cudaSuccess)
                return done(cuda_fail(e, "cudaEventCreateWithFlags"));
            b->ev_done.push_back(ed);
        }
    }
    if (b->schedule == OPIV_BATCH_QUEUE) {
        // every pair up, the queue passes (a recorded graph if there is
        // one), every pair's final vectors down; all on the batch's stream
        cudaStream_t s = b->main;
        for (int i = 0; i < n; ++i) {
            const opiv_plan* p0 = b->pairs[i]->passes[0];
            const size_t row = (size_t)p0->img_w * px_bytes(p0->dtype);
            CUDA_TRY_D(cudaMemcpy2DAsync(b->d_fa[i], b->pitch[i], frames_a[i], pitch_bytes[i], row,
                                         p0->img_h, cudaMemcpyHostToDevice, s));
            CUDA_TRY_D(cudaMemcpy2DAsync(b->d_fb[i], b->pitch[i], frames_b[i], pitch_bytes[i], row,
                                         p0->img_h, cudaMemcpyHostToDevice, s));
        }
        if (b->exec) {
            CUDA_TRY_D(cudaGraphLaunch(b->exec, s));
            g_launches += batch_queue_launches(b);
        } else {
            const int rc = batch_queue_enqueue(b, s);
            if (rc != OPIV_OK) {
                cudaStreamSynchronize(s);
                return done(rc);
            }
        }
        for (int i = 0; i < n; ++i) {
            const opiv_plan* pl = b->pairs[i]->passes.back();
            CUDA_TRY_D(cudaMemcpyAsync(out_vec[i], pl->d_vec, sizeof(opiv_vector) * pl->n_win,
                                       cudaMemcpyDeviceToHost, s));
            if (out_peak)
                CUDA_TRY_D(cudaMemcpyAsync(out_peak[i], pl->d_peak, sizeof(int32_t) * pl->n_win,
                                           cudaMemcpyDeviceToHost, s));
        }
        CUDA_TRY_D(cudaStreamSynchronize(s));
        return done(OPIV_OK);
    }
    // work already queued on the batch's stream comes first
    const int ns = (int)b->streams.size();
    CUDA_TRY_D(cudaEventRecord(b->events[ns], b->main));
    CUDA_TRY_D(cudaStreamWaitEvent(b->up, b->events[ns], 0));
    for (int i = 0; i < ns; ++i) CUDA_TRY_D(cudaStreamWaitEvent(b->streams[i], b->events[ns], 0));
    for (int i = 0; i < n; ++i) {
        const opiv_plan* p0 = b->pairs[i]->passes[0];
        const size_t row = (size_t)p0->img_w * px_bytes(p0->dtype);
        CUDA_TRY_D(cudaMemcpy2DAsync(b->d_fa[i], b->pitch[i], frames_a[i], pitch_bytes[i], row, p0->img_h,
                                     cudaMemcpyHostToDevice, b->up));
        CUDA_TRY_D(cudaMemcpy2DAsync(b->d_fb[i], b->pitch[i], frames_b[i], pitch_bytes[i], row, p0->img_h,
                                     cudaMemcpyHostToDevice, b->up));
        CUDA_TRY_D(cudaEventRecord(b->ev_up[i], b->up));
    }
    for (int i = 0; i < n; ++i) {
        cudaStream_t cs = b->streams[i % ns];
        CUDA_TRY_D(cudaStreamWaitEvent(cs, b->ev_up[i], 0));
        const int rc = opiv_multipass_process_device(b->pairs[i], b->d_fa[i], b->d_fb[i], b->pitch[i], cs);
        if (rc != OPIV_OK) {
            cudaDeviceSynchronize();
            return done(rc);
        }
        CUDA_TRY_D(cudaEventRecord(b->ev_done[i], cs));
        const opiv_plan* pl = b->pairs[i]->passes.back();
        CUDA_TRY_D(cudaStreamWaitEvent(b->down, b->ev_done[i], 0));
        CUDA_TRY_D(cudaMemcpyAsync(out_vec[i], pl->d_vec, sizeof(opiv_vector) * pl->n_win,
                                   cudaMemcpyDeviceToHost, b->down));
        if (out_peak)
            CUDA_TRY_D(cudaMemcpyAsync(out_peak[i], pl->d_peak, sizeof(int32_t) * pl->n_win,
                                       cudaMemcpyDeviceToHost, b->down));
    }
    if ((e = cudaStreamSynchronize(b->down)) != cudaSuccess) return done(cuda_fail(e, "cudaStreamSynchronize"));
    // the fork streams have finished too (every pair's download waited on them)
    return done(OPIV_OK);
}

int64_t opiv_batch_window_count(const opiv_batch* b, int pair, int pass)
{
    if (!b || pair < 0 || pair >= (int)b->pairs.size()) return fail(OPIV_ERR_ARG, "no such pair");
    return opiv_multipass_window_count(b->pairs[pair], pass);
}

int opiv_batch_results(opiv_batch* b, int pair, int pass, opiv_vector* out_vec, int32_t* out_peak,
                       int32_t* out_disp)
{
    if (!b || pair < 0 || pair >= (int)b->pairs.size()) return fail(OPIV_ERR_ARG, "no such pair");
    return opiv_multipass_results(b->pairs[pair], pass, out_vec, out_peak, out_disp);
}

namespace {
// whether the plan's tensor-core kernel has a choice of tile shape
bool tile_choice(const opiv_plan* p)
{
    return is_tc(p->precision) && p->ia == 32 && p->dy <= 8;
}
}  // namespace

int opiv_plan_test_mma_timeout(opiv_plan* plan, int on)
{
    if (!plan) return fail(OPIV_ERR_ARG, "plan is null");
    if (!is_tc(plan->precision) || plan->ia != 32)
        return fail(OPIV_ERR_UNSUPPORTED, "the MMA-timeout test needs a 32 px tensor-core plan");
    plan->mma_skip = on ? 1 : 0;
    return OPIV_OK;
}

int opiv_plan_set_tile(opiv_plan* plan, int tile)
{
    if (!plan) return fail(OPIV_ERR_ARG, "plan is null");
    if (tile != OPIV_TILE_AUTO && tile != OPIV_TILE_VERTICAL && tile != OPIV_TILE_HORIZONTAL)
        return fail(OPIV_ERR_ARG, "unknown tile shape %d", tile);
    plan->tc_tile = tile;
    return OPIV_OK;
}

int opiv_plan_get_tile(const opiv_plan* plan)
{
    if (!plan) return fail(OPIV_ERR_ARG, "plan is null");
    if (!is_tc(plan->precision) || plan->ia != 32) return OPIV_TILE_AUTO;
    return (tile_choice(plan) && plan->tc_tile != OPIV_TILE_HORIZONTAL) ? OPIV_TILE_VERTICAL
                                                                        : OPIV_TILE_HORIZONTAL;
}

int opiv_plan_autotune(opiv_plan* plan, const void* d_fa, const void* d_fb, size_t pitch_bytes, void* stream)
{
    if (!plan || !d_fa || !d_fb) return fail(OPIV_ERR_ARG, "null argument");
    if (!tile_choice(plan)) return OPIV_OK;   // one shape only
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(plan->device);
    auto done = [&](int st) { cudaSetDevice(prev); return st; };
    cudaStream_t s = (cudaStream_t)stream;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    CUDA_TRY_D(cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return done(fail(OPIV_ERR_CUDA, "cudaEventCreate"));
    }
    const bool timing = plan->timing;
    plan->timing = false;
    int rc = OPIV_OK, best = OPIV_TILE_VERTICAL;
    float best_ms = 3.4e38f;
    for (int tile : { OPIV_TILE_VERTICAL, OPIV_TILE_HORIZONTAL }) {
        plan->tc_tile = tile;
        float t_min = 3.4e38f;
        for (int r = 0; r < 4 && rc == OPIV_OK; ++r) {   // one warm-up, three timed
            cudaEventRecord(e0, s);
            rc = run_pass(plan, d_fa, d_fb, pitch_bytes, plan->d_vec, plan->d_peak, s);
            cudaEventRecord(e1, s);
            if (rc != OPIV_OK) break;
            const cudaError_t e = cudaEventSynchronize(e1);
            if (e != cudaSuccess) {
                rc = cuda_fail(e, "autotune run");
                break;
            }
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (r > 0 && ms < t_min) t_min = ms;
        }
        if (rc != OPIV_OK) break;
        if (t_min < best_ms) {
            best_ms = t_min;
            best = tile;
        }
    }
    plan->timing = timing;
    plan->tc_tile = best;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc == OPIV_OK && plan->d_status) rc = opiv_plan_status(plan);
    return done(rc);
}

int opiv_plan_adjoint(opiv_plan* plan, const void* d_fa, const void* d_fb, size_t pitch_bytes,
                      const int32_t* d_peak, const float* d_cotangent, float* d_grad_a,
                      float* d_grad_b, size_t grad_pitch_bytes, float var_a, float var_b,
                      float* d_sigma, void* stream)
{
    if (!plan || !d_fa || !d_fb || !d_peak) return fail(OPIV_ERR_ARG, "null argument");
    if (d_cotangent && (!d_grad_a || !d_grad_b))
        return fail(OPIV_ERR_ARG, "a cotangent needs both gradient images");
    if (d_cotangent && (grad_pitch_bytes % sizeof(float) != 0 ||
                        grad_pitch_bytes < sizeof(float) * plan->img_w))
        return fail(OPIV_ERR_ARG, "gradient pitch %zu too small or not a multiple of 4", grad_pitch_bytes);
    if (!is_pow2(plan->ia))
        return fail(OPIV_ERR_NOT_POW2, "dimensions must be power of 2: %ux%u", plan->ia, plan->ia);
    if (pitch_bytes < (size_t)plan->img_w * px_bytes(plan->dtype) ||
        pitch_bytes % px_bytes(plan->dtype) != 0)
        return fail(OPIV_ERR_ARG, "pitch %zu too small or not a multiple of the pixel size", pitch_bytes);
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(plan->device);
    PivParams k = base_params(plan);
    k.fa = d_fa;
    k.fb = d_fb;
    k.pitch = pitch_bytes;
    const cudaError_t e = launch_piv_adjoint(k, (int)plan->ia, plan->dtype, plan->mode, d_peak, d_cotangent,
                                             d_grad_a, d_grad_b, grad_pitch_bytes / sizeof(float),
                                             var_a, var_b, d_sigma, (cudaStream_t)stream);
    cudaSetDevice(prev);
    if (e != cudaSuccess) return cuda_fail(e, "opiv_plan_adjoint");
    ++g_launches;
    return OPIV_OK;
}

int opiv_plan_set_precision(opiv_plan* plan, int precision)
{
    if (!plan) return fail(OPIV_ERR_ARG, "plan is null");
    if (precision < OPIV_PREC_FP32 || precision > OPIV_PREC_TC_SPLIT2_FP16)
        return fail(OPIV_ERR_ARG, "unknown precision %d", precision);
    if (!is_tc(precision) && !is_pow2(plan->ia))
        return fail(OPIV_ERR_NOT_POW2, "dimensions must be power of 2: %ux%u", plan->ia, plan->ia);
    if (is_tc(precision)) {
        if (!tc_supports((int)plan->ia, plan->dtype))
            return fail(OPIV_ERR_UNSUPPORTED,
                        "the tensor-core path takes 16, 32, 48 or 64 px windows of u8/u16 frames");
        if (plan->ia == 32 && (plan->g.xs % 8 != 0 || plan->dx % 8 != 0))
            return fail(OPIV_ERR_UNSUPPORTED,
                        "the 32 px tensor-core path needs window x positions on multiples of 8 pixels");
        if (!plan->d_tc) {
            int prev = 0;
            cudaGetDevice(&prev);
            cudaSetDevice(plan->device);
            std::vector<unsigned char> host(tc_constant_bytes((int)plan->ia));
            tc_constants((int)plan->ia, host.data());
            cudaError_t e = cudaMalloc(&plan->d_tc, host.size());
            if (e == cudaSuccess)
                e = cudaMemcpy(plan->d_tc, host.data(), host.size(), cudaMemcpyHostToDevice);
            if (e == cudaSuccess) e = cudaMalloc(&plan->d_status, sizeof(int));
            if (e == cudaSuccess) e = cudaMemset(plan->d_status, 0, sizeof(int));
            cudaSetDevice(prev);
            if (e != cudaSuccess) return cuda_fail(e, "tensor-core set-up");
        }
    }
    plan->precision = precision;
    return OPIV_OK;
}

int opiv_plan_status(opiv_plan* plan)
{
    if (!plan) return fail(OPIV_ERR_ARG, "plan is null");
    if (!plan->d_status) return OPIV_OK;
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(plan->device);
    int h = 0;
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(&h, plan->d_status, sizeof(int), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && h) e = cudaMemset(plan->d_status, 0, sizeof(int));
    cudaSetDevice(prev);
    if (e != cudaSuccess) return cuda_fail(e, "opiv_plan_status");
    return h ? fail(OPIV_ERR_TIMEOUT, "a tensor-core pass gave up waiting for its MMAs") : OPIV_OK;
}

int opiv_plan_set_plane_output(opiv_plan* plan, float* d_planes, double* d_pedestals)
{
    if (!plan) return fail(OPIV_ERR_ARG, "plan is null");
    plan->d_planes = d_planes;
    plan->d_peds = d_pedestals;
    return OPIV_OK;
}

int opiv_plan_set_timing(opiv_plan* plan, int enable)
{
    if (!plan) return fail(OPIV_ERR_ARG, "plan is null");
    if (enable && !plan->ev[0]) {
        int prev = 0;
        cudaGetDevice(&prev);
        cudaSetDevice(plan->device);
        for (cudaEvent_t& e : plan->ev) {
            const cudaError_t r = cudaEventCreate(&e);
            if (r != cudaSuccess) {
                cudaSetDevice(prev);
                return cuda_fail(r, "cudaEventCreate");
            }
        }
        cudaSetDevice(prev);
    }
    plan->timing = enable != 0;
    return OPIV_OK;
}

int opiv_plan_last_timing(opiv_plan* plan, float* fp32_ms, float* exact_ms)
{
    if (!plan || !fp32_ms || !exact_ms) return fail(OPIV_ERR_ARG, "null argument");
    if (!plan->timing) return fail(OPIV_ERR_ARG, "timing is not enabled on this plan");
    CUDA_TRY(cudaEventSynchronize(plan->ev[2]));
    CUDA_TRY(cudaEventElapsedTime(fp32_ms, plan->ev[0], plan->ev[1]));
    CUDA_TRY(cudaEventElapsedTime(exact_ms, plan->ev[1], plan->ev[2]));
    return OPIV_OK;
}

int opiv_cross_correlate_batch(const double* a, const double* b, uint32_t w, int64_t n, int mode,
                               int exact, double* out_planes, int device)
{
    if (!a || !b || !out_planes || n < 0) return fail(OPIV_ERR_ARG, "null argument");
    if (mode < OPIV_CORR_REAL || mode > OPIV_CORR_POCKET_REAL)
        return fail(OPIV_ERR_ARG, "unknown correlation mode %d", mode);
    mode = kernel_mode(mode);
    if (!is_pow2(w)) return fail(OPIV_ERR_NOT_POW2, "dimensions must be power of 2: %ux%u", w, w);
    if (exact ? !exact_supports((int)w) : !fp32_supports((int)w))
        return fail(OPIV_ERR_UNSUPPORTED, "no kernel for %ux%u windows", w, w);
    // the windows are stacked as rows of one frame, indexed in 32 bits
    if (n > (int64_t)INT32_MAX / (int64_t)w)
        return fail(OPIV_ERR_CAPACITY, "%lld windows of %u rows: at most 2^31 - 1 rows in one call", (long long)n, w);
    if (n == 0) return OPIV_OK;
    int prev = 0;
    cudaGetDevice(&prev);
    if (cudaSetDevice(device) != cudaSuccess) return fail(OPIV_ERR_NO_DEVICE, "cannot use device %d", device);
    const size_t N = (size_t)w * w;
    // The windows are stacked into one w x (n*w) double "frame"; window k
    // sits at (0, k*w).
    double *d_a = nullptr, *d_b = nullptr, *d_pl64 = nullptr, *d_peds = nullptr;
    float* d_pl = nullptr;
    int32_t* d_xy = nullptr;
    opiv_vector* d_vec = nullptr;
    double2* d_tw = nullptr;
    std::vector<int32_t> xy(2 * n);
    for (int64_t k = 0; k < n; ++k) { xy[2 * k] = 0; xy[2 * k + 1] = (int32_t)(k * w); }
    int rc = OPIV_OK;
    cudaError_t e = cudaSuccess;
    do {
        if ((e = cudaMalloc(&d_a, sizeof(double) * N * n)) != cudaSuccess) break;
        if ((e = cudaMalloc(&d_b, sizeof(double) * N * n)) != cudaSuccess) break;
        if ((e = cudaMalloc(&d_xy, sizeof(int32_t) * 2 * n)) != cudaSuccess) break;
        if ((e = cudaMalloc(&d_vec, sizeof(opiv_vector) * n)) != cudaSuccess) break;
        if ((e = cudaMemcpy(d_a, a, sizeof(double) * N * n, cudaMemcpyHostToDevice)) != cudaSuccess) break;
        if ((e = cudaMemcpy(d_b, b, sizeof(double) * N * n, cudaMemcpyHostToDevice)) != cudaSuccess) break;
        if ((e = cudaMemcpy(d_xy, xy.data(), sizeof(int32_t) * 2 * n, cudaMemcpyHostToDevice)) != cudaSuccess) break;
        PivParams k;
        k.fa = d_a;
        k.fb = d_b;
        k.pitch = sizeof(double) * w;
        k.img_w = (int)w;
        k.img_h = (int)(w * n);
        k.win_xy = d_xy;
        k.n_win = n;
        k.out_vec = d_vec;
        if (exact) {
            std::vector<double2> tw = reference_twiddles(w, -1), tr = reference_twiddles(w, +1);
            tw.insert(tw.end(), tr.begin(), tr.end());
            if ((e = cudaMalloc(&d_tw, sizeof(double2) * tw.size())) != cudaSuccess) break;
            if ((e = cudaMemcpy(d_tw, tw.data(), sizeof(double2) * tw.size(), cudaMemcpyHostToDevice)) != cudaSuccess) break;
            if ((e = cudaMalloc(&d_pl64, sizeof(double) * N * n)) != cudaSuccess) break;
            k.tw_fwd = d_tw;
            k.tw_rev = d_tw + w;
            k.planes64 = d_pl64;
            const int blocks = (int)std::min<int64_t>(n, 4096);
            if ((e = launch_piv_exact(k, (int)w, kF64, mode, 0, false, blocks, nullptr)) != cudaSuccess) break;
            ++g_launches;
            if ((e = cudaMemcpy(out_planes, d_pl64, sizeof(double) * N * n, cudaMemcpyDeviceToHost)) != cudaSuccess) break;
        } else {
            if ((e = cudaMalloc(&d_pl, sizeof(float) * N * n)) != cudaSuccess) break;
            if ((e = cudaMalloc(&d_peds, sizeof(double) * n)) != cudaSuccess) break;
            k.planes = d_pl;
            k.peds = d_peds;
            if ((e = launch_piv_fp32(k, (int)w, kF64, mode, 0, true, nullptr)) != cudaSuccess) break;
            ++g_launches;
            std::vector<float> pl(N * n);
            std::vector<double> peds(n);
            if ((e = cudaMemcpy(pl.data(), d_pl, sizeof(float) * N * n, cudaMemcpyDeviceToHost)) != cudaSuccess) break;
            if ((e = cudaMemcpy(peds.data(), d_peds, sizeof(double) * n, cudaMemcpyDeviceToHost)) != cudaSuccess) break;
            for (int64_t q = 0; q < n; ++q)
                for (size_t i = 0; i < N; ++i)
                    out_planes[q * N + i] = (double)pl[q * N + i] + peds[q];
        }
        e = cudaDeviceSynchronize();
    } while (0);
    if (e != cudaSuccess) rc = cuda_fail(e, "opiv_cross_correlate_batch");
    cudaFree(d_a);
    cudaFree(d_b);
    cudaFree(d_pl64);
    cudaFree(d_peds);
    cudaFree(d_pl);
    cudaFree(d_xy);
    cudaFree(d_vec);
    cudaFree(d_tw);
    cudaSetDevice(prev);
    return rc;
}

// FFT::transform / transform_real / auto_correlate on a batch of windows
// (fft.h:87-186, :229-242): host buffers, the exact double kernel, one CTA
// per window.  in_c / out_* are interleaved complex (re, im) doubles.
static int spectral_batch(int op, const double* in_c, const double* in_ra, const double* in_rb,
                          uint32_t w, int64_t n, int direction, double* out_a, double* out_b,
                          int device, const char* name)
{
    if (n < 0) return fail(OPIV_ERR_ARG, "%s: negative window count", name);
    if (direction != OPIV_FORWARD && direction != OPIV_REVERSE)
        return fail(OPIV_ERR_ARG, "%s: unknown direction %d", name, direction);
    if (!is_pow2(w)) return fail(OPIV_ERR_NOT_POW2, "dimensions must be power of 2: %ux%u", w, w);
    if (!exact_supports((int)w)) return fail(OPIV_ERR_UNSUPPORTED, "no kernel for %ux%u windows", w, w);
    if (n == 0) return OPIV_OK;
    int prev = 0;
    cudaGetDevice(&prev);
    if (cudaSetDevice(device) != cudaSuccess) return fail(OPIV_ERR_NO_DEVICE, "cannot use device %d", device);
    const size_t N = (size_t)w * w * n;
    double2 *d_in = nullptr, *d_oa = nullptr, *d_ob = nullptr, *d_tw = nullptr;
    double *d_ra = nullptr, *d_rb = nullptr;
    int rc = OPIV_OK;
    cudaError_t e = cudaSuccess;
    do {
        std::vector<double2> tw = reference_twiddles(w, direction == OPIV_REVERSE ? +1 : -1);
        if (op == kSpectralAuto) {
            const std::vector<double2> tr = reference_twiddles(w, +1);
            tw = reference_twiddles(w, -1);
            tw.insert(tw.end(), tr.begin(), tr.end());
        }
        if ((e = cudaMalloc(&d_tw, sizeof(double2) * tw.size())) != cudaSuccess) break;
        if ((e = cudaMemcpy(d_tw, tw.data(), sizeof(double2) * tw.size(), cudaMemcpyHostToDevice)) != cudaSuccess) break;
        if ((e = cudaMalloc(&d_oa, sizeof(double2) * N)) != cudaSuccess) break;
        SpectralParams q;
        q.w = (int)w;
        q.n = n;
        q.tw = d_tw;
        q.out_a = d_oa;
        if (op == kSpectralReal) {
            if ((e = cudaMalloc(&d_ob, sizeof(double2) * N)) != cudaSuccess) break;
            if ((e = cudaMalloc(&d_ra, sizeof(double) * N)) != cudaSuccess) break;
            if ((e = cudaMalloc(&d_rb, sizeof(double) * N)) != cudaSuccess) break;
            if ((e = cudaMemcpy(d_ra, in_ra, sizeof(double) * N, cudaMemcpyHostToDevice)) != cudaSuccess) break;
            if ((e = cudaMemcpy(d_rb, in_rb, sizeof(double) * N, cudaMemcpyHostToDevice)) != cudaSuccess) break;
            q.in_ra = d_ra;
            q.in_rb = d_rb;
            q.out_b = d_ob;
        } else {
            if ((e = cudaMalloc(&d_in, sizeof(double2) * N)) != cudaSuccess) break;
            if ((e = cudaMemcpy(d_in, in_c, sizeof(double2) * N, cudaMemcpyHostToDevice)) != cudaSuccess) break;
            q.in_c = d_in;
        }
        const int blocks = (int)std::min<int64_t>(n, 8 * (int64_t)device_sm_count(device));
        if ((e = launch_spectral_exact(q, op, blocks, nullptr)) != cudaSuccess) break;
        ++g_launches;
        if ((e = cudaMemcpy(out_a, d_oa, sizeof(double2) * N, cudaMemcpyDeviceToHost)) != cudaSuccess) break;
        if (op == kSpectralReal &&
            (e = cudaMemcpy(out_b, d_ob, sizeof(double2) * N, cudaMemcpyDeviceToHost)) != cudaSuccess)
            break;
        e = cudaDeviceSynchronize();
    } while (0);
    if (e != cudaSuccess) rc = cuda_fail(e, name);
    cudaFree(d_in);
    cudaFree(d_oa);
    cudaFree(d_ob);
    cudaFree(d_tw);
    cudaFree(d_ra);
    cudaFree(d_rb);
    cudaSetDevice(prev);
    return rc;
}

int opiv_transform_batch(const double* in, uint32_t w, int64_t n, int direction, double* out,
                         int device)
{
    if (!in || !out) return fail(OPIV_ERR_ARG, "null argument");
    return spectral_batch(kSpectralTransform, in, nullptr, nullptr, w, n, direction, out, nullptr, device,
                          "opiv_transform_batch");
}

int opiv_transform_real_batch(const double* a, const double* b, uint32_t w, int64_t n, int direction,
                              double* out_a, double* out_b, int device)
{
    if (!a || !b || !out_a || !out_b) return fail(OPIV_ERR_ARG, "null argument");
    return spectral_batch(kSpectralReal, nullptr, a, b, w, n, direction, out_a, out_b, device,
                          "opiv_transform_real_batch");
}

int opiv_auto_correlate_batch(const double* in, uint32_t w, int64_t n, double* out, int device)
{
    if (!in || !out) return fail(OPIV_ERR_ARG, "null argument");
    return spectral_batch(kSpectralAuto, in, nullptr, nullptr, w, n, OPIV_FORWARD, out, nullptr, device,
                          "opiv_auto_correlate_batch");
}

// The 3-point Gaussian offsets of fit_simple_gaussian (image_utils.impl.h:
// 86-98) on a 3 x 3 block, row-major: the caller adds them to its view's
// midpoint, as the reference does.
int opiv_gaussian_offsets(const double* v9, double* out_fxfy)
{
    if (!v9 || !out_fxfy) return fail(OPIV_ERR_ARG, "null argument");
    auto f = [](double l, double c, double r) {
        const double num = std::log(l) - std::log(r);
        const double den = 2.0 * (std::log(l) + std::log(r) - 2.0 * std::log(c));
        if (den == 0.0) return 0.0;
        return num / den;
    };
    out_fxfy[0] = f(v9[3], v9[4], v9[5]);
    out_fxfy[1] = f(v9[1], v9[4], v9[7]);
    return OPIV_OK;
}

// core::find_peaks, image_utils.impl.h:42-74 (host).  The sort is the
// reference's: std::sort, descending by centre value.
int opiv_find_peaks(const double* im, uint32_t w, uint32_t h, uint16_t num_peaks, uint32_t r,
                    int32_t* out_xy, double* out_value)
{
    if (!im || !out_xy || !out_value) return fail(OPIV_ERR_ARG, "null argument");
    struct pk { double v; int32_t x, y; };
    std::vector<pk> res;
    for (uint32_t y = r; y < h - 2 * r; ++y) {
        const double* above = im + (size_t)(y - 1) * w;
        const double* line = im + (size_t)y * w;
        const double* below = im + (size_t)(y + 1) * w;
        for (uint32_t x = r; x < w - r; ++x)
            if (line[x - 1] < line[x] && line[x + 1] < line[x] && above[x] < line[x] &&
                below[x] < line[x])
                res.push_back(pk{ line[x], (int32_t)x, (int32_t)y });
    }
    std::sort(res.begin(), res.end(), [](const pk& p, const pk& q) { return p.v > q.v; });
    const size_t n = std::min(res.size(), (size_t)num_peaks);
    for (size_t i = 0; i < n; ++i) {
        out_xy[2 * i] = res[i].x;
        out_xy[2 * i + 1] = res[i].y;
        out_value[i] = res[i].v;
    }
    return (int)n;
}

// core::fit_simple_gaussian on the 3x3 view centred at (px, py):
// image_utils.impl.h:77-101 (host).
int opiv_fit_simple_gaussian(const double* plane, uint32_t w, uint32_t h, int32_t px, int32_t py,
                             double* out_xy)
{
    if (!plane || !out_xy) return fail(OPIV_ERR_ARG, "null argument");
    if (px < 1 || py < 1 || (uint32_t)px + 1 >= w || (uint32_t)py + 1 >= h)
        return fail(OPIV_ERR_ARG, "fit_simple_gaussian: input must be 3x3");
    auto f = [](double l, double c, double r) {
        const double num = std::log(l) - std::log(r);
        const double den = 2.0 * (std::log(l) + std::log(r) - 2.0 * std::log(c));
        if (den == 0.0) return 0.0;
        return num / den;
    };
    const double* row = plane + (size_t)py * w;
    out_xy[0] = (double)px + f(row[px - 1], row[px], row[px + 1]);
    out_xy[1] = (double)py + f(plane[(size_t)(py - 1) * w + px], row[px], plane[(size_t)(py + 1) * w + px]);
    return OPIV_OK;
}

}  // extern "C"
