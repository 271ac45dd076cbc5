// noalloc.cu -- opiv_process_pair_device_noalloc: a whole PIV pass over one
// image pair that allocates no memory.
//
// Who needs it.  The plan-based calls allocate their device scratch (the
// list of windows handed to the exact pass, the twiddle tables) when the plan
// is created.  Some callers cannot allocate at all: a frame-grabber or
// real-time acquisition loop whose memory budget is fixed at start-up and
// that must not call cudaMalloc once it is running; a host application or
// plugin framework that owns the device allocator and forbids libraries to
// allocate behind its back; code that must not risk the synchronisation a
// cudaMalloc / cudaFree can cause in the middle of a stream.  This entry
// point takes the caller's device frames and output buffers and keeps its own
// scratch in one statically sized device array instead.
//
// The scratch.  g_noalloc_scratch below is a file-scope __device__ array of
// kScratchBytes (about 4 MiB): a window counter, room for the indices of up
// to kNoAllocMaxWindows windows, and the double-precision twiddle tables the
// exact pass needs.  Every GPU that loads this library holds the array until
// the process exits.  In host code its name is only a host-side stand-in, so
// the host obtains its device address with cudaGetSymbolAddress, once per
// device, and passes that address to the kernels.
//
// Limits and rules.
//   * At most kNoAllocMaxWindows windows per call (every grid of a 4096^2
//     image down to 16 x 16 windows at step 4 fits); larger requests are
//     rejected with OPIV_ERR_CAPACITY before anything runs.
//   * 16 and 32 px windows only (the twiddle tables of the exact pass are
//     sized for those two); 64 px windows are refused with
//     OPIV_ERR_UNSUPPORTED.  All four correlation modes are taken; the
//     PocketFFT modes run the COMPLEX kernels, as the plan path does.
//   * The set-up is not repeated: after a cudaDeviceReset (or any teardown
//     of the device's primary context) the cached address and the uploaded
//     tables are stale, so the entry point must not be used again in that
//     process.
//   * The first call on a device performs the set-up (symbol address lookup
//     and a synchronous upload of the twiddle tables).  Make that first call
//     before any stream capture begins.
//   * All calls share the one array and it keeps the last call's contents.
//     The counter is cleared at the start of every call; the list and
//     tables are rewritten or unchanged.  Two calls whose work overlaps on
//     the GPU (different streams, or different host threads without
//     ordering) race on the array: order them on one stream.

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <mutex>
#include <vector>

#include <cuda_runtime.h>

#include "openpiv_gb300.h"
#include "piv_kernels.h"

using namespace opiv;

namespace {

constexpr int64_t kNoAllocMaxWindows = 1 << 20;
// byte layout of the scratch array
constexpr size_t kOffCount = 0;                                   // unsigned int
constexpr size_t kOffList = 256;                                  // int32 x max windows
constexpr size_t kOffTw16 = kOffList + 4 * (size_t)kNoAllocMaxWindows;   // double2 x 2*16
constexpr size_t kOffTw32 = kOffTw16 + sizeof(double2) * 2 * 16;          // double2 x 2*32
constexpr size_t kScratchBytes = kOffTw32 + sizeof(double2) * 2 * 32;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Same calibration as the plan-based path: error-bound factor of the FP32
// kernel; the exact pass runs two CTAs per SM.
constexpr float kNoAllocKappa = 8.0f;

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
unsigned char* g_scratch_ptr[kMaxDevices] = {};

int na_fail(int status, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    return record_error(status, buf);
}

// twiddle table as the reference builds it (fft.h:274-294)
void reference_table(uint32_t n, int dir, double2* out)
{
    const double s = dir < 0 ? -1.0 : 1.0;
    for (uint32_t i = 0; i < n; ++i) {
        const double theta = (s * M_PI * (double)(int)i) / (double)n;
        out[i] = make_double2(std::cos(theta), std::sin(theta));
    }
}

// Once per device, with that device current: the scratch's device address
// and the twiddle tables.  Returns the address or nullptr (error recorded).
unsigned char* scratch_for_device(int device)
{
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (g_scratch_ptr[device]) return g_scratch_ptr[device];
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess) {
        na_fail(OPIV_ERR_CUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
        return nullptr;
    }
    double2 tw[2 * 16 + 2 * 32];
    reference_table(16, -1, tw);
    reference_table(16, +1, tw + 16);
    reference_table(32, -1, tw + 32);
    reference_table(32, +1, tw + 64);
    e = cudaMemcpy(static_cast<unsigned char*>(ptr) + kOffTw16, tw, sizeof tw, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        na_fail(OPIV_ERR_CUDA, "uploading twiddle tables: %s", cudaGetErrorString(e));
        return nullptr;
    }
    g_scratch_ptr[device] = static_cast<unsigned char*>(ptr);
    return g_scratch_ptr[device];
}

size_t pixel_bytes(int dtype)
{
    switch (dtype) {
    case OPIV_U8: return 1;
    case OPIV_U16: return 2;
    case OPIV_F32: return 4;
    default: return 0;
    }
}

}  // namespace

extern "C" int opiv_process_pair_device_noalloc(const void* d_frame_a, const void* d_frame_b,
                                                size_t pitch_bytes, uint32_t img_w, uint32_t img_h,
                                                int dtype, uint32_t ia, uint32_t dx, uint32_t dy,
                                                int mode, int limit_search, opiv_vector* d_out_vec,
                                                int32_t* d_out_peak, void* stream)
{
    if (!d_frame_a || !d_frame_b || !d_out_vec) return na_fail(OPIV_ERR_ARG, "null argument");
    const size_t px = pixel_bytes(dtype);
    if (px == 0) return na_fail(OPIV_ERR_ARG, "unknown pixel type %d", dtype);
    if (mode != OPIV_CORR_REAL && mode != OPIV_CORR_COMPLEX && mode != OPIV_CORR_POCKET &&
        mode != OPIV_CORR_POCKET_REAL)
        return na_fail(OPIV_ERR_ARG, "unknown correlation mode %d", mode);
    // the PocketFFT modes are the true circular correlation: COMPLEX kernels
    if (mode != OPIV_CORR_REAL) mode = OPIV_CORR_COMPLEX;
    // grid checks and geometry as generate_cartesian_grid (grid.impl.h:29-48)
    if ((uint64_t)img_w * img_h == 0) return na_fail(OPIV_ERR_IMAGE_EMPTY, "image size must be non-zero");
    if (ia == 0) return na_fail(OPIV_ERR_IA_EMPTY, "interrogation size must be non-zero");
    if (dx == 0 || dy == 0) return na_fail(OPIV_ERR_OFFSET_ZERO, "offsets must be non-zero");
    if (ia > img_w || ia > img_h)
        return na_fail(OPIV_ERR_IA_TOO_BIG, "interrogation size is bigger than image");
    if ((ia & (ia - 1)) != 0)
        return na_fail(OPIV_ERR_NOT_POW2, "dimensions must be power of 2: %ux%u", ia, ia);
    if (ia != 16 && ia != 32)
        return na_fail(OPIV_ERR_UNSUPPORTED, "no kernel for %ux%u windows", ia, ia);
    if (pitch_bytes < (size_t)img_w * px || pitch_bytes % px != 0)
        return na_fail(OPIV_ERR_ARG, "pitch %zu too small or not a multiple of the pixel size",
                       pitch_bytes);
    const uint32_t xc = 1 + (img_w - ia) / dx;
    const uint32_t yc = 1 + (img_h - ia) / dy;
    const int64_t n = (int64_t)xc * yc;
    if (n > kNoAllocMaxWindows)
        return na_fail(OPIV_ERR_CAPACITY,
                       "opiv_process_pair_device_noalloc: %lld windows exceed the fixed scratch "
                       "of %lld windows; use a plan (opiv_plan_create) for this grid",
                       (long long)n, (long long)kNoAllocMaxWindows);

    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) return na_fail(OPIV_ERR_NO_DEVICE, "no CUDA device: %s", cudaGetErrorString(e));
    if (device < 0 || device >= kMaxDevices) return na_fail(OPIV_ERR_ARG, "device %d not supported", device);
    unsigned char* scratch = scratch_for_device(device);
    if (!scratch) return OPIV_ERR_CUDA;

    PivParams k;
    k.fa = d_frame_a;
    k.fb = d_frame_b;
    k.pitch = pitch_bytes;
    k.img_w = (int)img_w;
    k.img_h = (int)img_h;
    k.gx0 = (int)((img_w - ia - dx * (xc - 1)) / 2);
    k.gy0 = (int)((img_h - ia - dy * (yc - 1)) / 2);
    k.gdx = (int)dx;
    k.gdy = (int)dy;
    k.gnx = (int)xc;
    k.n_win = n;
    k.out_vec = d_out_vec;
    k.out_peak = d_out_peak;
    k.kappa = kNoAllocKappa;
    k.flag_count = reinterpret_cast<unsigned int*>(scratch + kOffCount);
    k.flag_list = reinterpret_cast<int32_t*>(scratch + kOffList);
    const double2* tw = reinterpret_cast<const double2*>(scratch + (ia == 16 ? kOffTw16 : kOffTw32));
    k.tw_fwd = tw;
    k.tw_rev = tw + ia;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if ((e = cudaMemsetAsync(scratch + kOffCount, 0, sizeof(unsigned int), s)) != cudaSuccess)
        return na_fail(OPIV_ERR_CUDA, "clearing the scratch counter: %s", cudaGetErrorString(e));
    if ((e = launch_piv_fp32(k, (int)ia, dtype, mode, limit_search ? 1 : 0, false, s)) != cudaSuccess)
        return na_fail(OPIV_ERR_CUDA, "FP32 pass: %s", cudaGetErrorString(e));
    if ((e = launch_piv_exact(k, (int)ia, dtype, mode, limit_search ? 1 : 0, true,
                              2 * device_sm_count(device), s)) != cudaSuccess)
        return na_fail(OPIV_ERR_CUDA, "exact pass: %s", cudaGetErrorString(e));
    return OPIV_OK;
}
