// fft_reg.cuh -- radix-2 FFTs held entirely in one thread's registers.
//
// A thread owns N complex values (float2 v[N]) and transforms them without
// touching memory: every loop is fully unrolled, so array indices and twiddle
// indices are compile-time constants and v[] stays in registers.  Twiddles
// come from a __constant__ table (constant-bank operands of FFMA, no extra
// instruction); the trivial ones (1, -i, i) are folded away at compile time.
//
// Conventions: forward = exp(-2*pi*i*k*n/N), inverse = exp(+...), no 1/N
// scaling (as the reference's FFT class, openpiv/algos/fft.h:274-294).
#pragma once
#include <cuda_runtime.h>

namespace opiv {

// ---------------------------------------------------------------------------
// cos / sin of 2*pi*k/N evaluated at compile time.  The angle is reduced to
// [0, pi/4] exactly with integer arithmetic on k (quarter turns, then the
// complementary angle), then summed as a Taylor series (truncation < 1e-17
// for |x| <= pi/4).  This is plain mathematics, evaluated by the C++ front
// end; no device math library is involved.
constexpr double kPi = 3.141592653589793238462643383279502884;

constexpr double series_sin(double x)
{
    double x2 = x * x, term = x, sum = x;
    for (int n = 1; n < 14; ++n) {
        term *= -x2 / ((2.0 * n) * (2.0 * n + 1.0));
        sum += term;
    }
    return sum;
}

constexpr double series_cos(double x)
{
    double x2 = x * x, term = 1.0, sum = 1.0;
    for (int n = 1; n < 14; ++n) {
        term *= -x2 / ((2.0 * n - 1.0) * (2.0 * n));
        sum += term;
    }
    return sum;
}

// {cos, sin} of (pi/2) * r / N for 0 <= r <= N
constexpr void quarter(long r, long N, double& c, double& s)
{
    if (2 * r <= N) {
        const double x = (kPi / 2.0) * (double)r / (double)N;
        c = series_cos(x);
        s = series_sin(x);
    } else {
        const double x = (kPi / 2.0) * (double)(N - r) / (double)N;
        c = series_sin(x);
        s = series_cos(x);
    }
}

constexpr void cis_2pi(long k, long N, double& c, double& s)
{
    k %= N;
    if (k < 0) k += N;
    const long q = (4 * k) / N;          // quarter turn index
    const long r = 4 * k - q * N;        // remainder, in units of 1/(4N) turn
    double qc = 0, qs = 0;
    quarter(r, N, qc, qs);
    switch (q) {
    case 0: c = qc; s = qs; break;
    case 1: c = -qs; s = qc; break;
    case 2: c = -qc; s = -qs; break;
    default: c = qs; s = -qc; break;
    }
}

// exp(-2*pi*i*k/64) for k < 64; length-N transforms use entry k*(64/N).
constexpr int kTwMax = 64;
struct TwiddleTable {
    float re[kTwMax];
    float im[kTwMax];
};

constexpr TwiddleTable make_twiddles()
{
    TwiddleTable t{};
    for (int k = 0; k < kTwMax; ++k) {
        double c = 0, s = 0;
        cis_2pi(k, kTwMax, c, s);
        t.re[k] = (float)c;
        t.im[k] = (float)(-s);
    }
    return t;
}

static __constant__ TwiddleTable c_tw = make_twiddles();

// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }

// z * exp(-+2*pi*i*k/N); INV selects the + sign.
template <int N, bool INV>
__device__ __forceinline__ float2 twiddle(float2 z, int k)
{
    k &= (N - 1);
    if (k == 0) return z;
    if (4 * k == N) return INV ? make_float2(-z.y, z.x) : make_float2(z.y, -z.x);
    if (2 * k == N) return make_float2(-z.x, -z.y);
    if (4 * k == 3 * N) return INV ? make_float2(z.y, -z.x) : make_float2(-z.y, z.x);
    const float wr = c_tw.re[k * (kTwMax / N)];
    const float wi = INV ? -c_tw.im[k * (kTwMax / N)] : c_tw.im[k * (kTwMax / N)];
    return make_float2(z.x * wr - z.y * wi, z.x * wi + z.y * wr);
}

// Decimation in frequency: natural-order input, bit-reversed output
// (v[i] holds X[bitrev(i)]).
template <int N, bool INV>
__device__ __forceinline__ void fft_dif(float2 (&v)[N])
{
#pragma unroll
    for (int half = N / 2; half >= 1; half >>= 1) {
#pragma unroll
        for (int base = 0; base < N; base += 2 * half) {
#pragma unroll
            for (int j = 0; j < half; ++j) {
                const float2 a = v[base + j], b = v[base + j + half];
                v[base + j] = cadd(a, b);
                v[base + j + half] = twiddle<N, INV>(csub(a, b), j * (N / (2 * half)));
            }
        }
    }
}

// Decimation in time: bit-reversed input (v[i] holds x[bitrev(i)]),
// natural-order output.
template <int N, bool INV>
__device__ __forceinline__ void fft_dit(float2 (&v)[N])
{
#pragma unroll
    for (int half = 1; half < N; half <<= 1) {
#pragma unroll
        for (int base = 0; base < N; base += 2 * half) {
#pragma unroll
            for (int j = 0; j < half; ++j) {
                const float2 a = v[base + j];
                const float2 b = twiddle<N, INV>(v[base + j + half], j * (N / (2 * half)));
                v[base + j] = cadd(a, b);
                v[base + j + half] = csub(a, b);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Decimation in time in fused multiply-add form: with w = wx + i wy and
// t = wy / wx, w*b = wx * (b + i t b), so a +- w*b costs 2 FMAs for
// c = b + i t b and 4 FMAs for a +- wx*c: 6 instructions per twiddled
// butterfly instead of 8.  The factor with the larger magnitude is pulled
// out (wx when |wx| >= |wy|, else wy with w*b = wy * ((wx/wy) b + i b)), which
// keeps the ratio within [-1, 1].  Tables are evaluated at compile time.
struct FmaTwiddles {
    float m[kTwMax];      // pulled-out factor: wx or wy of exp(-2 pi i k / 64)
    float r[kTwMax];      // ratio: wy / wx or wx / wy
    bool by_cos[kTwMax];  // |wx| >= |wy|
};

__host__ __device__ constexpr bool fma_by_cos(int k)
{
    // |cos| >= |sin| for angles within 45 degrees of the real axis
    const int q = k & (kTwMax / 2 - 1);   // k mod 32 (period pi for |cos|, |sin|)
    return q <= kTwMax / 8 || q >= 3 * kTwMax / 8;
}

constexpr FmaTwiddles make_fma_twiddles()
{
    FmaTwiddles t{};
    for (int k = 0; k < kTwMax; ++k) {
        double c = 0, s = 0;
        cis_2pi(k, kTwMax, c, s);
        const double wx = c, wy = -s;   // forward twiddle exp(-2 pi i k / 64)
        const bool bc = fma_by_cos(k);
        t.by_cos[k] = bc;
        t.m[k] = (float)(bc ? wx : wy);
        t.r[k] = (float)(bc ? wy / wx : wx / wy);
    }
    return t;
}

static __constant__ FmaTwiddles c_fma = make_fma_twiddles();

// a, b -> a + w b, a - w b with w = exp(-+2 pi i k / N)
template <int N, bool INV>
__device__ __forceinline__ void bfly_dit(float2& a, float2& b, int k)
{
    k &= (N - 1);
    if (k == 0) {
        const float2 t = b;
        b = csub(a, t);
        a = cadd(a, t);
        return;
    }
    if (4 * k == N) {   // w = -i (forward) or i (inverse)
        const float2 wb = INV ? make_float2(-b.y, b.x) : make_float2(b.y, -b.x);
        b = csub(a, wb);
        a = cadd(a, wb);
        return;
    }
    const int q = k * (kTwMax / N);
    const float m = (INV && !fma_by_cos(q)) ? -c_fma.m[q] : c_fma.m[q];
    const float r = INV ? -c_fma.r[q] : c_fma.r[q];
    float2 c;
    if (fma_by_cos(q)) {    // w b = wx (bx - t by, by + t bx), t = wy / wx
        c = make_float2(fmaf(-r, b.y, b.x), fmaf(r, b.x, b.y));
    } else {                // w b = wy (s bx - by, s by + bx), s = wx / wy
        c = make_float2(fmaf(r, b.x, -b.y), fmaf(r, b.y, b.x));
    }
    b = make_float2(fmaf(-m, c.x, a.x), fmaf(-m, c.y, a.y));
    a = make_float2(fmaf(m, c.x, a.x), fmaf(m, c.y, a.y));
}

// Decimation in time, FMA form: bit-reversed input (v[i] holds
// x[bitrev(i)]), natural-order output.
template <int N, bool INV>
__device__ __forceinline__ void fft_dit_fma(float2 (&v)[N])
{
#pragma unroll
    for (int half = 1; half < N; half <<= 1) {
#pragma unroll
        for (int base = 0; base < N; base += 2 * half) {
#pragma unroll
            for (int j = 0; j < half; ++j)
                bfly_dit<N, INV>(v[base + j], v[base + j + half], j * (N / (2 * half)));
        }
    }
}

template <int N>
__host__ __device__ constexpr int bitrev(int i)
{
    int r = 0;
    for (int b = 1; b < N; b <<= 1) {
        r = (r << 1) | (i & 1);
        i >>= 1;
    }
    return r;
}

}  // namespace opiv
