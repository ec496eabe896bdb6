// map_params.cu -- room-acoustic parameters of many energy-time curves at once, on the device.
//
// A map of 10^3..10^5 receivers x 8 bands is 10^4..10^6 curves that already sit in HBM after the
// trace; the reference derives its parameter maps one curve at a time on the host
// (Pach_Map_Receiver.cs:925-1270 calling AcousticalMath, Classes_Math.cs:282-586, 934-962).  Here one
// warp takes one curve through three streaming passes (totals, limits, fit), FP64 throughout.
#include <cmath>

#include "engine.h"

namespace pach {
namespace {

constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
    return v;
}

// inclusive prefix sum over the warp
__device__ __forceinline__ double warp_scan(double v, int lane) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const double u = __shfl_up_sync(FULL, v, o);
        if (lane >= o) v += u;
    }
    return v;
}

// Log10Data (Classes_Math.cs:392-408) of the Schroeder curve at bin i: 10 log10(S) floored at -60 dB,
// bin 0 left at 0.
__device__ __forceinline__ double level(double S, int i) {
    if (i == 0) return 0.0;
    return S >= 1e-6 ? 10.0 * log10(S) : -60.0;
}

// first index >= from (and >= 1) of a warp chunk whose flag is set, or -1
__device__ __forceinline__ int first_set(unsigned ballot, int base, int from) {
    const int skip = from - base;
    if (skip >= 32) return -1;
    if (skip > 0) ballot &= ~((1u << skip) - 1u);
    return ballot ? base + __ffs(ballot) - 1 : -1;
}

__global__ void __launch_bounds__(256) k_map_params(const double *etc, int n, int T, double fs, double scale,
                                                    int depth, double clar_s, double *t_x, double *edt, double *clar,
                                                    double *defi, double *sum) {
    const int w = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (w >= n) return;
    const double *x = etc + (size_t)w * T;
    // pass 1: total, and the early sums of Clarity (start 0: bins [0, ei)) and Definition
    const int ei_c = (int)floor((clar_s + 0.0) * fs), ei_d = (int)floor(0.05 * fs);
    double tot = 0, ec = 0, lc = 0, ed = 0;
    for (int i = lane; i < T; i += 32) {
        const double v = x[i] * scale;
        tot += v;
        if (i < ei_c) ec += v;
        if (i > ei_c) lc += v;
        if (i < ei_d) ed += v;
    }
    tot = warp_sum(tot);
    ec = warp_sum(ec);
    lc = warp_sum(lc);
    ed = warp_sum(ed);
    // Clarity (559-586): the boundary bin is split between early and late
    const double bw = 1.0 / fs;
    if (ei_c >= 0 && ei_c < T) {
        const double split = (clar_s + 0.0 - ei_c * bw) / bw, v = x[ei_c] * scale;
        ec += split * v;
        lc += (1 - split) * v;
    }
    double edd = ed;
    if (ei_d >= 0 && ei_d < T) edd += (0.05 + 0.0 - ei_d * bw) / bw * x[ei_d] * scale;
    // pass 2: fit limits on the Schroeder curve S[i] = 1 - cumsum[i] / total (Schroeder_Limits, 417-438)
    const double first30 = -5.0, second30 = -5.0 - fabs((double)depth);
    const double first_e = -1.0, second_e = -10.0001;
    int a30 = -1, b30 = -1, ae = -1, be = -1;
    double carry = 0;
    for (int base = 0; base < T && (b30 < 0 || be < 0); base += 32) {
        const int i = base + lane;
        const double v = i < T ? x[i] * scale : 0.0;
        const double cum = carry + warp_scan(v, lane);
        carry = __shfl_sync(FULL, cum, 31);
        const double S = tot == 0 ? 0.0 : 1.0 - cum / tot;
        const double l = i < T ? level(S, i) : 0.0;
        const bool ok = i < T;
        if (a30 < 0) a30 = first_set(__ballot_sync(FULL, ok && i >= 1 && l < first30), base, 1);
        if (a30 >= 0 && b30 < 0) b30 = first_set(__ballot_sync(FULL, ok && l < second30), base, a30);
        if (ae < 0) ae = first_set(__ballot_sync(FULL, ok && i >= 1 && l < first_e), base, 1);
        if (ae >= 0 && be < 0) be = first_set(__ballot_sync(FULL, ok && l < second_e), base, ae);
    }
    // not found: index 0, as the reference's loops leave them
    if (a30 < 0) a30 = 0;
    if (ae < 0) ae = 0;
    if (b30 < 0) b30 = 0;
    if (be < 0) be = 0;
    // pass 3: least-squares slopes over [a, b] of each fit, time axis (i - a) / fs (Least_Square_Fit, 446-473)
    double s30[4] = {0, 0, 0, 0}, se[4] = {0, 0, 0, 0};  // sum q, sum y, sum q^2, sum q y
    const int end = max(b30, be);
    carry = 0;
    for (int base = 0; base <= end; base += 32) {
        const int i = base + lane;
        const double v = i < T ? x[i] * scale : 0.0;
        const double cum = carry + warp_scan(v, lane);
        carry = __shfl_sync(FULL, cum, 31);
        if (i >= T) continue;
        const double S = tot == 0 ? 0.0 : 1.0 - cum / tot;
        const double l = level(S, i);
        if (i >= a30 && i <= b30) {
            const double q = (i - a30) / fs;
            s30[0] += q; s30[1] += l; s30[2] += q * q; s30[3] += q * l;
        }
        if (i >= ae && i <= be) {
            const double q = (i - ae) / fs;
            se[0] += q; se[1] += l; se[2] += q * q; se[3] += q * l;
        }
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        s30[k] = warp_sum(s30[k]);
        se[k] = warp_sum(se[k]);
    }
    if (lane) return;
    auto fit = [&](const double (&s)[4], int a, int b) -> double {
        const int len = b - a + 1;
        if (len < 1) return NAN;
        const double slope = (len * s[3] - s[0] * s[1]) / (len * s[2] - s[0] * s[0]);
        return -60.0 / slope;
    };
    if (t_x) t_x[w] = fit(s30, a30, b30);
    if (edt) edt[w] = fit(se, ae, be);
    if (clar) clar[w] = 10.0 * log10(ec / lc);
    if (defi) defi[w] = edd / tot * 100.0;
    if (sum) sum[w] = tot;
}

}  // namespace

cudaError_t launch_map_params(const double *etc, int n, int T, double fs, double scale, int decay_depth,
                              double clarity_s, double *t_x, double *edt, double *clarity, double *definition,
                              double *sum, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    const int blocks = (int)(((long long)n * 32 + 255) / 256);
    k_map_params<<<blocks, 256, 0, s>>>(etc, n, T, fs, scale, decay_depth, clarity_s, t_x, edt, clarity, definition,
                                        sum);
    return cudaGetLastError();
}

}  // namespace pach
