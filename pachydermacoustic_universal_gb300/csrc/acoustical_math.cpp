// acoustical_math.cpp -- room-acoustic parameters from energy-time curves, as AcousticalMath
// computes them (Classes_Math.cs).  Host-side post-processing of the tracer's histograms.
#include <algorithm>
#include <cmath>
#include <vector>

#include "engine.h"

namespace {

// Log10Data (Classes_Math.cs:392-408): 10 log10(x) floored at limit_in_db; index 0 left at 0.
std::vector<double> log10_floor(const double *x, int n, double limit_db) {
    std::vector<double> out((size_t)(n > 0 ? n : 0), 0.0);
    const double lv = std::pow(10.0, limit_db / 10.0);
    for (int i = 1; i < n; ++i) out[i] = x[i] >= lv ? 10.0 * std::log10(x[i]) : limit_db;
    return out;
}

// Schroeder_Limits (417-438): first index (from 1) below `first`, then first index from there below `second`.
void decay_limits(const std::vector<double> &l, double first, double second, int &a, int &b) {
    a = 0;
    b = 0;
    const int n = (int)l.size();
    for (int i = 1; i < n; ++i)
        if (l[i] < first) { a = i; break; }
    for (int i = a; i < n; ++i)
        if (l[i] < second) { b = i; break; }
}

// Least_Square_Fit slope (446-473), time axis i / fs.
double fit_slope(const double *y, int len, double fs) {
    double st = 0, sy = 0, stt = 0, sty = 0;
    for (int i = 0; i < len; ++i) {
        const double q = i / fs;
        st += q; sy += y[i]; stt += q * q; sty += q * y[i];
    }
    return (len * sty - st * sy) / (len * stt - st * st);
}

double decay_time(const double *sch, int n, double first, double second, int fs) {
    const std::vector<double> l = log10_floor(sch, n, -60);
    int a, b;
    decay_limits(l, first, second, a, b);
    const int len = b - a + 1;
    if (len < 1) return NAN;
    return -60.0 / fit_slope(l.data() + a, len, fs);
}

}  // namespace

extern "C" {

pach_status pach_math_schroeder(const double *etc, int32_t n, double *out) {
    if ((!etc || !out) && n > 0) return PACH_ERR_INVALID_ARGUMENT;
    double total = 0;
    for (int i = 0; i < n; ++i) { total += etc[i]; out[i] = total; }
    for (int i = 0; i < n; ++i) out[i] = total == 0 ? 0.0 : 1.0 - out[i] / total;
    return PACH_OK;
}

double pach_math_t_x(const double *sch, int32_t n, int32_t depth, int32_t fs) {
    return decay_time(sch, n, -5, -5 - std::abs(depth), fs);
}

double pach_math_edt(const double *sch, int32_t n, int32_t fs) { return decay_time(sch, n, -1, -10.0001, fs); }

double pach_math_clarity(const double *etc, int32_t n, double fs, double seconds, double start, int32_t pressure) {
    if (pressure) seconds += 8192.0 / fs;
    const double bw = 1.0 / fs;
    const int si = (int)std::floor(start * fs), ei = (int)std::floor((seconds + start) * fs);
    double early = 0, late = 0;
    for (int q = si; q < ei && q < n; ++q) early += etc[q];
    const double split = (seconds + start - ei * bw) / bw;  // share of the boundary bin that is early
    if (ei >= 0 && ei < n) { early += split * etc[ei]; late += (1 - split) * etc[ei]; }
    for (int q = ei + 1; q < n; ++q) late += etc[q];
    return 10.0 * std::log10(early / late);
}

double pach_math_definition(const double *etc, int32_t n, double fs, double seconds, double start, int32_t pressure) {
    if (pressure) start += 8192.0 / fs;
    const double bw = 1.0 / fs;
    const int si = (int)std::floor(start * fs);
    const int ei = (int)std::floor(seconds * fs) + si;
    double early = 0, all = 0;
    for (int q = 0; q < ei && q < n; ++q) early += etc[q];  // the early sum starts at bin 0
    const double split = (seconds + start - ei * bw) / bw;
    if (ei >= 0 && ei < n) early += split * etc[ei];
    for (int q = 0; q < n; ++q) all += etc[q];
    return early / all * 100.0;
}

double pach_math_center_time(const double *etc, int32_t n, int32_t fs, double direct, int32_t pressure) {
    if (pressure) direct += 8192.0 / fs;
    const double bw = 1.0 / (double)fs;
    double spt = 0, st = 0;
    for (int i = std::max(0, (int)std::floor(direct * fs)); i < n; ++i) {
        spt += etc[i] * (i * bw - direct);
        st += etc[i];
    }
    return spt / st;
}

double pach_math_strength(const double *etc, int32_t n, double swl, int32_t) {
    double all = 0;
    for (int q = 0; q < n; ++q) all += etc[q];
    double spl = 10.0 * std::log10(all / 1e-12);  // SPL_Intensity (Classes_Math.cs:97-102)
    if (spl < 0) spl = 0;
    return spl - swl + 31.0;
}

double pach_math_sound_speed(double temp_c) { return 331.0 + 0.6 * temp_c; }

}  // extern "C"
