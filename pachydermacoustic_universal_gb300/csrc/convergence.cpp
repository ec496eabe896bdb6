// convergence.cpp -- convergence mode of the split ray tracer (SplitRayTracer with rayCount < 1).
//
// The reference ("Classes_Complete_Trace - TaskAll.cs") then traces in revolutions of
// Source.Revolution_Period() primaries (80 per point source, the members' sum for a SourceCluster,
// Classes_Sources.cs:197-200, 680-688, 731-734) and after each revolution asks its convergence checks
// (TaskAll:300-330); it stops when every check answers true.  The checks watch the raw (unscaled)
// energy histogram of band h_oct at two receivers chosen by the ctor (TaskAll:111-176): the farthest
// receiver the source sees directly (check 0) and the farthest it does not (check 1).  rayCount == 0
// selects SpecMin_Convergence_Check (TaskAll:806-921), rayCount < 0 Minimum_Convergence_Check
// (TaskAll:1015-1107).  This file holds the checks as host code; the device captures each revolution's
// contribution to the two receivers' histograms, and the run worker (capi.cpp) replays the checks
// revolution by revolution.
#include <cmath>
#include <vector>

#include "engine.h"

namespace pach {
namespace {

// AcousticalMath.SPL_Intensity (Classes_Math.cs:97-102): 10 log10(I / 1e-12), negative levels -> 0.
double spl_intensity(double I) {
    const double spl = 10.0 * std::log10(I / 1e-12);
    return spl < 0 ? 0.0 : spl;
}

// AcousticalMath.SlidingMax (Classes_Math.cs:362-388) as written: a monotone deque kept in a ring of
// `window` index slots.  The push comes before the stale head is dropped, so after `window` falling
// samples the push overwrites the head's slot and the result is the new sample -- kept, since the
// checks' envelopes depend on it.
std::vector<double> sliding_max(const std::vector<double> &x, int window) {
    const int n = (int)x.size();
    std::vector<double> out(x.size());
    std::vector<int> dq((size_t)window, 0);
    int head = 0, tail = -1;
    for (int i = 0; i < n; ++i) {
        while (tail >= head && x[(size_t)i] >= x[(size_t)dq[(size_t)(tail % window)]]) --tail;
        ++tail;
        dq[(size_t)(tail % window)] = i;
        const int start = i - window + 1;
        if (dq[(size_t)(head % window)] < start) ++head;
        out[(size_t)i] = x[(size_t)dq[(size_t)(head % window)]];
    }
    return out;
}

// AcousticalMath.Envelope (Classes_Math.cs:327-360) with localMaxWindow 0.02 s and monotonicDown off.
// The first step starts from the input's first sample (prev = x[0]), not from the clamped output.
std::vector<double> envelope(const std::vector<double> &x, double fs, double attack, double release) {
    if (x.empty()) return {};
    const int w = std::max(1, (int)std::nearbyint(0.02 * fs));
    const std::vector<double> lm = sliding_max(x, w);
    const double a = 1.0 - std::exp(-1.0 / (attack * fs)), r = 1.0 - std::exp(-1.0 / (release * fs));
    std::vector<double> y(x.size());
    double prev = x[0];
    y[0] = std::min(prev, lm[0]);
    for (size_t i = 1; i < x.size(); ++i) {
        const double c = x[i] > prev ? a : r;
        double yn = prev + c * (x[i] - prev);
        yn = std::min(yn, lm[i]);
        y[i] = yn;
        prev = yn;
    }
    return y;
}

}  // namespace

void conv_setup(ConvCheck &c, int mode, int row, double dist_m, double c_mps, int fs, int T) {
    c = ConvCheck();
    c.mode = mode;
    c.row = row;
    c.fs = fs;
    c.T = T;
    c.E.assign((size_t)T, 0.0);
    c.A0.assign((size_t)T, 0.0);
    c.A1.assign((size_t)T, 0.0);
    c.A2.assign((size_t)T, 0.0);
    if (mode == 1) {
        // Minimum_Convergence_Check ctor (TaskAll:1023-1030)
        c.s_start = (int)std::floor(dist_m / c_mps * fs);
        c.s50 = (int)std::floor(50.0 * fs / 1000) + c.s_start;
        c.s80 = (int)std::floor(80.0 * fs / 1000) + c.s_start;
        c.s_inf = T;
    } else {
        // SpecMin_Convergence_Check ctor (TaskAll:816-835): blocks of SampleRate / 20 samples
        c.step = std::max(1, fs / 20);
        c.binct = T / c.step;
        c.snapshot.assign((size_t)c.binct, 0.0);
    }
}

bool ConvCheck::check() {
    if (mode == 1) {
        // Minimum_Convergence_Check.Check (TaskAll:1033-1100): the energy before 50 ms, before 80 ms and
        // after 80 ms of the direct arrival must each change by at most 2 %, 2 % and 10 % between
        // revolutions, six revolutions in a row.  (Its T30 is display only.)
        double sn50 = 0, sn80 = 0, sninf = 0;
        for (int i = s_start; i < s50 && i < T; ++i) sn50 += E[(size_t)i];
        sn80 += sn50;
        for (int i = s50; i < s80; ++i)
            if (i < T) sn80 += E[(size_t)i];
        for (int i = s80; i < s_inf; ++i) sninf += E[(size_t)i];
        const double conv1 = std::fabs(sn50 - snap50) / snap50, conv2 = std::fabs(sn80 - snap80) / snap80,
                     convinf = std::fabs(sninf - snapinf) / snapinf;
        // (C# comparisons with NaN are false, as here)
        if (sn50 == 0 || conv1 > 0.02 || sn80 == 0 || conv2 > 0.02 || sninf == 0 || convinf > 0.1) count = 0;
        else ++count;
        snap50 = sn50;
        snap80 = sn80;
        snapinf = sninf;
        return count > 5;
    }
    // SpecMin_Convergence_Check.Check (TaskAll:838-915)
    rayct += 80;  // as written: 80 per revolution whatever the source's period
    std::vector<double> sn((size_t)binct, 0.0), sn_spec((size_t)binct, 0.0), sn_diff((size_t)binct, 0.0);
    for (int i = 0; i < binct; ++i)
        for (int j = 0; j < step; ++j) {
            const size_t k = (size_t)(i * step + j);
            sn[(size_t)i] += E[k];
            sn_spec[(size_t)i] += A0[k];
            sn_diff[(size_t)i] += A1[k];
        }
    std::vector<double> si_spec = envelope(A0, fs, 0.001, 0.01);
    const std::vector<double> si_diff = envelope(A1, fs, 0.001, 0.01), si_rogue = envelope(A2, fs, 0.001, 0.01);
    std::vector<double> si_comb(si_spec.size());
    for (size_t i = 0; i < si_spec.size(); ++i) si_comb[i] = si_diff[i] + si_rogue[i];
    for (size_t i = 0; i < si_spec.size(); ++i) {
        si_spec[i] = spl_intensity(si_spec[i]) - 110;
        si_comb[i] = spl_intensity(si_comb[i]) - 110;
    }
    // the last 50 ms block whose specular energy is still above 1e-6 of the first diffuse block
    double conv = 0;
    if (binct > 0) {
        const double inf60diff = sn_diff[0] * 1e-6;
        int stop = binct - 1;
        while (stop >= 0 && sn_spec[(size_t)stop] < inf60diff && stop != 1) --stop;
        for (int i = 0; i < binct; ++i) {
            if (sn[(size_t)i] == 0 || snapshot[(size_t)i] == 0) continue;
            const double d = std::fabs(sn[(size_t)i] - snapshot[(size_t)i]) / snapshot[(size_t)i];
            if (i < stop) conv = std::max(conv, d);
        }
    }
    // the latest sample where the specular envelope stands 4 dB above the scattered one
    int spec_cross = 0;
    for (int i = (int)si_spec.size() - 1; i > 0; --i) {
        spec_cross = i;
        if (si_spec[(size_t)i] > si_comb[(size_t)i] + 4) break;
    }
    // Nmin = max(5000, 4 n^2) with n = 343 spec_cross / T in C# integer arithmetic
    const double n = T > 0 ? (double)((343LL * spec_cross) / T) : 0.0;
    nmin = std::max(5000LL, (long long)std::ceil(4 * n * n));
    snapshot = sn;
    if (conv == 0) return false;
    if (conv > 0.1) count = 0;
    ++count;
    return count > 10 && rayct > nmin;
}

// The ctor's receiver choice (TaskAll:111-176): from the source's origin (a cluster's centre) towards
// each receiver, Check_Validity shoots one ray (TaskAll:178-200): the receiver is visible when nothing
// is hit before it.  rows[0] = the farthest visible receiver, rows[1] = the farthest hidden one (-1 when
// there is none); dist[k] = its distance.
void pick_conv_receivers(const HostScene &hs, const double src[3], const pach_receiver_desc *rec, int R, int rows[2],
                         double dist[2]) {
    double max_t = 0, max_f = 0;
    rows[0] = rows[1] = -1;
    dist[0] = dist[1] = 0;
    for (int i = 0; i < R; ++i) {
        double d[3] = {rec[i].origin[0] - src[0], rec[i].origin[1] - src[1], rec[i].origin[2] - src[2]};
        const double len = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        if (!(len > 0)) continue;
        for (double &x : d) x /= len;
        int tri = -1;
        double t = 0;
        const bool hit = bvh_shoot_host(hs, src, d, 1e-10, tri, t);
        const bool valid = !hit || t >= len;
        if (valid) {
            if (max_t < len) { rows[0] = i; max_t = len; dist[0] = len; }
        } else if (max_f < len) {
            rows[1] = i;
            max_f = len;
            dist[1] = len;
        }
    }
}

}  // namespace pach

extern "C" pach_status pach_convergence_replay(const double *per_rev, int32_t revs, int32_t T, int32_t sample_rate,
                                               int32_t mode, double distance_m, double sound_speed, int32_t *stop_rev,
                                               int64_t *nmin_out) {
    auto report = [](pach_status s, const std::string &m) {
        pach::set_last_error(m.c_str());
        return s;
    };
    return pach::guarded([&]() -> pach_status {
        if (!per_rev || !stop_rev || revs < 0 || T < 1 || sample_rate < 1 || mode < 0 || mode > 1 ||
            !(sound_speed > 0) || !(distance_m >= 0))
            return report(PACH_ERR_INVALID_ARGUMENT, "pach_convergence_replay: bad arguments");
        pach::ConvCheck c;
        pach::conv_setup(c, mode, 0, distance_m, sound_speed, sample_rate, T);
        *stop_rev = 0;
        for (int r = 0; r < revs; ++r) {
            const double *h = per_rev + (size_t)r * 4 * T;
            for (int b = 0; b < T; ++b) {
                c.E[(size_t)b] += h[b];
                c.A0[(size_t)b] += h[T + b];
                c.A1[(size_t)b] += h[2 * T + b];
                c.A2[(size_t)b] += h[3 * T + b];
            }
            if (c.check()) {
                *stop_rev = r + 1;
                break;
            }
        }
        if (nmin_out) *nmin_out = c.nmin;
        return PACH_OK;
    }, report);
}
