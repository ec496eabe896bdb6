// autotune.cpp -- picks the wavefront loop's packet size and block shape for a set of rooms by
// timing short sample runs, and remembers the choice in a small text cache.
//
// Knobs (pach_trace_params): wave_kilo_items (octave rays per wave, the packet), block_threads and
// blocks_per_sm (block shape and the trace kernel's register variant), traversal (one leaf at a time,
// speculative, or inside the shading kernel).  Search: coordinate descent from the defaults --
// traversal x register variant,
// then the wave size, then the block size -- each candidate timed on a sample of the rooms' primaries
// (device time per segment of the whole run, the stats' device_ms).  No counterpart in the reference.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "engine.h"

using namespace pach;

namespace {

std::mutex g_cache_mu;

struct Knobs {
    int wave_kilo, threads, bps, traversal;
};

std::string default_cache_path() {
    if (const char *p = std::getenv("PACH_TUNE_CACHE")) return p;
    if (const char *h = std::getenv("HOME")) return std::string(h) + "/.cache/pach_gb300_tune.txt";
    return "pach_gb300_tune.txt";
}

// Cache key: device, SM count and a coarse signature of the workload (rooms, triangles, receivers,
// octave range), bucketed by powers of two so that similar batches share an entry.
std::string cache_key(const pach_room_desc *rooms, int n_rooms, const pach_trace_params &p) {
    cudaDeviceProp prop{};
    int dev = 0;
    cudaGetDevice(&dev);
    cudaGetDeviceProperties(&prop, dev);
    long long tris = 0, rec = 0;
    for (int i = 0; i < n_rooms; ++i) {
        int32_t np = 0, nt = 0;
        pach_scene_info(rooms[i].scene, &np, &nt, nullptr, nullptr, nullptr, nullptr);
        tris += nt;
        rec += rooms[i].n_receivers;
    }
    auto lg = [](long long x) { return x > 0 ? (int)std::floor(std::log2((double)x)) : -1; };
    std::ostringstream k;
    std::string name = prop.name;
    std::replace(name.begin(), name.end(), ' ', '_');
    k << name << "|sm" << prop.multiProcessorCount << "|rooms" << lg(n_rooms) << "|tris" << lg(tris) << "|rec"
      << lg(rec) << "|oct" << p.oct_lo << "-" << p.oct_hi;
    return k.str();
}

bool cache_get(const std::string &path, const std::string &key, Knobs &k, double &rate) {
    std::lock_guard<std::mutex> lk(g_cache_mu);
    std::ifstream f(path);
    std::string line;
    bool found = false;
    while (std::getline(f, line)) {  // the last entry of a key wins
        std::istringstream s(line);
        std::string kk;
        Knobs x{};
        double r = 0;
        if (s >> kk >> x.wave_kilo >> x.threads >> x.bps >> x.traversal >> r && kk == key) {
            k = x;
            rate = r;
            found = true;
        }
    }
    return found;
}

void cache_put(const std::string &path, const std::string &key, const Knobs &k, double rate) {
    std::lock_guard<std::mutex> lk(g_cache_mu);
    std::ofstream f(path, std::ios::app);
    if (f) f << key << " " << k.wave_kilo << " " << k.threads << " " << k.bps << " " << k.traversal << " " << rate << "\n";
}

// Segments per second of one sample batch run with the given knobs (< 0 on failure).
double time_sample(const std::vector<pach_room_desc> &rooms, const pach_trace_params &base, const Knobs &k) {
    pach_trace_params p = base;
    p.wave_kilo_items = k.wave_kilo;
    p.block_threads = k.threads;
    p.blocks_per_sm = k.bps;
    p.traversal = k.traversal;
    p.kernel_timing = 0;
    pach_run *run = nullptr;
    if (pach_batch_begin(rooms.data(), (int32_t)rooms.size(), &p, &run) != PACH_OK) return -1;
    double rate = -1;
    pach_stats s{};
    if (pach_trace_wait(run, -1) == PACH_OK && pach_trace_get_stats(run, &s) == PACH_OK && s.device_ms > 0)
        rate = (double)s.segments / (s.device_ms * 1e-3);
    pach_run_destroy(run);
    return rate;
}

}  // namespace

extern "C" pach_status pach_autotune(const pach_room_desc *rooms, int32_t n_rooms, const pach_trace_params *params,
                                     int64_t sample_rays, const char *cache_path, int32_t force,
                                     pach_tune_result *out) {
    if (!rooms || n_rooms < 1 || !params || !out || sample_rays < 1) {
        set_last_error("autotune: rooms, params, out and sample_rays >= 1 are required");
        return PACH_ERR_INVALID_ARGUMENT;
    }
    if (pach_device_count() <= 0) {
        set_last_error("autotune: no CUDA device visible");
        return PACH_ERR_NO_DEVICE;
    }
    std::memset(out, 0, sizeof(*out));
    const std::string path = cache_path && *cache_path ? cache_path : default_cache_path();
    const std::string key = cache_key(rooms, n_rooms, *params);
    Knobs best{};
    double best_rate = 0;
    if (!force && cache_get(path, key, best, best_rate)) {
        out->wave_kilo_items = best.wave_kilo;
        out->block_threads = best.threads;
        out->blocks_per_sm = best.bps;
        out->traversal = best.traversal;
        out->segments_per_s = best_rate;
        out->from_cache = 1;
        return PACH_OK;
    }
    // the sample: every room keeps its share of sample_rays (at least one primary)
    long long total = 0;
    for (int i = 0; i < n_rooms; ++i) total += std::max<int64_t>(1, rooms[i].ray_count);
    std::vector<pach_room_desc> sample(rooms, rooms + n_rooms);
    for (pach_room_desc &d : sample)
        d.ray_count = std::max<int64_t>(1, (int64_t)std::llround((double)std::max<int64_t>(1, d.ray_count) * sample_rays / total));
    const auto t0 = std::chrono::steady_clock::now();
    int trials = 0;
    Knobs cur{8192, 256, 6, 0};
    if (time_sample(sample, *params, cur) < 0) {  // warm-up (and a check that the sample runs at all)
        return PACH_ERR_INVALID_ARGUMENT;
    }
    best = cur;
    best_rate = -1;
    auto consider = [&](const Knobs &k) {
        const double r = time_sample(sample, *params, k);
        ++trials;
        if (r > best_rate) {
            best_rate = r;
            best = k;
        }
    };
    for (int trav : {1, 2})
        for (int bps : {4, 6}) consider(Knobs{cur.wave_kilo, cur.threads, bps, trav});
    consider(Knobs{cur.wave_kilo, cur.threads, 4, 3});  // the walk inside the shading kernel
    const Knobs stage1 = best;
    for (int w : {2048, 4096, 16384}) consider(Knobs{w, stage1.threads, stage1.bps, stage1.traversal});
    const Knobs stage2 = best;
    consider(Knobs{stage2.wave_kilo, 128, stage2.bps, stage2.traversal});
    if (best_rate <= 0) {
        set_last_error("autotune: no sample run succeeded");
        return PACH_ERR_GAVE_UP;
    }
    cache_put(path, key, best, best_rate);
    out->wave_kilo_items = best.wave_kilo;
    out->block_threads = best.threads;
    out->blocks_per_sm = best.bps;
    out->traversal = best.traversal;
    out->segments_per_s = best_rate;
    out->trials = trials;
    out->tune_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return PACH_OK;
}
