// noalloc.cu -- pach_trace_run_noalloc: the split ray tracer on caller-provided device buffers,
// with its working memory in a file-scope device array, so that the call allocates nothing.
//
// Who needs it: a host that traces from a thread on which device allocation is not allowed -- the
// processing callback of an audio or plug-in host, or code whose device memory is owned by another
// framework's allocator -- creates the scene once at set-up (pach_scene_create allocates) and then
// calls this entry point per run with its own output buffers.  The trade-off is capacity: the
// working set (ray ring, wave hits, schedule, receiver and source tables) is fixed at compile time.
#include <chrono>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "engine.h"

using namespace pach;

namespace {

constexpr unsigned long long kNaRing = 1ull << 16;  // octave rays in flight
constexpr unsigned long long kNaWave = 1ull << 15;  // octave rays per wave
constexpr int kNaMaxReceivers = 256;
constexpr int kNaMaxSources = 16;
constexpr int kNaStall = 64;  // synchronisations without progress before the call gives up

constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t kOffRing = 0;
constexpr size_t kOffHits = align256(kOffRing + kNaRing * sizeof(ORayItem));
constexpr size_t kOffCtl = align256(kOffHits + kNaWave * sizeof(int4));
constexpr size_t kOffCnt = align256(kOffCtl + sizeof(WaveCtl));
constexpr size_t kOffRec = align256(kOffCnt + sizeof(DevCounters));
constexpr size_t kOffSrc = align256(kOffRec + kNaMaxReceivers * sizeof(float4));
constexpr size_t kOffE0 = align256(kOffSrc + kNaMaxSources * sizeof(float4));
constexpr size_t kOffGeo = align256(kOffE0 + kNaMaxSources * kBands * sizeof(float));
constexpr size_t kOffRoom = align256(kOffGeo + kGeoFaces * 3 * sizeof(float4));
constexpr size_t kOffRoomPrim = align256(kOffRoom + sizeof(RoomParams));
constexpr size_t kScratchBytes = align256(kOffRoomPrim + 2 * sizeof(long long));  // ~4.7 MB

// The working memory of every pach_trace_run_noalloc call on this device.  It is resident on each
// GPU that loads the library until the process exits.  In host code the name stands for a
// host-side shadow, not a device address: the kernels get the address from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
unsigned char *g_scratch_addr[kMaxDevices] = {nullptr};

pach_status na_fail(pach_status s, const char *msg) {
    set_last_error(msg);
    return s;
}

}  // namespace

extern "C" pach_status pach_trace_run_noalloc(const pach_scene *scene, const pach_source_desc *sources,
                                              int32_t n_sources, const pach_receiver_desc *receivers,
                                              int32_t n_receivers, const pach_trace_params *params, void *stream_ptr,
                                              double *d_energy, double *d_pressure, double *d_dir_pos,
                                              double *d_dir_neg, double *d_analysis, pach_stats *stats) {
    const auto wall0 = std::chrono::steady_clock::now();
    if (!scene || !params || !sources) return na_fail(PACH_ERR_INVALID_ARGUMENT, "null scene, sources or params");
    if (!d_energy || !d_pressure || !d_dir_pos || !d_dir_neg || !d_analysis)
        return na_fail(PACH_ERR_INVALID_ARGUMENT, "all five device histogram buffers are required");
    // the checks of the allocating entry points (same inputs rejected with the same messages), then
    // the limits of the fixed working memory
    if (pach_status st = check_room(sources, n_sources, receivers, n_receivers, "")) return st;
    const pach_trace_params &p = *params;
    if (pach_status st = check_common(p)) return st;
    if (n_sources > kNaMaxSources) return na_fail(PACH_ERR_INVALID_ARGUMENT, "pach_trace_run_noalloc takes 1..16 sources");
    if (n_receivers > kNaMaxReceivers)
        return na_fail(PACH_ERR_INVALID_ARGUMENT, "pach_trace_run_noalloc takes 0..256 receivers");
    if (p.prim_dirs || p.prim_weights || p.proposal || p.capture || p.map)
        return na_fail(PACH_ERR_INVALID_ARGUMENT,
                       "pach_trace_run_noalloc does not take emission overrides, a proposal, capture or a map");
    if (p.ray_count < 1 || p.ray_begin < 0 || p.ray_begin + p.ray_count > (1ll << 32))
        return na_fail(PACH_ERR_INVALID_ARGUMENT, "ray_count must be >= 1 and ray_begin + ray_count <= 2^32");
    if (!(p.cutoff_length_m > 0)) return na_fail(PACH_ERR_INVALID_ARGUMENT, "cutoff_length_m must be positive");
    const long long T = (long long)((double)p.sample_rate * (p.hist_cotime_ms / 1000.0));

    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev != scene_device(scene) || dev < 0 || dev >= kMaxDevices)
        return na_fail(PACH_ERR_INVALID_ARGUMENT, "make the scene's device current before pach_trace_run_noalloc");
    // Set-up, once per device, with that device current: the device address of the scratch array.  It
    // is cached for the life of the process: a cudaDeviceReset (which also invalidates every scene
    // handle of that device) leaves it stale, so no call may follow a reset of its device.
    unsigned char *base = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_setup_mu);
        if (!g_scratch_addr[dev]) {
            void *addr = nullptr;
            const cudaError_t e = cudaGetSymbolAddress(&addr, g_noalloc_scratch);
            if (e != cudaSuccess) return na_fail(PACH_ERR_CUDA, cudaGetErrorString(e));
            g_scratch_addr[dev] = static_cast<unsigned char *>(addr);
        }
        base = g_scratch_addr[dev];
    }

    // The scene's device arrays must exist already: this call does not upload (it would allocate).
    if (!scene_dev(scene))
        return na_fail(PACH_ERR_INVALID_ARGUMENT, "the scene has no device copy yet (a scene of pach_scenes_create is "
                                                  "uploaded by its first single-room run); use pach_scene_create");

    // The ctor's derived quantities (TaskAll:83-109): COTime, h_oct, and the phase-A bound.
    const HostScene &hs = *scene_host(scene);
    double total_abs[kBands] = {0}, power[kBands] = {0};
    for (int s = 0; s < n_sources; ++s)
        for (int o = 0; o < kBands; ++o) power[o] = std::fmax(power[o], 1e-12 * std::pow(10.0, .1 * sources[s].power_db[o]));
    for (int q = 0; q < hs.npoly; ++q)
        for (int o = p.oct_lo; o <= p.oct_hi; ++o) total_abs[o] += hs.area[q] * hs.alpha[q * 8 + o];
    double mn = HUGE_VAL, octpower = 0;
    for (int o = p.oct_lo; o <= p.oct_hi; ++o) octpower = std::fmax(octpower, power[o]);
    int h_oct = p.oct_lo;
    for (int o = p.oct_lo; o <= p.oct_hi; ++o) {
        if (power[o] < octpower * 1e-6) continue;
        if (mn > total_abs[o]) { mn = total_abs[o]; h_oct = o; }
    }
    unsigned long long max_broad = p.max_broadband_bounces > 0 ? (unsigned long long)p.max_broadband_bounces
                                                               : derived_broadband_bound(hs, h_oct, p.pure_specular != 0);
    if (max_broad == 0)
        return na_fail(PACH_ERR_INVALID_ARGUMENT, "a surface reflects band h_oct without loss; set max_broadband_bounces");
    const bool pure = p.pure_specular != 0;
    const unsigned long long bound =
        (unsigned long long)kBands * ((hs.has_trans && !pure) ? 3 : 1) * max_broad + kBands;
    if (bound * 4 > kNaRing)
        return na_fail(PACH_ERR_INVALID_ARGUMENT,
                       "one primary can leave more phase-A rays than the no-alloc ring (65536 octave rays) can plan "
                       "for; use pach_trace_begin or set max_broadband_bounces");

    cudaStream_t stream = static_cast<cudaStream_t>(stream_ptr);
    cudaError_t e = cudaSuccess;
    const char *where = "";
#define NA_TRY(x)                                          \
    do {                                                   \
        e = (x);                                           \
        if (e != cudaSuccess) { where = #x; goto cuda_fail; } \
    } while (0)

    {
        // small tables, staged on the host stack
        float4 rec[kNaMaxReceivers];
        for (int i = 0; i < n_receivers; ++i)
            rec[i] = make_float4((float)receivers[i].origin[0], (float)receivers[i].origin[1], (float)receivers[i].origin[2],
                                 (float)(receivers[i].radius * receivers[i].radius));
        float4 src[kNaMaxSources];
        float e0[kNaMaxSources * kBands];
        for (int s = 0; s < n_sources; ++s) {
            src[s] = make_float4((float)sources[s].origin[0], (float)sources[s].origin[1], (float)sources[s].origin[2],
                                 (float)sources[s].kind);
            for (int o = 0; o < kBands; ++o) e0[s * kBands + o] = (float)(1e-12 * std::pow(10.0, .1 * sources[s].power_db[o]));
        }
        double gf[kGeoFaces * 9];
        geodesic_faces_fixed(gf);
        float4 geo[kGeoFaces * 3];
        for (int i = 0; i < kGeoFaces * 3; ++i) geo[i] = make_float4((float)gf[3 * i], (float)gf[3 * i + 1], (float)gf[3 * i + 2], 0.f);
        const size_t nE = (size_t)n_receivers * kBands * (size_t)T, nD = 3 * nE;

        // The scratch keeps the previous call's contents: clear the schedule and counters, and the
        // caller's histograms, which accumulate.
        WaveCtl h_ctl;
        std::memset(&h_ctl, 0, sizeof(h_ctl));
        h_ctl.next_prim = p.ray_begin;
        h_ctl.prim_end = p.ray_begin + p.ray_count;
        h_ctl.prim_first = p.ray_begin;
        if (n_receivers > 0) NA_TRY(cudaMemcpyAsync(base + kOffRec, rec, n_receivers * sizeof(float4), cudaMemcpyHostToDevice, stream));
        NA_TRY(cudaMemcpyAsync(base + kOffSrc, src, n_sources * sizeof(float4), cudaMemcpyHostToDevice, stream));
        NA_TRY(cudaMemcpyAsync(base + kOffE0, e0, n_sources * kBands * sizeof(float), cudaMemcpyHostToDevice, stream));
        NA_TRY(cudaMemcpyAsync(base + kOffGeo, geo, sizeof(geo), cudaMemcpyHostToDevice, stream));
        RoomParams room{};
        room.prim_begin = p.ray_begin;
        room.prim_end = p.ray_begin + p.ray_count;
        room.inv_c = (float)(1.0 / hs.c);
        room.inv_c_d = 1.0 / hs.c;
        for (int o = 0; o < kBands; ++o) room.atten_k[o] = (float)(-0.1 * std::log2(10.0) * hs.atten[o] * hs.c);
        room.rho_c = (float)hs.rho_c;
        room.cotime = p.cutoff_length_m / hs.c;
        room.bvh_root = 0;
        room.t_eps = (float)(2e-7 * hs.scale);
        room.rec_begin = 0;
        room.R = n_receivers;
        room.src_begin = 0;
        room.nsrc = n_sources;
        room.h_oct = h_oct;
        room.oct_lo = p.oct_lo;
        room.oct_hi = p.oct_hi;
        room.is_order = p.is_order;
        room.pure_specular = p.pure_specular;
        room.max_broad = (int)std::fmin((double)max_broad, (double)(1u << 30));
        const long long room_prim[2] = {room.prim_begin, room.prim_end};
        NA_TRY(cudaMemcpyAsync(base + kOffRoom, &room, sizeof(room), cudaMemcpyHostToDevice, stream));
        NA_TRY(cudaMemcpyAsync(base + kOffRoomPrim, room_prim, sizeof(room_prim), cudaMemcpyHostToDevice, stream));
        NA_TRY(cudaMemcpyAsync(base + kOffCtl, &h_ctl, sizeof(WaveCtl), cudaMemcpyHostToDevice, stream));
        NA_TRY(cudaMemsetAsync(base + kOffCnt, 0, sizeof(DevCounters), stream));
        NA_TRY(cudaMemsetAsync(d_energy, 0, nE * sizeof(double), stream));
        NA_TRY(cudaMemsetAsync(d_pressure, 0, nE * sizeof(double), stream));
        NA_TRY(cudaMemsetAsync(d_dir_pos, 0, nD * sizeof(double), stream));
        NA_TRY(cudaMemsetAsync(d_dir_neg, 0, nD * sizeof(double), stream));
        NA_TRY(cudaMemsetAsync(d_analysis, 0, nD * sizeof(double), stream));

        DevRun r{};
        r.S = *scene_dev(scene);
        r.rec = reinterpret_cast<const float4 *>(base + kOffRec);
        r.R = n_receivers;
        r.T = (int)T;
        r.fs = (double)p.sample_rate;
        r.rooms = reinterpret_cast<const RoomParams *>(base + kOffRoom);
        r.room_prim = reinterpret_cast<const long long *>(base + kOffRoomPrim);
        r.n_rooms = 1;
        r.src = reinterpret_cast<const float4 *>(base + kOffSrc);
        r.e0 = reinterpret_cast<const float *>(base + kOffE0);
        r.geo = reinterpret_cast<const float4 *>(base + kOffGeo);
        r.prim_base = p.ray_begin;
        r.seed = p.seed;
        r.max_seg = p.max_segments_per_ray > 0 ? p.max_segments_per_ray : (1ll << 22);
        r.hE = d_energy; r.hP = d_pressure; r.hDp = d_dir_pos; r.hDn = d_dir_neg; r.hAn = d_analysis;
        r.cnt = reinterpret_cast<DevCounters *>(base + kOffCnt);
        r.ring = reinterpret_cast<ORayItem *>(base + kOffRing);
        r.ring_cap = kNaRing;
        r.ctl = reinterpret_cast<WaveCtl *>(base + kOffCtl);
        r.hits = reinterpret_cast<int4 *>(base + kOffHits);
        r.max_wave = kNaWave;
        r.feed_bound = bound;
        // Feed only into an empty ring, 8 primaries at a time: their split trees then grow alone,
        // so the fixed ring holds at most 8 trees at once.
        r.low_water = 0;
        r.feed_batch = 8;

        int sms = 0, bps_tr = 0, bps_sh = 0;
        NA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        const bool quant = use_quantised_nodes(p.bvh_format, (int)hs.tri_poly.size()) && r.S.bvhq != nullptr;
        if (!quant) r.S.bvhq = nullptr;
        const int variant = trace_variant(p.blocks_per_sm, p.traversal, (int)hs.tri_poly.size(), quant);
        NA_TRY(wave_kernel_occupancy(variant, 256, receiver_smem_bytes(n_receivers), &bps_tr, &bps_sh,
                                     fused_walk(p.traversal, (int)hs.tri_poly.size())));
        const int tr_blocks = sms * (bps_tr > 0 ? bps_tr : 1), sh_blocks = sms * (bps_sh > 0 ? bps_sh : 1);
        long long launches = 0;
        // Every iteration of the loop either traces a wave or feeds primaries, so the schedule moves on
        // each time; if it stops moving for kNaStall synchronisations in a row (kNaStall x 32
        // iterations) the call gives up instead of waiting on a loop that no longer progresses.
        unsigned long long seen_waves = 0;
        long long seen_prim = -1;
        int stalls = 0;
        for (;;) {
            for (int k = 0; k < 32; ++k) {
                NA_TRY(launch_feed(r, stream));
                NA_TRY(launch_broadband(r, sms * 2, 128, stream, false, hs.ntri <= kFuseMaxTris));
                NA_TRY(launch_wave(r, stream));
                const bool fused = fused_walk(p.traversal, (int)hs.tri_poly.size());
                if (!fused) NA_TRY(launch_trace(r, variant, tr_blocks, 256, stream));
                NA_TRY(launch_shade(r, sh_blocks, 256, stream, fused));
                launches += 5;
            }
            NA_TRY(cudaMemcpyAsync(&h_ctl, base + kOffCtl, sizeof(WaveCtl), cudaMemcpyDeviceToHost, stream));
            NA_TRY(cudaStreamSynchronize(stream));
            if (h_ctl.done) break;
            if (h_ctl.waves == seen_waves && h_ctl.next_prim == seen_prim) {
                if (++stalls >= kNaStall) return na_fail(PACH_ERR_GAVE_UP, "wavefront loop stopped making progress");
            } else {
                stalls = 0;
            }
            seen_waves = h_ctl.waves;
            seen_prim = h_ctl.next_prim;
        }
        if (h_ctl.overflow)
            return na_fail(PACH_ERR_BOUNDS, "the split trees outgrew the no-alloc ring (65536 octave rays); "
                                            "use pach_trace_begin");
        if (stats) {
            DevCounters c;
            NA_TRY(cudaMemcpyAsync(&c, base + kOffCnt, sizeof(DevCounters), cudaMemcpyDeviceToHost, stream));
            NA_TRY(cudaStreamSynchronize(stream));
            std::memset(stats, 0, sizeof(*stats));
            stats->primaries = (int64_t)c.primaries;
            stats->segments_broadband = (int64_t)c.seg_broad;
            stats->segments_phase_b = (int64_t)c.seg_b;
            stats->segments_phase_c = (int64_t)c.seg_c;
            stats->segments = stats->segments_broadband + stats->segments_phase_b + stats->segments_phase_c;
            stats->octave_rays = (int64_t)c.octave_rays;
            stats->end_traces = (int64_t)c.end_traces;
            stats->detections = (int64_t)c.detections;
            stats->capped = (int64_t)c.capped;
            stats->fp64_retests = (int64_t)c.retests;
            stats->lost_energy = c.lost_energy;
            stats->initial_energy = c.initial_energy;
            stats->percent_lost = c.initial_energy > 0 ? 100.0 * c.lost_energy / c.initial_energy : 0.0;
            stats->h_oct = h_oct;
            stats->bins = (int32_t)T;
            stats->cotime_s = room.cotime;
            stats->sound_speed = hs.c;
            stats->rho_c = hs.rho_c;
            for (int o = 0; o < kBands; ++o) stats->air_atten_db_per_m[o] = hs.atten[o];
            stats->waves = (int64_t)h_ctl.waves;
            stats->kernel_launches = launches;
            stats->peak_live_rays = (int64_t)h_ctl.peak_live;
            stats->bvh_nodes_visited = (int64_t)c.bvh_nodes;
            stats->tri_tests = (int64_t)c.tri_tests;
            stats->accel[0] = hs.bvh_nodes;
            stats->accel[1] = hs.bvh_leaves;
            stats->accel[2] = hs.bvh_depth;
            stats->wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - wall0).count();
        }
        return PACH_OK;
    }
cuda_fail:
    set_last_error((std::string(where) + ": " + cudaGetErrorString(e)).c_str());
    return PACH_ERR_CUDA;
#undef NA_TRY
}
