// capi.cpp -- the C ABI (include/pach_gpu.h): scene and run handles, the run worker, error strings.
//
// pach_trace_begin mirrors SplitRayTracer's ctor + Begin ("Classes_Complete_Trace - TaskAll.cs":68-240):
// it derives COTime and h_oct, then starts a host worker that drives the device in chunks of primary
// rays and returns at once; pach_trace_poll mirrors ThreadState/ProgressMsg; pach_trace_get_histograms
// with scaled = 1 mirrors Combine_ThreadLocal_Results (TaskAll:768-774).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "engine.h"

using namespace pach;

namespace {

thread_local std::string g_err;

pach_status fail(pach_status s, const std::string &msg) {
    g_err = msg;
    return s;
}

std::string cuda_msg(cudaError_t e, const char *what) {
    return std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
}

struct DevMem {
    void *p = nullptr;
    size_t bytes = 0;
    cudaError_t alloc(size_t n) {
        release();
        bytes = n;
        return n ? cudaMalloc(&p, n) : cudaSuccess;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <class T> T *as() const { return reinterpret_cast<T *>(p); }
};

}  // namespace

struct pach_scene {
    int device = 0;
    HostScene hs;
    DevScene dev{};
    DevMem tri, tri64, norm, mat, trans, cs, ct;
    std::mutex mu;
    ~pach_scene() {
        cudaSetDevice(device);
        for (DevMem *m : {&tri, &tri64, &norm, &mat, &trans, &cs, &ct}) m->release();
    }
};

struct pach_run {
    pach_scene *scene = nullptr;
    pach_trace_params p{};
    std::vector<pach_source_desc> src;
    std::vector<pach_receiver_desc> rec;
    std::vector<double> prim_dirs, prim_weights;
    int R = 0, T = 0, nsrc = 0, h_oct = 0;
    double cotime = 0;
    unsigned long long max_broad = 0;
    // device buffers
    DevMem hE, hP, hDp, hDn, hAn, cnt, qa, qs0, qs1, qctl, drec, dsrc, de0, dgeo, ddirs, dw;
    // worker
    std::thread worker;
    std::mutex mu;
    std::condition_variable cv;
    bool finished = false;
    std::atomic<int> state{PACH_RUN_RUNNING};
    std::atomic<bool> cancel{false};
    std::atomic<long long> rays_done{0}, end_traces{0}, segments{0};
    pach_status status = PACH_OK;
    std::string err;
    pach_stats stats{};
    ~pach_run() {
        if (worker.joinable()) {
            cancel = true;
            worker.join();
        }
        cudaSetDevice(scene ? scene->device : 0);
        for (DevMem *m : {&hE, &hP, &hDp, &hDn, &hAn, &cnt, &qa, &qs0, &qs1, &qctl, &drec, &dsrc, &de0, &dgeo, &ddirs, &dw})
            m->release();
    }
};

namespace {

cudaError_t upload(DevMem &m, const void *src, size_t bytes) {
    cudaError_t e = m.alloc(bytes);
    if (e != cudaSuccess) return e;
    return bytes ? cudaMemcpy(m.p, src, bytes, cudaMemcpyHostToDevice) : cudaSuccess;
}

// The run worker: chunks of primaries -> k_broadband -> k_octave (+ spill drains).
void run_worker(pach_run *run) {
    auto finish = [&](pach_status s, const std::string &msg, int st) {
        std::lock_guard<std::mutex> lk(run->mu);
        run->status = s;
        run->err = msg;
        run->state = st;
        run->finished = true;
        run->cv.notify_all();
    };
    auto wall0 = std::chrono::steady_clock::now();
    pach_scene *sc = run->scene;
    cudaError_t e = cudaSetDevice(sc->device);
    if (e != cudaSuccess) return finish(PACH_ERR_CUDA, cuda_msg(e, "cudaSetDevice"), PACH_RUN_FAILED);
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, eo0 = nullptr, eo1 = nullptr;
    std::string where;
    pach_status status = PACH_OK;
    std::string msg;
    int final_state = PACH_RUN_STOPPED;
    do {
#define TRY(x)                                      \
    do {                                            \
        e = (x);                                    \
        if (e != cudaSuccess) { where = #x; break; } \
    } while (0)
        TRY(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        if (e) break;
        TRY(cudaEventCreate(&ev0));
        if (e) break;
        TRY(cudaEventCreate(&ev1));
        if (e) break;
        TRY(cudaEventCreate(&eo0));
        if (e) break;
        TRY(cudaEventCreate(&eo1));
        if (e) break;
        const HostScene &hs = sc->hs;
        const int R = run->R, T = run->T;
        const size_t nE = (size_t)R * kBands * T, nD = (size_t)R * 3 * kBands * T;
        TRY(run->hE.alloc(std::max<size_t>(nE, 1) * 8)); if (e) break;
        TRY(run->hP.alloc(std::max<size_t>(nE, 1) * 8)); if (e) break;
        TRY(run->hDp.alloc(std::max<size_t>(nD, 1) * 8)); if (e) break;
        TRY(run->hDn.alloc(std::max<size_t>(nD, 1) * 8)); if (e) break;
        TRY(run->hAn.alloc(std::max<size_t>(nD, 1) * 8)); if (e) break;
        TRY(run->cnt.alloc(sizeof(DevCounters))); if (e) break;
        TRY(run->qctl.alloc(8 * sizeof(unsigned long long))); if (e) break;
        TRY(cudaMemsetAsync(run->hE.p, 0, run->hE.bytes, stream)); if (e) break;
        TRY(cudaMemsetAsync(run->hP.p, 0, run->hP.bytes, stream)); if (e) break;
        TRY(cudaMemsetAsync(run->hDp.p, 0, run->hDp.bytes, stream)); if (e) break;
        TRY(cudaMemsetAsync(run->hDn.p, 0, run->hDn.bytes, stream)); if (e) break;
        TRY(cudaMemsetAsync(run->hAn.p, 0, run->hAn.bytes, stream)); if (e) break;
        TRY(cudaMemsetAsync(run->cnt.p, 0, sizeof(DevCounters), stream)); if (e) break;
        // receivers, sources, powers, geodesic faces
        std::vector<float4> rec(std::max(R, 1));
        for (int i = 0; i < R; ++i)
            rec[i] = make_float4((float)run->rec[i].origin[0], (float)run->rec[i].origin[1], (float)run->rec[i].origin[2],
                                 (float)(run->rec[i].radius * run->rec[i].radius));
        TRY(upload(run->drec, rec.data(), rec.size() * sizeof(float4))); if (e) break;
        std::vector<float4> src(run->nsrc);
        std::vector<float> e0((size_t)run->nsrc * kBands);
        for (int s = 0; s < run->nsrc; ++s) {
            src[s] = make_float4((float)run->src[s].origin[0], (float)run->src[s].origin[1], (float)run->src[s].origin[2],
                                 (float)run->src[s].kind);
            for (int o = 0; o < kBands; ++o) e0[s * kBands + o] = (float)(1e-12 * std::pow(10.0, .1 * run->src[s].power_db[o]));
        }
        TRY(upload(run->dsrc, src.data(), src.size() * sizeof(float4))); if (e) break;
        TRY(upload(run->de0, e0.data(), e0.size() * sizeof(float))); if (e) break;
        std::vector<double> gf;
        geodesic_faces(gf);
        std::vector<float4> geo(kGeoFaces * 3);
        for (int i = 0; i < kGeoFaces * 3; ++i) geo[i] = make_float4((float)gf[3 * i], (float)gf[3 * i + 1], (float)gf[3 * i + 2], 0.f);
        TRY(upload(run->dgeo, geo.data(), geo.size() * sizeof(float4))); if (e) break;

        int dev_sms = 0;
        TRY(cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, sc->device)); if (e) break;
        const int oct_threads = run->p.block_threads > 0 ? run->p.block_threads : 256;
        int bps = run->p.blocks_per_sm;
        if (bps <= 0) {
            TRY(octave_kernel_occupancy(oct_threads, &bps)); if (e) break;
            bps = std::max(bps, 1);
        }
        const int oct_blocks = dev_sms * bps;

        // Queue sizing: every primary emits at most bound items in phase A.
        const bool pure = run->p.pure_specular != 0;
        const unsigned long long per_bounce = (unsigned long long)kBands * ((hs.has_trans && !pure) ? 3 : 1);
        const unsigned long long bound = per_bounce * run->max_broad + kBands;
        const unsigned long long budget = run->p.queue_budget_items > 0 ? (unsigned long long)run->p.queue_budget_items
                                                                        : (1ull << 25);
        const long long N = run->p.ray_count;
        long long chunk = (long long)std::max<unsigned long long>(1, budget / bound);
        chunk = std::min(chunk, N);
        const unsigned long long qa_cap = (unsigned long long)chunk * bound;
        const unsigned long long spill_cap = std::max<unsigned long long>(1ull << 20, qa_cap / 16);
        TRY(run->qa.alloc(qa_cap * sizeof(ORayItem))); if (e) break;
        TRY(run->qs0.alloc(spill_cap * sizeof(ORayItem))); if (e) break;
        TRY(run->qs1.alloc(spill_cap * sizeof(ORayItem))); if (e) break;
        if (!run->prim_dirs.empty()) { TRY(run->ddirs.alloc(sizeof(double) * 3 * chunk)); if (e) break; }
        if (!run->prim_weights.empty()) { TRY(run->dw.alloc(sizeof(double) * chunk)); if (e) break; }

        DevRun r{};
        r.S = sc->dev;
        r.rec = run->drec.as<float4>();
        r.R = R;
        r.T = T;
        r.fs = (double)run->p.sample_rate;
        r.inv_c = (float)(1.0 / hs.c);
        r.inv_c_d = 1.0 / hs.c;
        for (int o = 0; o < kBands; ++o) r.atten_k[o] = (float)(-0.1 * std::log2(10.0) * hs.atten[o] * hs.c);
        r.rho_c = (float)hs.rho_c;
        r.cotime = run->cotime;
        r.nsrc = run->nsrc;
        r.src = run->dsrc.as<float4>();
        r.e0 = run->de0.as<float>();
        r.geo = run->dgeo.as<float4>();
        r.h_oct = run->h_oct;
        r.oct_lo = run->p.oct_lo;
        r.oct_hi = run->p.oct_hi;
        r.is_order = run->p.is_order;
        r.pure_specular = run->p.pure_specular;
        r.max_broad = (int)std::min<unsigned long long>(run->max_broad, 1u << 30);
        r.seed = run->p.seed;
        r.max_seg = run->p.max_segments_per_ray > 0 ? run->p.max_segments_per_ray : (1ll << 22);
        r.hE = run->hE.as<double>(); r.hP = run->hP.as<double>(); r.hDp = run->hDp.as<double>();
        r.hDn = run->hDn.as<double>(); r.hAn = run->hAn.as<double>();
        r.cnt = run->cnt.as<DevCounters>();
        unsigned long long *ctl = run->qctl.as<unsigned long long>();  // [qa_count, qa_head, s0_count, s0_head, s1_count, s1_head]

        float oct_ms = 0.f;
        long long oct_launches = 0, launches = 0;
        int chunks = 0;
        unsigned long long *h_ctl = nullptr;
        TRY(cudaMallocHost(&h_ctl, 8 * sizeof(unsigned long long))); if (e) break;
        DevCounters *h_cnt = nullptr;
        TRY(cudaMallocHost(&h_cnt, sizeof(DevCounters))); if (e) { cudaFreeHost(h_ctl); break; }
        TRY(cudaEventRecord(ev0, stream));
        const long long first = run->p.ray_begin;
        for (long long q0 = 0; q0 < N && !e; q0 += chunk) {
            const long long q1 = std::min(N, q0 + chunk);
            const long long p0 = first + q0, p1 = first + q1;  // global primary indices (RNG keys)
            TRY(cudaMemsetAsync(ctl, 0, 8 * sizeof(unsigned long long), stream)); if (e) break;
            r.prim_base = p0;
            r.prim_dirs = nullptr;
            r.prim_weights = nullptr;
            if (!run->prim_dirs.empty()) {
                TRY(cudaMemcpyAsync(run->ddirs.p, run->prim_dirs.data() + 3 * q0, sizeof(double) * 3 * (q1 - q0),
                                    cudaMemcpyHostToDevice, stream)); if (e) break;
                r.prim_dirs = run->ddirs.as<double>();
            }
            if (!run->prim_weights.empty()) {
                TRY(cudaMemcpyAsync(run->dw.p, run->prim_weights.data() + q0, sizeof(double) * (q1 - q0),
                                    cudaMemcpyHostToDevice, stream)); if (e) break;
                r.prim_weights = run->dw.as<double>();
            }
            // phase A
            r.q_out = run->qa.as<ORayItem>();
            r.q_out_count = ctl + 0;
            r.q_out_cap = qa_cap;
            const int bb_threads = 128;
            const long long need_blocks = (p1 - p0 + bb_threads - 1) / bb_threads;
            const int bb_blocks = (int)std::max<long long>(1, std::min<long long>(need_blocks, (long long)dev_sms * 16));
            TRY(launch_broadband(r, p0, p1, bb_blocks, bb_threads, stream)); if (e) break;
            ++launches;
            // phases B and C
            // Input: the phase-A queue; output: spill queue 0.  While a launch spilled, the spill
            // queue it filled becomes the next input and the other spill queue the next output.
            ORayItem *spq[2] = {run->qs0.as<ORayItem>(), run->qs1.as<ORayItem>()};
            unsigned long long *spc[2] = {ctl + 2, ctl + 4};
            r.q_in = run->qa.as<ORayItem>();
            r.q_in_count = ctl + 0;
            r.q_in_head = ctl + 1;
            r.q_in_cap = qa_cap;
            int out_idx = 0, pass = 0;
            for (; pass < 1000; ++pass) {
                r.q_out = spq[out_idx];
                r.q_out_count = spc[out_idx];
                r.q_out_cap = spill_cap;
                TRY(cudaMemsetAsync(spc[out_idx], 0, 2 * sizeof(unsigned long long), stream)); if (e) break;
                TRY(cudaEventRecord(eo0, stream)); if (e) break;
                TRY(launch_octave(r, oct_blocks, oct_threads, stream)); if (e) break;
                TRY(cudaEventRecord(eo1, stream)); if (e) break;
                ++launches;
                ++oct_launches;
                TRY(cudaMemcpyAsync(h_ctl, ctl, 8 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, stream)); if (e) break;
                TRY(cudaStreamSynchronize(stream)); if (e) break;
                float ms = 0.f;
                TRY(cudaEventElapsedTime(&ms, eo0, eo1)); if (e) break;
                oct_ms += ms;
                if (h_ctl[2 + 2 * out_idx] == 0) break;
                r.q_in = spq[out_idx];
                r.q_in_count = spc[out_idx];
                r.q_in_head = spc[out_idx] + 1;
                r.q_in_cap = spill_cap;
                out_idx ^= 1;
            }
            if (e) break;
            if (pass >= 1000) {
                status = PACH_ERR_GAVE_UP;
                msg = "spill queue still non-empty after 1000 drain launches";
                final_state = PACH_RUN_FAILED;
                break;
            }
            TRY(cudaMemcpyAsync(h_cnt, run->cnt.p, sizeof(DevCounters), cudaMemcpyDeviceToHost, stream)); if (e) break;
            TRY(cudaStreamSynchronize(stream)); if (e) break;
            run->rays_done = q1;
            run->end_traces = (long long)h_cnt->end_traces;
            run->segments = (long long)(h_cnt->seg_broad + h_cnt->seg_b + h_cnt->seg_c);
            ++chunks;
            if (h_cnt->queue_overflow) {
                status = PACH_ERR_BOUNDS;
                msg = "device queue capacity exceeded (" + std::to_string(h_cnt->queue_overflow) + " pushes dropped)";
                final_state = PACH_RUN_FAILED;
                break;
            }
            if (run->cancel) {
                status = PACH_ERR_CANCELLED;
                msg = "run cancelled";
                final_state = PACH_RUN_CANCELLED;
                break;
            }
        }
        if (!e) { TRY(cudaEventRecord(ev1, stream)); }
        if (!e) { TRY(cudaStreamSynchronize(stream)); }
        float dev_ms = 0.f;
        if (!e) { TRY(cudaEventElapsedTime(&dev_ms, ev0, ev1)); }
        if (!e) { TRY(cudaMemcpy(h_cnt, run->cnt.p, sizeof(DevCounters), cudaMemcpyDeviceToHost)); }
        if (!e) {
            pach_stats &s = run->stats;
            s.primaries = (int64_t)h_cnt->primaries;
            s.segments_broadband = (int64_t)h_cnt->seg_broad;
            s.segments_phase_b = (int64_t)h_cnt->seg_b;
            s.segments_phase_c = (int64_t)h_cnt->seg_c;
            s.segments = s.segments_broadband + s.segments_phase_b + s.segments_phase_c;
            s.octave_rays = (int64_t)h_cnt->octave_rays;
            s.end_traces = (int64_t)h_cnt->end_traces;
            s.detections = (int64_t)h_cnt->detections;
            s.capped = (int64_t)h_cnt->capped;
            s.fp64_retests = (int64_t)h_cnt->retests;
            s.queue_overflows = (int64_t)h_cnt->queue_overflow;
            s.stack_spills = (int64_t)h_cnt->stack_spills;
            s.lost_energy = h_cnt->lost_energy;
            s.initial_energy = h_cnt->initial_energy;
            s.percent_lost = s.initial_energy > 0 ? 100.0 * s.lost_energy / s.initial_energy : 0.0;
            s.h_oct = run->h_oct;
            s.bins = T;
            s.cotime_s = run->cotime;
            s.sound_speed = hs.c;
            s.rho_c = hs.rho_c;
            for (int o = 0; o < kBands; ++o) s.air_atten_db_per_m[o] = hs.atten[o];
            s.device_ms = dev_ms;
            s.octave_kernel_ms = oct_ms;
            s.octave_kernel_launches = oct_launches;
            s.kernel_launches = launches;
            for (int k = 0; k < 3; ++k) s.grid_dims[k] = hs.dims[k];
            s.chunks = chunks;
            run->segments = s.segments;
            run->end_traces = s.end_traces;
        }
        cudaFreeHost(h_ctl);
        cudaFreeHost(h_cnt);
#undef TRY
    } while (0);
    run->stats.wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - wall0).count();
    for (cudaEvent_t ev : {ev0, ev1, eo0, eo1})
        if (ev) cudaEventDestroy(ev);
    if (stream) cudaStreamDestroy(stream);
    // release the queues; histograms and counters stay until the run is destroyed
    for (DevMem *m : {&run->qa, &run->qs0, &run->qs1, &run->ddirs, &run->dw}) m->release();
    if (e != cudaSuccess) return finish(PACH_ERR_CUDA, cuda_msg(e, where.c_str()), PACH_RUN_FAILED);
    finish(status, msg, final_state);
}

pach_status check_run(pach_run *run) {
    if (!run) return fail(PACH_ERR_INVALID_ARGUMENT, "null run handle");
    return PACH_OK;
}

}  // namespace

extern "C" {

const char *pach_version(void) { return "pach_gpu 0.1.0 (sm_103a)"; }

int pach_last_error(char *buf, size_t cap) {
    if (buf && cap) {
        size_t n = std::min(cap - 1, g_err.size());
        std::memcpy(buf, g_err.data(), n);
        buf[n] = 0;
    }
    return (int)g_err.size();
}

int pach_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

pach_status pach_medium_properties(double temp_c, double hr, double pa_hpa, int32_t air_choice, int32_t edge,
                                   double atten[PACH_BANDS], double *c, double *rho) {
    if (!atten) return fail(PACH_ERR_INVALID_ARGUMENT, "atten is null");
    if (!(pa_hpa > 0) || !(hr > 0) || air_choice < 0 || air_choice > 2)
        return fail(PACH_ERR_INVALID_ARGUMENT, "medium: pressure and humidity must be positive, air_choice 0..2");
    medium_properties(temp_c, hr, pa_hpa, air_choice, edge, atten, c, rho);
    return PACH_OK;
}

pach_status pach_scene_create(const pach_scene_desc *desc, pach_scene **out) {
    if (!out) return fail(PACH_ERR_INVALID_ARGUMENT, "out is null");
    *out = nullptr;
    if (!desc) return fail(PACH_ERR_INVALID_ARGUMENT, "desc is null");
    if (!(desc->pressure_hpa > 0) || !(desc->rel_humidity > 0) || desc->air_choice < 0 || desc->air_choice > 2)
        return fail(PACH_ERR_INVALID_ARGUMENT, "scene: pressure and humidity must be positive, air_choice 0..2");
    auto *sc = new pach_scene();
    std::string err;
    if (!build_host_scene(desc, sc->hs, err)) {
        delete sc;
        return fail(PACH_ERR_INVALID_ARGUMENT, err);
    }
    if (pach_device_count() <= 0) {
        delete sc;
        return fail(PACH_ERR_NO_DEVICE, "no CUDA device visible: the GB300 engine has no CPU fallback");
    }
    cudaGetDevice(&sc->device);
    const HostScene &hs = sc->hs;
    std::vector<float4> tri((size_t)hs.ntri * 3);
    for (int i = 0; i < hs.ntri; ++i) {
        const double *t = &hs.tri64[9 * (size_t)i];
        const double ax = t[4] * t[8] - t[5] * t[7], ay = t[5] * t[6] - t[3] * t[8], az = t[3] * t[7] - t[4] * t[6];
        const double graze = 1e-4 * std::sqrt(ax * ax + ay * ay + az * az);  // |det| < 1e-4 |e1 x e2|: near grazing
        int plane = hs.tri_plane[i], poly = hs.tri_poly[i];
        float pw, qw;
        std::memcpy(&pw, &plane, 4);
        std::memcpy(&qw, &poly, 4);
        tri[3 * i] = make_float4((float)t[0], (float)t[1], (float)t[2], pw);
        tri[3 * i + 1] = make_float4((float)t[3], (float)t[4], (float)t[5], qw);
        tri[3 * i + 2] = make_float4((float)t[6], (float)t[7], (float)t[8], (float)graze);
    }
    std::vector<float4> norm(hs.npoly), mat((size_t)hs.npoly * kBands);
    std::vector<float> trans((size_t)hs.npoly * kBands);
    for (int p = 0; p < hs.npoly; ++p) {
        norm[p] = make_float4((float)hs.normal[3 * p], (float)hs.normal[3 * p + 1], (float)hs.normal[3 * p + 2], 0.f);
        for (int o = 0; o < kBands; ++o) {
            // Lambert_Scattering thresholds (Classes_Materials.cs:4466-4485)
            const double s = hs.scat[p * 8 + o];
            double lo, hi;
            if (s < 0.25) { lo = 0.1; hi = 0.4; }
            else { const double mod = std::fabs(1 - s) / 5; lo = s - mod; hi = s + mod; }
            mat[p * kBands + o] = make_float4((float)(1.0 - hs.alpha[p * 8 + o]), (float)lo, (float)s, (float)hi);
            trans[p * kBands + o] = (float)hs.trans[p * 8 + o];
        }
    }
    cudaError_t e;
    if ((e = upload(sc->tri, tri.data(), tri.size() * sizeof(float4))) ||
        (e = upload(sc->tri64, hs.tri64.data(), hs.tri64.size() * sizeof(double))) ||
        (e = upload(sc->norm, norm.data(), norm.size() * sizeof(float4))) ||
        (e = upload(sc->mat, mat.data(), mat.size() * sizeof(float4))) ||
        (e = upload(sc->trans, trans.data(), trans.size() * sizeof(float))) ||
        (e = upload(sc->cs, hs.cell_start.data(), hs.cell_start.size() * sizeof(uint32_t))) ||
        (e = upload(sc->ct, hs.cell_tris.data(), std::max<size_t>(hs.cell_tris.size(), 1) * sizeof(uint32_t)))) {
        delete sc;
        return fail(e == cudaErrorMemoryAllocation ? PACH_ERR_OUT_OF_MEMORY : PACH_ERR_CUDA, cuda_msg(e, "scene upload"));
    }
    DevScene &d = sc->dev;
    d.tri = sc->tri.as<float4>();
    d.tri64 = sc->tri64.as<double>();
    d.pnormal = sc->norm.as<float4>();
    d.mat = sc->mat.as<float4>();
    d.trans = sc->trans.as<float>();
    d.cell_start = sc->cs.as<uint32_t>();
    d.cell_tris = sc->ct.as<uint32_t>();
    d.nx = hs.dims[0]; d.ny = hs.dims[1]; d.nz = hs.dims[2];
    d.ntri = hs.ntri;
    d.bminx = (float)hs.bmin[0]; d.bminy = (float)hs.bmin[1]; d.bminz = (float)hs.bmin[2];
    d.bmaxx = (float)hs.bmax[0]; d.bmaxy = (float)hs.bmax[1]; d.bmaxz = (float)hs.bmax[2];
    d.cellx = (float)((hs.bmax[0] - hs.bmin[0]) / hs.dims[0]);
    d.celly = (float)((hs.bmax[1] - hs.bmin[1]) / hs.dims[1]);
    d.cellz = (float)((hs.bmax[2] - hs.bmin[2]) / hs.dims[2]);
    d.icellx = (float)(hs.dims[0] / (hs.bmax[0] - hs.bmin[0]));
    d.icelly = (float)(hs.dims[1] / (hs.bmax[1] - hs.bmin[1]));
    d.icellz = (float)(hs.dims[2] / (hs.bmax[2] - hs.bmin[2]));
    d.t_eps = (float)(2e-7 * hs.scale);
    d.has_trans = hs.has_trans ? 1 : 0;
    *out = sc;
    return PACH_OK;
}

void pach_scene_destroy(pach_scene *scene) { delete scene; }

pach_status pach_scene_info(const pach_scene *scene, int32_t *n_polys, int32_t *n_triangles, double *sound_speed,
                            double *rho_c, double atten[PACH_BANDS], double *poly_area) {
    if (!scene) return fail(PACH_ERR_INVALID_ARGUMENT, "null scene");
    const HostScene &hs = scene->hs;
    if (n_polys) *n_polys = hs.npoly;
    if (n_triangles) *n_triangles = hs.ntri;
    if (sound_speed) *sound_speed = hs.c;
    if (rho_c) *rho_c = hs.rho_c;
    if (atten) for (int o = 0; o < kBands; ++o) atten[o] = hs.atten[o];
    if (poly_area) for (int p = 0; p < hs.npoly; ++p) poly_area[p] = hs.area[p];
    return PACH_OK;
}

pach_status pach_trace_begin(pach_scene *scene, const pach_source_desc *sources, int32_t n_sources,
                             const pach_receiver_desc *receivers, int32_t n_receivers, const pach_trace_params *params,
                             pach_run **out) {
    if (!out) return fail(PACH_ERR_INVALID_ARGUMENT, "out is null");
    *out = nullptr;
    if (!scene || !params) return fail(PACH_ERR_INVALID_ARGUMENT, "null scene or params");
    if (!sources || n_sources < 1 || n_sources > kMaxSources)
        return fail(PACH_ERR_INVALID_ARGUMENT, "need 1.." + std::to_string(kMaxSources) + " sources");
    if (n_receivers < 0 || (n_receivers > 0 && !receivers)) return fail(PACH_ERR_INVALID_ARGUMENT, "bad receivers");
    if (n_receivers > 2048) return fail(PACH_ERR_INVALID_ARGUMENT, "at most 2048 receivers per run");
    const pach_trace_params &p = *params;
    if (p.ray_count < 1 || p.ray_begin < 0 || p.ray_begin + p.ray_count > (1ll << 32))
        return fail(PACH_ERR_INVALID_ARGUMENT,
                    "ray_count must be >= 1 and ray_begin + ray_count <= 2^32 (convergence mode is not supported)");
    if (p.oct_lo < 0 || p.oct_hi > 7 || p.oct_lo > p.oct_hi) return fail(PACH_ERR_INVALID_ARGUMENT, "octave range must lie in 0..7");
    if (p.sample_rate < 1) return fail(PACH_ERR_INVALID_ARGUMENT, "sample_rate must be positive");
    if (!(p.cutoff_length_m > 0)) return fail(PACH_ERR_INVALID_ARGUMENT, "cutoff_length_m must be positive");
    const long long T = (long long)((double)p.sample_rate * (p.hist_cotime_ms / 1000.0));
    if (T < 1 || T > (1ll << 24)) return fail(PACH_ERR_INVALID_ARGUMENT, "histogram length must be 1..2^24 bins");
    for (int i = 0; i < n_receivers; ++i)
        if (!(receivers[i].radius > 0) || !std::isfinite(receivers[i].origin[0]) || !std::isfinite(receivers[i].origin[1]) ||
            !std::isfinite(receivers[i].origin[2]))
            return fail(PACH_ERR_INVALID_ARGUMENT, "receiver " + std::to_string(i) + ": radius must be positive, origin finite");
    for (int s = 0; s < n_sources; ++s)
        if (sources[s].kind < 0 || sources[s].kind > 2) return fail(PACH_ERR_INVALID_ARGUMENT, "unknown source kind");
    const HostScene &hs = scene->hs;
    auto *run = new pach_run();
    run->scene = scene;
    run->p = p;
    run->src.assign(sources, sources + n_sources);
    run->rec.assign(receivers, receivers + n_receivers);
    if (p.prim_dirs) run->prim_dirs.assign(p.prim_dirs, p.prim_dirs + 3 * p.ray_count);
    if (p.prim_weights) run->prim_weights.assign(p.prim_weights, p.prim_weights + p.ray_count);
    run->p.prim_dirs = nullptr;
    run->p.prim_weights = nullptr;
    run->R = n_receivers;
    run->T = (int)T;
    run->nsrc = n_sources;
    // TaskAll:83 -- the ctor's cutoff argument is a length
    run->cotime = p.cutoff_length_m / hs.c;
    // TaskAll:88-109 -- h_oct: least total absorption among bands carrying >= 1e-6 of the peak power
    // (SourceCluster power = per-band maximum over members, Classes_Sources.cs:680-688)
    double total_abs[kBands] = {0}, power[kBands] = {0};
    for (int s = 0; s < n_sources; ++s)
        for (int o = 0; o < kBands; ++o) power[o] = std::max(power[o], 1e-12 * std::pow(10.0, .1 * sources[s].power_db[o]));
    for (int q = 0; q < hs.npoly; ++q)
        for (int o = p.oct_lo; o <= p.oct_hi; ++o) total_abs[o] += hs.area[q] * hs.alpha[q * 8 + o];
    double mn = HUGE_VAL, octpower = 0;
    for (int o = p.oct_lo; o <= p.oct_hi; ++o) octpower = std::max(octpower, power[o]);
    run->h_oct = p.oct_lo;
    for (int o = p.oct_lo; o <= p.oct_hi; ++o) {
        if (power[o] < octpower * 1e-6) continue;
        if (mn > total_abs[o]) { mn = total_abs[o]; run->h_oct = o; }
    }
    if (p.max_broadband_bounces > 0) {
        run->max_broad = (unsigned long long)p.max_broadband_bounces;
    } else {
        run->max_broad = derived_broadband_bound(hs, run->h_oct, p.pure_specular != 0);
        if (run->max_broad == 0) {
            delete run;
            return fail(PACH_ERR_INVALID_ARGUMENT,
                        "a surface reflects band h_oct without loss: the broadband loop would not terminate; "
                        "set max_broadband_bounces");
        }
    }
    run->worker = std::thread(run_worker, run);
    *out = run;
    return PACH_OK;
}

pach_status pach_trace_poll(pach_run *run, pach_progress *pr) {
    if (pach_status s = check_run(run)) return s;
    if (!pr) return fail(PACH_ERR_INVALID_ARGUMENT, "progress is null");
    pr->state = run->state.load();
    {
        std::lock_guard<std::mutex> lk(run->mu);
        pr->last_status = run->status;
    }
    pr->rays_done = run->rays_done.load();
    pr->rays_total = run->p.ray_count;
    pr->end_traces = run->end_traces.load();
    pr->segments = run->segments.load();
    return PACH_OK;
}

pach_status pach_trace_cancel(pach_run *run) {
    if (pach_status s = check_run(run)) return s;
    run->cancel = true;
    return PACH_OK;
}

pach_status pach_trace_wait(pach_run *run, int64_t timeout_ms) {
    if (pach_status s = check_run(run)) return s;
    std::unique_lock<std::mutex> lk(run->mu);
    if (timeout_ms < 0) {
        run->cv.wait(lk, [&] { return run->finished; });
    } else if (!run->cv.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] { return run->finished; })) {
        return fail(PACH_ERR_TIMEOUT, "run still in progress");
    }
    lk.unlock();
    if (run->worker.joinable()) run->worker.join();
    if (run->status != PACH_OK) return fail(run->status, run->err);
    return PACH_OK;
}

pach_status pach_trace_get_histograms(pach_run *run, int32_t scaled, double *energy, double *pressure, double *dir_pos,
                                      double *dir_neg, double *analysis, size_t cap_bins) {
    if (pach_status s = check_run(run)) return s;
    {
        std::lock_guard<std::mutex> lk(run->mu);
        if (!run->finished) return fail(PACH_ERR_NOT_READY, "run still in progress");
        if (run->status != PACH_OK && run->status != PACH_ERR_CANCELLED) return fail(run->status, run->err);
    }
    const size_t nE = (size_t)run->R * kBands * run->T, nD = nE * 3;
    if (cap_bins < nE) return fail(PACH_ERR_INVALID_ARGUMENT, "cap_bins < receivers * 8 * bins");
    cudaSetDevice(run->scene->device);
    const double N = (double)std::max<long long>(1, run->rays_done.load());
    const double ns = (double)run->nsrc;
    // Receiver_Bank.Scale(N) then, for a cluster, Scale(1/n_sources) (TaskAll:770-771)
    const double fE = ns / N, fP = std::sqrt(ns) / std::sqrt(N);
    struct Item { double *dst; DevMem *src; size_t n; double f; };
    const Item items[5] = {{energy, &run->hE, nE, fE}, {pressure, &run->hP, nE, fP}, {dir_pos, &run->hDp, nD, fE},
                           {dir_neg, &run->hDn, nD, fE}, {analysis, &run->hAn, nD, fE}};
    for (const Item &it : items) {
        if (!it.dst || it.n == 0) continue;
        cudaError_t e = cudaMemcpy(it.dst, it.src->p, it.n * sizeof(double), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return fail(PACH_ERR_CUDA, cuda_msg(e, "histogram copy"));
        if (scaled)
            for (size_t i = 0; i < it.n; ++i) it.dst[i] *= it.f;
    }
    return PACH_OK;
}

pach_status pach_trace_get_stats(pach_run *run, pach_stats *stats) {
    if (pach_status s = check_run(run)) return s;
    if (!stats) return fail(PACH_ERR_INVALID_ARGUMENT, "stats is null");
    std::lock_guard<std::mutex> lk(run->mu);
    if (!run->finished) return fail(PACH_ERR_NOT_READY, "run still in progress");
    *stats = run->stats;
    return PACH_OK;
}

void pach_run_destroy(pach_run *run) { delete run; }

pach_status pach_trace_run(pach_scene *scene, const pach_source_desc *sources, int32_t n_sources,
                           const pach_receiver_desc *receivers, int32_t n_receivers, const pach_trace_params *params,
                           int32_t scaled, double *energy, double *pressure, double *dir_pos, double *dir_neg,
                           double *analysis, size_t cap_bins, pach_stats *stats) {
    pach_run *run = nullptr;
    pach_status s = pach_trace_begin(scene, sources, n_sources, receivers, n_receivers, params, &run);
    if (s) return s;
    s = pach_trace_wait(run, -1);
    if (!s) s = pach_trace_get_histograms(run, scaled, energy, pressure, dir_pos, dir_neg, analysis, cap_bins);
    if (!s && stats) s = pach_trace_get_stats(run, stats);
    std::string keep = g_err;
    pach_run_destroy(run);
    g_err = keep;
    return s;
}

pach_status pach_trace_specular_paths(pach_scene *scene, int32_t n, const double *origins, const double *dirs,
                                      int32_t max_bounces, int32_t *poly_out, double *t_out, double *pts_out) {
    if (!scene || n < 0 || max_bounces < 1 || !origins || !dirs || !poly_out || !t_out || !pts_out)
        return fail(PACH_ERR_INVALID_ARGUMENT, "bad arguments");
    if (n == 0) return PACH_OK;
    cudaSetDevice(scene->device);
    DevMem o, d, pl, t, pt;
    const size_t k = (size_t)n * max_bounces;
    cudaError_t e;
    if ((e = upload(o, origins, sizeof(double) * 3 * n)) || (e = upload(d, dirs, sizeof(double) * 3 * n)) ||
        (e = pl.alloc(sizeof(int32_t) * k)) || (e = t.alloc(sizeof(double) * k)) || (e = pt.alloc(sizeof(double) * 3 * k)) ||
        (e = launch_paths(scene->dev, n, o.as<double>(), d.as<double>(), max_bounces, pl.as<int>(), t.as<double>(),
                          pt.as<double>(), 0)) ||
        (e = cudaMemcpy(poly_out, pl.p, sizeof(int32_t) * k, cudaMemcpyDeviceToHost)) ||
        (e = cudaMemcpy(t_out, t.p, sizeof(double) * k, cudaMemcpyDeviceToHost)) ||
        (e = cudaMemcpy(pts_out, pt.p, sizeof(double) * 3 * k, cudaMemcpyDeviceToHost)))
        return fail(PACH_ERR_CUDA, cuda_msg(e, "specular paths"));
    return PACH_OK;
}

pach_status pach_emit_directions(uint64_t seed, int64_t ray_begin, int32_t n, int32_t n_sources, int32_t kind,
                                 double *dirs_out) {
    if (n < 0 || n_sources < 1 || n_sources > kMaxSources || kind < 0 || kind > 2 || !dirs_out)
        return fail(PACH_ERR_INVALID_ARGUMENT, "bad arguments");
    if (n == 0) return PACH_OK;
    if (pach_device_count() <= 0) return fail(PACH_ERR_NO_DEVICE, "no CUDA device visible");
    std::vector<float4> src(n_sources, make_float4(0, 0, 0, (float)kind));
    std::vector<double> gf;
    geodesic_faces(gf);
    std::vector<float4> geo(kGeoFaces * 3);
    for (int i = 0; i < kGeoFaces * 3; ++i) geo[i] = make_float4((float)gf[3 * i], (float)gf[3 * i + 1], (float)gf[3 * i + 2], 0.f);
    DevMem ds, dg, dout;
    cudaError_t e;
    DevRun r{};
    r.seed = seed;
    r.nsrc = n_sources;
    if ((e = upload(ds, src.data(), src.size() * sizeof(float4))) || (e = upload(dg, geo.data(), geo.size() * sizeof(float4))) ||
        (e = dout.alloc(sizeof(double) * 3 * n)))
        return fail(PACH_ERR_CUDA, cuda_msg(e, "emit setup"));
    r.src = ds.as<float4>();
    r.geo = dg.as<float4>();
    if ((e = launch_emit(r, ray_begin, n, dout.as<double>(), 0)) ||
        (e = cudaMemcpy(dirs_out, dout.p, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost)))
        return fail(PACH_ERR_CUDA, cuda_msg(e, "emit"));
    return PACH_OK;
}

}  // extern "C"
