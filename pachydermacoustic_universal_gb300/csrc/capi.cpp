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
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
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
    DevMem tri, tri64, norm, mat, trans, bvh, bvhq;
    // the device copy above exists (pach_scene_create makes it at once; pach_scenes_create leaves it to the
    // first single-room use, since a batch run uploads the concatenation of its rooms instead)
    bool on_device = false;
    std::mutex mu;  // guards the first upload
    ~pach_scene() {
        cudaSetDevice(device);
        for (DevMem *m : {&tri, &tri64, &norm, &mat, &trans, &bvh, &bvhq}) m->release();
    }
};

// One room of a run: a scene handle, its sources and receivers, its primaries and cutoff, and the
// values the SplitRayTracer ctor derives from them (TaskAll:68-177).
struct RoomSpec {
    pach_scene *scene = nullptr;
    std::vector<pach_source_desc> src;
    std::vector<pach_receiver_desc> rec;
    long long rays = 0, prim_begin = 0;
    double cutoff_len = 0, cotime = 0;
    int h_oct = 0;
    unsigned long long max_broad = 0;
};

struct pach_run {
    pach_scene *scene = nullptr;  // the first room's scene (device and single-room fast path)
    pach_trace_params p{};
    std::vector<RoomSpec> rooms;
    std::vector<double> prim_dirs, prim_weights;
    std::vector<float> prop;  // learned-proposal lobe table ([n_proposal][kLobes][8])
    int R = 0, T = 0, nsrc = 0;   // receivers and sources over all rooms
    // device buffers
    DevMem hE, hP, hDp, hDn, hAn, cnt, qa, qs0, qs1, qctl, drec, dsrc, de0, dgeo, ddirs, dw, sortbins, dprop, dcap;
    DevMem droom, droomprim, btri, btri64, bnorm, bmat, btrans, bbvh, bbvhq;
    // mapping receivers (has_map): the host grid and its device copy, histograms [M][8][Tm]
    bool has_map = false;
    MapGrid mg;
    std::vector<double> map_org;
    DevMem mrec, mdir, mcell, mentry, mE, mP, mDp, mDn, drecid;
    // convergence mode (ray_count < 1): -1 off, 0 SpecMin, 1 Minimum; the checks, their receivers, the
    // per-revolution capture and the pre-chunk copies of the histograms and counters
    int conv_mode = -1;
    int conv_rows[2] = {-1, -1};
    long long conv_period = 80, conv_revs = 0;
    bool conv_converged = false;
    std::vector<ConvCheck> conv_checks;
    DevMem conv, bak[6];
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
        for (DevMem *m : {&hE, &hP, &hDp, &hDn, &hAn, &cnt, &qa, &qs0, &qs1, &qctl, &drec, &dsrc, &de0, &dgeo, &ddirs, &dw,
                          &sortbins, &dprop, &dcap, &droom, &droomprim, &btri, &btri64, &bnorm, &bmat, &btrans, &bbvh, &bbvhq,
                          &mrec, &mdir, &mcell, &mentry, &mE, &mP, &mDp, &mDn, &drecid, &conv, &bak[0], &bak[1], &bak[2],
                          &bak[3], &bak[4], &bak[5]})
            m->release();
    }
};

namespace {

// primaries of a run over all its rooms
long long rprim_total(const pach_run *run) {
    long long n = 0;
    for (const RoomSpec &rm : run->rooms) n += rm.rays;
    return n;
}

cudaError_t upload(DevMem &m, const void *src, size_t bytes) {
    cudaError_t e = m.alloc(bytes);
    if (e != cudaSuccess) return e;
    return bytes ? cudaMemcpy(m.p, src, bytes, cudaMemcpyHostToDevice) : cudaSuccess;
}

// Device layout of scenes: triangles (FP32 with plane and polygon ids), FP64 triangles, polygon
// normals, materials, transmission and the 4-wide BVH.  A batch run appends several scenes into one
// set of arrays: triangle, polygon, plane and node ids are offset, and each scene's root is kept.
struct SceneArrays {
    hvec<float4> tri, norm, mat;
    hvec<float> trans, bvh, bvhq;
    hvec<double> tri64;
    int planes = 0;
    float t_eps = 0.f;
    bool has_trans = false;
};

// Rebases one node array's child codes by node and triangle offsets (codes at `code_at` in each node
// of `stride` floats).
static void rebase_codes(float *nodes, size_t count, int stride, int code_at, int node_off, int tri_off) {
    parallel_chunks(count, 16384, [=](size_t q0, size_t q1) {
        for (size_t q = q0; q < q1; ++q)
            for (int k = 0; k < 4; ++k) {
                float *f = nodes + q * stride + code_at + k;
                int code;
                std::memcpy(&code, f, 4);
                if (code == (int)0x80000000) continue;       // empty slot
                if (code >= 0) code += node_off;              // inner child
                else {                                        // leaf ~(first * 16 + count - 1)
                    const int c = ~code;
                    code = ~(((c >> 4) + tri_off) * 16 + (c & 15));
                }
                std::memcpy(f, &code, 4);
            }
    });
}

// Rebases 48-byte quantised nodes (see quantize_bvh): the first inner child's node id and the first
// leaf triangle, which keeps its 24 bits (append_scene drops the quantised copy of a batch beyond that).
static void rebase_qnodes(float *nodes, size_t count, int node_off, int tri_off) {
    parallel_chunks(count, 16384, [=](size_t q0, size_t q1) {
        for (size_t q = q0; q < q1; ++q) {
            float *g = nodes + q * kBvhQNodeFloats;
            uint32_t nb, tw;
            std::memcpy(&nb, &g[10], 4);
            std::memcpy(&tw, &g[11], 4);
            nb += (uint32_t)node_off;
            tw = (((tw & 0xFFFFFFu) + (uint32_t)tri_off) & 0xFFFFFFu) | (tw & 0xFF000000u);
            std::memcpy(&g[10], &nb, 4);
            std::memcpy(&g[11], &tw, 4);
        }
    });
}

int append_scene(const HostScene &hs, SceneArrays &A) {
    const int tri_off = (int)(A.tri.size() / 3), poly_off = (int)A.norm.size(), plane_off = A.planes;
    const int node_off = (int)(A.bvh.size() / kBvhNodeFloats);
    const size_t t0 = A.tri.size(), d0 = A.tri64.size(), n0 = A.norm.size(), m0 = A.mat.size();
    A.tri.resize(t0 + 3 * (size_t)hs.ntri);
    A.tri64.resize(d0 + 9 * (size_t)hs.ntri);
    A.norm.resize(n0 + (size_t)hs.npoly);
    A.mat.resize(m0 + (size_t)kBands * hs.npoly);
    A.trans.resize(m0 + (size_t)kBands * hs.npoly);
    constexpr size_t kGrain = 65536;
    std::vector<int> chunk_plane(((size_t)hs.ntri + kGrain - 1) / kGrain, -1);
    parallel_chunks((size_t)hs.ntri, kGrain, [&](size_t i0, size_t i1) {
        int mp = -1;
        for (size_t i = i0; i < i1; ++i) {
            const double *t = &hs.tri64[9 * i];
            const double ax = t[4] * t[8] - t[5] * t[7], ay = t[5] * t[6] - t[3] * t[8], az = t[3] * t[7] - t[4] * t[6];
            const double graze = 1e-4 * std::sqrt(ax * ax + ay * ay + az * az);  // |det| < 1e-4 |e1 x e2|: near grazing
            int plane = hs.tri_plane[i] + plane_off, poly = hs.tri_poly[i] + poly_off;
            mp = std::max(mp, (int)hs.tri_plane[i]);
            float pw, qw;
            std::memcpy(&pw, &plane, 4);
            std::memcpy(&qw, &poly, 4);
            float4 *o = &A.tri[t0 + 3 * i];
            o[0] = make_float4((float)t[0], (float)t[1], (float)t[2], pw);
            o[1] = make_float4((float)t[3], (float)t[4], (float)t[5], qw);
            o[2] = make_float4((float)t[6], (float)t[7], (float)t[8], (float)graze);
            std::copy(t, t + 9, &A.tri64[d0 + 9 * i]);
        }
        chunk_plane[i0 / kGrain] = mp;
    });
    int max_plane = -1;
    for (int m : chunk_plane) max_plane = std::max(max_plane, m);
    A.planes = plane_off + max_plane + 1;
    parallel_chunks((size_t)hs.npoly, 16384, [&](size_t p0, size_t p1) {
        for (size_t p = p0; p < p1; ++p) {
            A.norm[n0 + p] = make_float4((float)hs.normal[3 * p], (float)hs.normal[3 * p + 1], (float)hs.normal[3 * p + 2], 0.f);
            for (int o = 0; o < kBands; ++o) {
                // Lambert_Scattering thresholds (Classes_Materials.cs:4466-4485)
                const double s = hs.scat[p * 8 + o];
                double lo, hi;
                if (s < 0.25) { lo = 0.1; hi = 0.4; }
                else { const double mod = std::fabs(1 - s) / 5; lo = s - mod; hi = s + mod; }
                A.mat[m0 + p * kBands + o] = make_float4((float)(1.0 - hs.alpha[p * 8 + o]), (float)lo, (float)s, (float)hi);
                A.trans[m0 + p * kBands + o] = (float)hs.trans[p * 8 + o];
            }
        }
    });
    const size_t b0 = A.bvh.size();
    A.bvh.insert(A.bvh.end(), hs.bvh.begin(), hs.bvh.end());
    // a quantised copy only when every scene of the array has one and the triangle ids fit 24 bits
    const bool quant = (node_off == 0 || !A.bvhq.empty()) && !hs.bvhq.empty() &&
                       (long long)tri_off + hs.ntri <= (1ll << 24);
    if (!quant) A.bvhq.clear();
    const size_t q0 = A.bvhq.size();
    if (quant) A.bvhq.insert(A.bvhq.end(), hs.bvhq.begin(), hs.bvhq.end());
    if (tri_off || node_off) {
        rebase_codes(&A.bvh[b0], hs.bvh.size() / kBvhNodeFloats, kBvhNodeFloats, 24, node_off, tri_off);
        if (quant) rebase_qnodes(&A.bvhq[q0], hs.bvhq.size() / kBvhQNodeFloats, node_off, tri_off);
    }
    A.t_eps = std::max(A.t_eps, (float)(2e-7 * hs.scale));
    A.has_trans = A.has_trans || hs.has_trans;
    return node_off;
}

cudaError_t upload_scene(const SceneArrays &A, DevMem &tri, DevMem &tri64, DevMem &norm, DevMem &mat, DevMem &trans,
                         DevMem &bvh, DevMem &bvhq, DevScene &d) {
    cudaError_t e;
    if ((e = upload(tri, A.tri.data(), A.tri.size() * sizeof(float4))) ||
        (e = upload(tri64, A.tri64.data(), A.tri64.size() * sizeof(double))) ||
        (e = upload(norm, A.norm.data(), A.norm.size() * sizeof(float4))) ||
        (e = upload(mat, A.mat.data(), A.mat.size() * sizeof(float4))) ||
        (e = upload(trans, A.trans.data(), A.trans.size() * sizeof(float))) ||
        (e = upload(bvh, A.bvh.data(), A.bvh.size() * sizeof(float))) ||
        (e = upload(bvhq, A.bvhq.data(), A.bvhq.size() * sizeof(float))))
        return e;
    d.bvhq = bvhq.as<float4>();
    d.tri = tri.as<float4>();
    d.tri64 = tri64.as<double>();
    d.pnormal = norm.as<float4>();
    d.mat = mat.as<float4>();
    d.trans = trans.as<float>();
    d.bvh = bvh.as<float4>();
    d.ntri = (int)(A.tri.size() / 3);
    d.t_eps = A.t_eps;
    d.has_trans = A.has_trans ? 1 : 0;
    return cudaSuccess;
}

// The scene's own device arrays, uploaded on first use (single-room runs, the specular-path and
// direct-sound probes); the caller has made the scene's device current.
cudaError_t scene_upload(pach_scene *sc) {
    std::lock_guard<std::mutex> lk(sc->mu);
    if (sc->on_device) return cudaSuccess;
    SceneArrays A;
    append_scene(sc->hs, A);
    const cudaError_t e = upload_scene(A, sc->tri, sc->tri64, sc->norm, sc->mat, sc->trans, sc->bvh, sc->bvhq, sc->dev);
    if (e == cudaSuccess) sc->on_device = true;
    return e;
}

// SplitRayTracer ctor values of one room (TaskAll:83-109): COTime from the cutoff length, h_oct (the
// band of least total absorption among bands carrying >= 1e-6 of the peak power; a SourceCluster's
// power is the per-band maximum over members, Classes_Sources.cs:680-688) and the phase-A bound.
bool room_setup(RoomSpec &rm, const pach_trace_params &p, std::string &err) {
    const HostScene &hs = rm.scene->hs;
    rm.cotime = rm.cutoff_len / hs.c;
    double total_abs[kBands] = {0}, power[kBands] = {0};
    for (const pach_source_desc &s : rm.src)
        for (int o = 0; o < kBands; ++o) power[o] = std::max(power[o], 1e-12 * std::pow(10.0, .1 * s.power_db[o]));
    for (int q = 0; q < hs.npoly; ++q)
        for (int o = p.oct_lo; o <= p.oct_hi; ++o) total_abs[o] += hs.area[q] * hs.alpha[q * 8 + o];
    double mn = HUGE_VAL, octpower = 0;
    for (int o = p.oct_lo; o <= p.oct_hi; ++o) octpower = std::max(octpower, power[o]);
    rm.h_oct = p.oct_lo;
    for (int o = p.oct_lo; o <= p.oct_hi; ++o) {
        if (power[o] < octpower * 1e-6) continue;
        if (mn > total_abs[o]) { mn = total_abs[o]; rm.h_oct = o; }
    }
    if (p.max_broadband_bounces > 0) {
        rm.max_broad = (unsigned long long)p.max_broadband_bounces;
    } else {
        rm.max_broad = derived_broadband_bound(hs, rm.h_oct, p.pure_specular != 0);
        if (rm.max_broad == 0) {
            err = "a surface reflects band h_oct without loss: the broadband loop would not terminate; "
                  "set max_broadband_bounces";
            return false;
        }
    }
    return true;
}

// The run worker: uploads the run's inputs, then drives the wavefront loop on one stream --
// iterations of feed -> broadband -> wave -> trace -> shade.  By default the whole loop is one CUDA
// graph launch: the iteration is captured into the body of a conditional while node whose last kernel
// (k_cond) ends the loop when the run is done; progress and cancellation go through mapped host
// memory.  With kernel_timing = 1 the host launches batches of iterations instead, with CUDA events
// around every kernel.
void run_worker_body(pach_run *run);

// The run's host thread: a C++ exception (a failed host allocation) ends the run as failed instead of
// ending the process.
void run_worker(pach_run *run) {
    try {
        run_worker_body(run);
    } catch (const std::exception &ex) {
        std::lock_guard<std::mutex> lk(run->mu);
        run->status = PACH_ERR_OUT_OF_MEMORY;
        run->err = std::string("host resources exhausted: ") + ex.what();
        run->state = PACH_RUN_FAILED;
        run->finished = true;
        run->cv.notify_all();
    }
}

void run_worker_body(pach_run *run) {
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
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::vector<cudaEvent_t> kev;  // per-kernel timing events (kernel_timing = 1)
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    std::string where;
    pach_status status = PACH_OK;
    std::string msg;
    int final_state = PACH_RUN_STOPPED;
    WaveCtl *h_ctl = nullptr;
    DevCounters *h_cnt = nullptr;
    HostMirror *h_mirror = nullptr;
    int *h_cancel = nullptr;
    const int n_rooms = (int)run->rooms.size();
    do {
#define TRY(x)                                        \
    {                                                 \
        e = (x);                                      \
        if (e != cudaSuccess) { where = #x; break; }  \
    }
        TRY(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        TRY(cudaEventCreate(&ev0));
        TRY(cudaEventCreate(&ev1));
        TRY(cudaMallocHost(&h_ctl, sizeof(WaveCtl)));
        TRY(cudaMallocHost(&h_cnt, sizeof(DevCounters)));
        const int R = run->R, T = run->T;
        const size_t nE = (size_t)R * kBands * T, nD = (size_t)R * 3 * kBands * T;
        TRY(run->hE.alloc(std::max<size_t>(nE, 1) * 8));
        TRY(run->hP.alloc(std::max<size_t>(nE, 1) * 8));
        TRY(run->hDp.alloc(std::max<size_t>(nD, 1) * 8));
        TRY(run->hDn.alloc(std::max<size_t>(nD, 1) * 8));
        TRY(run->hAn.alloc(std::max<size_t>(nD, 1) * 8));
        TRY(run->cnt.alloc(sizeof(DevCounters)));
        TRY(run->qctl.alloc(sizeof(WaveCtl)));
        for (DevMem *m : {&run->hE, &run->hP, &run->hDp, &run->hDn, &run->hAn, &run->cnt, &run->qctl})
            TRY(cudaMemsetAsync(m->p, 0, m->bytes, stream));
        if (e) break;

        // scene: the first room's own device arrays, or the concatenation of every room's
        if (n_rooms == 1) TRY(scene_upload(sc));
        DevScene S = sc->dev;
        std::vector<int> roots(n_rooms, 0);
        if (n_rooms > 1) {
            SceneArrays A;
            for (int i = 0; i < n_rooms; ++i) roots[i] = append_scene(run->rooms[i].scene->hs, A);
            TRY(upload_scene(A, run->btri, run->btri64, run->bnorm, run->bmat, run->btrans, run->bbvh, run->bbvhq, S));
        }
        // receivers, sources, powers and room table over all rooms
        std::vector<float4> rec(std::max(R, 1)), src;
        std::vector<int> rec_id(std::max(R, 1), 0);
        std::vector<float> e0;
        std::vector<RoomParams> rp(n_rooms);
        std::vector<long long> rprim(n_rooms + 1);
        double bmin[3] = {HUGE_VAL, HUGE_VAL, HUGE_VAL}, bmax[3] = {-HUGE_VAL, -HUGE_VAL, -HUGE_VAL};
        unsigned long long bound = 0;
        int ntri_max = 0;
        bool has_trans = false;
        const bool pure = run->p.pure_specular != 0;
        for (int i = 0, k = 0; i < n_rooms; ++i) {
            const RoomSpec &rm = run->rooms[i];
            const HostScene &hs = rm.scene->hs;
            RoomParams &P = rp[i];
            P.prim_begin = rm.prim_begin;
            P.prim_end = rm.prim_begin + rm.rays;
            rprim[i] = rm.prim_begin;
            P.inv_c_d = 1.0 / hs.c;
            P.inv_c = (float)(1.0 / hs.c);
            P.cotime = rm.cotime;
            P.rho_c = (float)hs.rho_c;
            for (int o = 0; o < kBands; ++o) P.atten_k[o] = (float)(-0.1 * std::log2(10.0) * hs.atten[o] * hs.c);
            P.bvh_root = roots[i];
            P.t_eps = (float)(2e-7 * hs.scale);
            P.rec_begin = k;
            P.R = (int)rm.rec.size();
            // the room's receivers ordered by the coordinate of their widest spread; rec_id keeps each
            // slot's histogram row
            {
                double lo[3] = {HUGE_VAL, HUGE_VAL, HUGE_VAL}, hi[3] = {-HUGE_VAL, -HUGE_VAL, -HUGE_VAL};
                for (const pach_receiver_desc &q : rm.rec)
                    for (int a = 0; a < 3; ++a) { lo[a] = std::min(lo[a], q.origin[a]); hi[a] = std::max(hi[a], q.origin[a]); }
                int ax = 0;
                for (int a = 1; a < 3; ++a)
                    if (hi[a] - lo[a] > hi[ax] - lo[ax]) ax = a;
                std::vector<int> ord(rm.rec.size());
                for (size_t i = 0; i < ord.size(); ++i) ord[i] = (int)i;
                std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) {
                    return (float)rm.rec[a].origin[ax] < (float)rm.rec[b].origin[ax];
                });
                for (int i : ord) {
                    const pach_receiver_desc &q = rm.rec[(size_t)i];
                    rec_id[k] = P.rec_begin + i;
                    rec[k++] = make_float4((float)q.origin[0], (float)q.origin[1], (float)q.origin[2],
                                           (float)(q.radius * q.radius));
                }
            }
            P.src_begin = (int)src.size();
            P.nsrc = (int)rm.src.size();
            for (const pach_source_desc &s : rm.src) {
                src.push_back(make_float4((float)s.origin[0], (float)s.origin[1], (float)s.origin[2], (float)s.kind));
                for (int o = 0; o < kBands; ++o) e0.push_back((float)(1e-12 * std::pow(10.0, .1 * s.power_db[o])));
            }
            P.h_oct = rm.h_oct;
            P.oct_lo = run->p.oct_lo;
            P.oct_hi = run->p.oct_hi;
            P.is_order = run->p.is_order;
            P.pure_specular = run->p.pure_specular;
            P.max_broad = (int)std::min<unsigned long long>(rm.max_broad, 1u << 30);
            const unsigned long long per_bounce = (unsigned long long)kBands * ((hs.has_trans && !pure) ? 3 : 1);
            bound = std::max(bound, per_bounce * rm.max_broad + kBands);
            ntri_max = std::max(ntri_max, hs.ntri);
            has_trans = has_trans || hs.has_trans;
            for (int a = 0; a < 3; ++a) {
                bmin[a] = std::min(bmin[a], hs.bmin[a]);
                bmax[a] = std::max(bmax[a], hs.bmax[a]);
            }
        }
        rprim[n_rooms] = rp[n_rooms - 1].prim_end;
        TRY(upload(run->drec, rec.data(), rec.size() * sizeof(float4)));
        TRY(upload(run->drecid, rec_id.data(), rec_id.size() * sizeof(int)));
        TRY(upload(run->dsrc, src.data(), src.size() * sizeof(float4)));
        TRY(upload(run->de0, e0.data(), e0.size() * sizeof(float)));
        TRY(upload(run->droom, rp.data(), rp.size() * sizeof(RoomParams)));
        TRY(upload(run->droomprim, rprim.data(), rprim.size() * sizeof(long long)));
        std::vector<double> gf;
        geodesic_faces(gf);
        std::vector<float4> geo(kGeoFaces * 3);
        for (int i = 0; i < kGeoFaces * 3; ++i) geo[i] = make_float4((float)gf[3 * i], (float)gf[3 * i + 1], (float)gf[3 * i + 2], 0.f);
        TRY(upload(run->dgeo, geo.data(), geo.size() * sizeof(float4)));
        if (!run->prim_dirs.empty()) TRY(upload(run->ddirs, run->prim_dirs.data(), run->prim_dirs.size() * sizeof(double)));
        if (!run->prim_weights.empty()) TRY(upload(run->dw, run->prim_weights.data(), run->prim_weights.size() * sizeof(double)));
        if (!run->prop.empty()) TRY(upload(run->dprop, run->prop.data(), run->prop.size() * sizeof(float)));
        if (run->p.capture) {
            const size_t per = run->p.capture == 2 ? (size_t)(rprim_total(run)) : (size_t)kDirBins;
            TRY(run->dcap.alloc((size_t)std::max(R, 1) * kCaptureWindows * per * sizeof(float)));
            TRY(cudaMemset(run->dcap.p, 0, run->dcap.bytes));
        }

        const bool map = run->has_map;
        if (map) {
            const MapGrid &g = run->mg;
            std::vector<float4> mr((size_t)g.M);
            for (int k = 0; k < g.M; ++k)
                mr[(size_t)k] = make_float4((float)run->map_org[3 * (size_t)k], (float)run->map_org[3 * (size_t)k + 1],
                                            (float)run->map_org[3 * (size_t)k + 2], (float)g.r2);
            TRY(upload(run->mrec, mr.data(), mr.size() * sizeof(float4)));
            TRY(upload(run->mdir, g.direct.data(), g.direct.size() * sizeof(double)));
            TRY(upload(run->mcell, g.cell_off.data(), g.cell_off.size() * sizeof(int)));
            TRY(upload(run->mentry, g.entry.data(), std::max<size_t>(g.entry.size(), 1) * sizeof(uint2)));
            const size_t nm = (size_t)g.M * kBands * g.T;
            TRY(run->mE.alloc(nm * sizeof(double)));
            TRY(run->mP.alloc(nm * sizeof(double)));
            TRY(cudaMemsetAsync(run->mE.p, 0, run->mE.bytes, stream));
            TRY(cudaMemsetAsync(run->mP.p, 0, run->mP.bytes, stream));
            if (g.directional) {
                TRY(run->mDp.alloc(3 * nm * sizeof(double)));
                TRY(run->mDn.alloc(3 * nm * sizeof(double)));
                TRY(cudaMemsetAsync(run->mDp.p, 0, run->mDp.bytes, stream));
                TRY(cudaMemsetAsync(run->mDn.p, 0, run->mDn.bytes, stream));
            }
        }

        // launch shapes: one resident wave of blocks for the trace and shade kernels
        int dev_sms = 0;
        TRY(cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, sc->device));
        const int threads = run->p.block_threads > 0 ? std::max(32, std::min(256, run->p.block_threads / 32 * 32)) : 256;
        int bps_tr = 0, bps_sh = 0;
        // blocks_per_sm picks the trace kernel's register variant (3..6 blocks of 256 per SM)
        const bool quant = use_quantised_nodes(run->p.bvh_format, ntri_max) && S.bvhq != nullptr;
        if (!quant) S.bvhq = nullptr;  // trace_ray walks whichever node array is set
        const int tr_variant = trace_variant(run->p.blocks_per_sm, run->p.traversal, ntri_max, quant);
        const bool fused = fused_walk(run->p.traversal, ntri_max) && run->p.ray_sort <= 0;
        size_t rec_max = 0;
        for (const RoomSpec &rm : run->rooms) rec_max = std::max(rec_max, rm.rec.size());
        const bool wide = rec_max >= (size_t)kShadeWideReceivers;
        TRY(wave_kernel_occupancy(tr_variant, threads, receiver_smem_bytes(R), &bps_tr, &bps_sh, fused, wide));
        const int tr_blocks = dev_sms * std::max(bps_tr, 1), sh_blocks = dev_sms * std::max(bps_sh, 1);

        // ring and wave sizing
        // default ring: room for the run's rays at up to 2048 live octave rays per primary, 2^22..2^28
        // (17 GB); default wave 8M rays -- measured against 2M: +7 % on a 20k-triangle hall and a
        // 500k-triangle arena, +19 % on a 12-triangle shoebox (fewer, fuller iterations)
        int ring_default = 22;
        while (ring_default < 28 && (1ull << ring_default) < (unsigned long long)rprim_total(run) * 2048ull) ++ring_default;
        const int ring_log2 = run->p.ring_log2 > 0 ? std::min(32, std::max(16, run->p.ring_log2)) : ring_default;
        const unsigned long long ring_cap = 1ull << ring_log2;
        const unsigned long long max_wave = run->p.wave_kilo_items > 0 ? 1024ull * run->p.wave_kilo_items : (1ull << 23);
        if (bound * 4 > ring_cap) {
            status = PACH_ERR_BOUNDS;
            msg = "the ring queue (2^" + std::to_string(ring_log2) + " rays) cannot hold the phase-A output of one "
                  "primary (" + std::to_string(bound) + " rays); raise ring_log2 or set max_broadband_bounces";
            final_state = PACH_RUN_FAILED;
            break;
        }
        TRY(run->qa.alloc(ring_cap * sizeof(ORayItem)));
        TRY(run->qs0.alloc(std::min(max_wave, ring_cap) * sizeof(int4)));
        const bool sorting = run->p.ray_sort > 0;
        if (sorting) {
            TRY(run->qs1.alloc(std::min(max_wave, ring_cap) * sizeof(ORayItem)));
            TRY(run->sortbins.alloc(2 * kSortBins * sizeof(unsigned)));
            TRY(cudaMemsetAsync(run->sortbins.p, 0, run->sortbins.bytes, stream));
        }
        const int sort_blocks = dev_sms * 4;
        const bool timing = run->p.kernel_timing != 0;
        if (!timing) {
            TRY(cudaHostAlloc(&h_mirror, sizeof(HostMirror), cudaHostAllocMapped));
            TRY(cudaHostAlloc(&h_cancel, sizeof(int), cudaHostAllocMapped));
            std::memset(h_mirror, 0, sizeof(HostMirror));
            *h_cancel = 0;
        }

        DevRun r{};
        r.S = S;
        r.rooms = run->droom.as<RoomParams>();
        r.room_prim = run->droomprim.as<long long>();
        r.n_rooms = n_rooms;
        r.rec = run->drec.as<float4>();
        r.rec_id = run->drecid.as<int>();
        r.R = R;
        r.T = T;
        r.fs = (double)run->p.sample_rate;
        r.src = run->dsrc.as<float4>();
        r.e0 = run->de0.as<float>();
        r.geo = run->dgeo.as<float4>();
        r.prim_dirs = run->prim_dirs.empty() ? nullptr : run->ddirs.as<double>();
        r.prim_weights = run->prim_weights.empty() ? nullptr : run->dw.as<double>();
        r.prim_base = run->rooms[0].prim_begin;
        r.prop = run->prop.empty() ? nullptr : run->dprop.as<float4>();
        r.n_prop = run->prop.empty() ? 0 : run->p.n_proposal;
        r.prop_mix = (float)(run->p.proposal_mix > 0 ? run->p.proposal_mix : 0.3);
        r.capture = run->p.capture ? run->dcap.as<float>() : nullptr;
        r.capture_mode = run->p.capture;
        r.count_work = run->p.kernel_timing != 0;
        {
            const bool given = run->p.capture_edges_ms[0] != 0 || run->p.capture_edges_ms[1] != 0 ||
                               run->p.capture_edges_ms[2] != 0;
            const double def[3] = {80.0, 400.0, 1200.0};
            for (int i = 0; i < 3; ++i) r.cap_edge[i] = (float)(given ? run->p.capture_edges_ms[i] : def[i]);
        }
        if (map) {
            const MapGrid &g = run->mg;
            MapDev &m = r.map;
            m.rec = run->mrec.as<float4>();
            m.direct = run->mdir.as<double>();
            m.cell = run->mcell.as<int>();
            m.entry = run->mentry.as<uint2>();
            m.E = run->mE.as<double>();
            m.P = run->mP.as<double>();
            m.Dp = g.directional ? run->mDp.as<double>() : nullptr;
            m.Dn = g.directional ? run->mDn.as<double>() : nullptr;
            m.directional = g.directional ? 1 : 0;
            for (int a = 0; a < 3; ++a) {
                m.lo[a] = (float)g.mn[a];
                m.hi[a] = (float)g.mx[a];
                m.vd[a] = (float)g.vd[a];
                m.n[a] = g.n[a];
            }
            m.M = g.M;
            m.T = g.T;
            m.one_pt = g.one_pt ? 1 : 0;
            m.walk = g.walk;
            m.size_mod = (float)(1.0 / (M_PI * g.r2));
            const HostScene &hs0 = run->rooms[0].scene->hs;
            for (int o = 0; o < kBands; ++o) m.atten_k[o] = (float)(-0.1 * std::log2(10.0) * hs0.atten[o]);
            m.rho_c = (float)(hs0.rho * hs0.c);  // Map_Receiver: Rho_C = rho * Sound_Speed
        }
        r.seed = run->p.seed;
        r.max_seg = run->p.max_segments_per_ray > 0 ? run->p.max_segments_per_ray : (1ll << 22);
        if (!timing) {
            void *dp = nullptr;
            TRY(cudaHostGetDevicePointer(&dp, h_mirror, 0));
            r.mirror = reinterpret_cast<HostMirror *>(dp);
            TRY(cudaHostGetDevicePointer(&dp, h_cancel, 0));
            r.cancel = reinterpret_cast<volatile int *>(dp);
        }
        r.max_iters = 1ull << 26;
        r.hE = run->hE.as<double>(); r.hP = run->hP.as<double>(); r.hDp = run->hDp.as<double>();
        r.hDn = run->hDn.as<double>(); r.hAn = run->hAn.as<double>();
        r.cnt = run->cnt.as<DevCounters>();
        r.ring = run->qa.as<ORayItem>();
        r.ring_cap = ring_cap;
        r.ctl = run->qctl.as<WaveCtl>();
        r.hits = run->qs0.as<int4>();
        r.wave_buf = sorting ? run->qs1.as<ORayItem>() : nullptr;
        r.bin_count = sorting ? run->sortbins.as<unsigned>() : nullptr;
        r.bin_cursor = sorting ? run->sortbins.as<unsigned>() + kSortBins : nullptr;
        for (int k = 0; k < 3; ++k) {
            r.sort_lo[k] = (float)bmin[k];
            r.sort_inv[k] = (float)(kSortGrid / std::max(bmax[k] - bmin[k], 1e-9));
        }
        r.max_wave = std::min(max_wave, ring_cap);
        r.feed_bound = bound;
        r.low_water = std::min(ring_cap / 4, 2 * r.max_wave);
        const long long N = rprim[n_rooms] - rprim[0];
        const long long fb_default = std::max<long long>(4096, (long long)(r.max_wave / 32));
        r.feed_batch = run->p.feed_batch > 0 ? run->p.feed_batch : fb_default;
        const int bb_threads = 128;
        const int bb_blocks = (int)std::max<long long>(1, std::min<long long>((r.feed_batch + bb_threads - 1) / bb_threads,
                                                                              (long long)dev_sms * 16));
        std::memset(h_ctl, 0, sizeof(WaveCtl));
        double t_trace = 0, t_shade = 0, t_bb = 0, t_sort = 0;
        long long launches = 0;
        bool cancelled = false;
        const bool conv_mode = run->conv_mode >= 0;
        if (conv_mode) {
            // per-revolution capture of the check receivers, and a copy of the histograms and counters
            // taken before each chunk (restored when the checks agree inside a chunk)
            r.conv = nullptr;
            r.conv_row[0] = run->conv_rows[0];
            r.conv_row[1] = run->conv_rows[1];
            r.conv_oct = run->rooms[0].h_oct;
            r.conv_period = run->conv_period;
            TRY(run->conv.alloc((size_t)kConvChunk * 2 * kConvKinds * T * sizeof(double)));
            r.conv = run->conv.as<double>();
            DevMem *src_[6] = {&run->hE, &run->hP, &run->hDp, &run->hDn, &run->hAn, &run->cnt};
            for (int i = 0; i < 6; ++i) TRY(run->bak[i].alloc(src_[i]->bytes));
            if (e) break;
        }
        auto one_iteration = [&](int k) -> cudaError_t {
            cudaError_t x;
            if ((x = launch_feed(r, stream))) return x;
            if (timing && (x = cudaEventRecord(kev[6 * k], stream))) return x;
            if ((x = launch_broadband(r, bb_blocks, bb_threads, stream, map, ntri_max <= kFuseMaxTris))) return x;
            if (timing && (x = cudaEventRecord(kev[6 * k + 1], stream))) return x;
            if ((x = launch_wave(r, stream))) return x;
            if (timing && (x = cudaEventRecord(kev[6 * k + 2], stream))) return x;
            if (sorting && (x = launch_sort(r, sort_blocks, stream))) return x;
            if (timing && (x = cudaEventRecord(kev[6 * k + 3], stream))) return x;
            if (!fused && (x = launch_trace(r, tr_variant, tr_blocks, threads, stream))) return x;
            if (timing && (x = cudaEventRecord(kev[6 * k + 4], stream))) return x;
            if ((x = launch_shade(r, sh_blocks, threads, stream, fused, map, wide))) return x;
            if (timing && (x = cudaEventRecord(kev[6 * k + 5], stream))) return x;
            return cudaSuccess;
        };
        if (!timing) {
            // the whole loop as one graph launch: while (k_cond says so) { one iteration }
            TRY(cudaGraphCreate(&graph, 0));
            cudaGraphConditionalHandle handle;
            TRY(cudaGraphConditionalHandleCreate(&handle, graph, 1, cudaGraphCondAssignDefault));
            cudaGraphNodeParams cp{};
            cp.type = cudaGraphNodeTypeConditional;
            cp.conditional.handle = handle;
            cp.conditional.type = cudaGraphCondTypeWhile;
            cp.conditional.size = 1;
            cudaGraphNode_t node;
            TRY(cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &cp));
            cudaGraph_t body = cp.conditional.phGraph_out[0];
            TRY(cudaStreamBeginCaptureToGraph(stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
            cudaError_t ce = one_iteration(0);
            if (ce == cudaSuccess) ce = launch_cond(r, handle, stream);
            cudaGraph_t captured = nullptr;
            cudaError_t ee = cudaStreamEndCapture(stream, &captured);
            TRY(ce);
            TRY(ee);
            TRY(cudaGraphInstantiate(&gexec, graph, 0));
        }
        double dev_ms_total = 0;
        long long done_before = 0;  // primaries of the ranges already run (progress offset)
        // Runs the device loop over primaries [p0, p1): the graph launch (progress and cancellation through
        // mapped host memory) or, with kernel_timing, host-launched batches of iterations with CUDA events
        // around every kernel.  Returns a CUDA error, or cudaSuccess with `status` set when it gave up.
#define RTRY(x)                                   \
    {                                             \
        const cudaError_t x_ = (x);               \
        if (x_ != cudaSuccess) { where = #x; return x_; } \
    }
        auto run_range = [&](long long p0, long long p1) -> cudaError_t {
            // the schedule starts afresh; the pilots' per-primary ring footprint carries over
            const unsigned long long per_prim = h_ctl->per_prim;
            const int pilot_room = h_ctl->pilot_room;
            std::memset(h_ctl, 0, sizeof(WaveCtl));
            h_ctl->next_prim = p0;
            h_ctl->prim_end = p1;
            h_ctl->prim_first = p0;
            h_ctl->per_prim = per_prim;
            h_ctl->pilot_room = pilot_room;
            RTRY(cudaMemcpyAsync(run->qctl.p, h_ctl, sizeof(WaveCtl), cudaMemcpyHostToDevice, stream));
            if (!timing) {
                *reinterpret_cast<volatile int *>(h_cancel) = 0;
                std::memset(h_mirror, 0, sizeof(HostMirror));
                h_mirror->next_prim = p0;
                // device time of the loop alone: the host's graph construction is not inside the events
                RTRY(cudaEventRecord(ev0, stream));
                RTRY(cudaGraphLaunch(gexec, stream));
                RTRY(cudaEventRecord(ev1, stream));
                launches += 6;
                // poll: progress from the mapped mirror, cancellation through the mapped flag (1: stop
                // feeding; 2, two seconds later: stop the loop without waiting for the fed primaries)
                auto t_cancel = std::chrono::steady_clock::now();
                for (;;) {
                    const cudaError_t q = cudaEventQuery(ev1);
                    run->rays_done = done_before + std::max(0ll, (long long)h_mirror->next_prim - p0);
                    run->end_traces = (long long)h_mirror->end_traces;
                    run->segments = (long long)h_mirror->segments;
                    if (q == cudaSuccess) break;
                    if (q != cudaErrorNotReady) { where = "graph run"; return q; }
                    if (run->cancel && !cancelled) {
                        cancelled = true;
                        t_cancel = std::chrono::steady_clock::now();
                        *reinterpret_cast<volatile int *>(h_cancel) = 1;
                    } else if (cancelled && std::chrono::steady_clock::now() - t_cancel > std::chrono::seconds(2)) {
                        *reinterpret_cast<volatile int *>(h_cancel) = 2;
                    }
                    std::this_thread::sleep_for(std::chrono::microseconds(500));
                }
            } else {
                RTRY(cudaEventRecord(ev0, stream));
                int batch = 8;
                for (long long it = 0;;) {
                    // one batch of iterations, no host synchronisation inside
                    while (kev.size() < (size_t)batch * 6) {
                        cudaEvent_t x;
                        RTRY(cudaEventCreate(&x));
                        kev.push_back(x);
                    }
                    for (int k = 0; k < batch; ++k, ++it) {
                        RTRY(one_iteration(k));
                        launches += (sorting ? 8 : 5) - (fused ? 1 : 0);
                    }
                    RTRY(cudaMemcpyAsync(h_ctl, run->qctl.p, sizeof(WaveCtl), cudaMemcpyDeviceToHost, stream));
                    RTRY(cudaMemcpyAsync(h_cnt, run->cnt.p, sizeof(DevCounters), cudaMemcpyDeviceToHost, stream));
                    RTRY(cudaStreamSynchronize(stream));
                    for (int k = 0; k < batch; ++k) {
                        float a = 0, b = 0, c = 0, so = 0;
                        RTRY(cudaEventElapsedTime(&a, kev[6 * k], kev[6 * k + 1]));
                        RTRY(cudaEventElapsedTime(&so, kev[6 * k + 2], kev[6 * k + 3]));
                        RTRY(cudaEventElapsedTime(&b, kev[6 * k + 3], kev[6 * k + 4]));
                        RTRY(cudaEventElapsedTime(&c, kev[6 * k + 4], kev[6 * k + 5]));
                        t_bb += a;
                        t_sort += so;
                        t_trace += b;
                        t_shade += c;
                    }
                    // progress: primaries whose phase A has run
                    run->rays_done = done_before + h_ctl->next_prim - p0;
                    run->end_traces = (long long)h_cnt->end_traces;
                    run->segments = (long long)(h_cnt->seg_broad + h_cnt->seg_b + h_cnt->seg_c);
                    if (h_ctl->done) break;
                    if (run->cancel && !cancelled) {
                        // stop feeding; the primaries already fed run to completion, so the histograms stay
                        // a consistent estimate over rays_done primaries
                        cancelled = true;
                        const long long stop = h_ctl->next_prim;
                        RTRY(cudaMemcpyAsync(&run->qctl.as<WaveCtl>()->prim_end, &stop, sizeof(long long),
                                             cudaMemcpyHostToDevice, stream));
                        RTRY(cudaStreamSynchronize(stream));
                    }
                    if (batch < 64) batch *= 2;
                    if (it > (1ll << 26)) {
                        status = PACH_ERR_GAVE_UP;
                        msg = "wavefront loop did not finish";
                        final_state = PACH_RUN_FAILED;
                        return cudaSuccess;
                    }
                }
                RTRY(cudaEventRecord(ev1, stream));
            }
            RTRY(cudaStreamSynchronize(stream));
            float ms = 0.f;
            RTRY(cudaEventElapsedTime(&ms, ev0, ev1));
            dev_ms_total += ms;
            RTRY(cudaMemcpy(h_ctl, run->qctl.p, sizeof(WaveCtl), cudaMemcpyDeviceToHost));
            return cudaSuccess;
        };
#undef RTRY
        if (!conv_mode) {
            if ((e = run_range(rprim[0], rprim[0] + N)) != cudaSuccess || status) break;
        } else {
            // Convergence mode (TaskAll:300-330): revolutions of conv_period primaries until every check
            // agrees.  Chunks of revolutions run as one device loop that also records each revolution's
            // contribution to the two check receivers; the host replays the checks revolution by
            // revolution.  When they agree inside a chunk, the histograms and counters are restored to
            // their state before the chunk and the chunk's primaries up to that revolution are traced
            // again -- the same Philox streams, so the result is the run that stopped there.
            const long long period = run->conv_period;
            const long long cap = run->p.max_rays > 0 ? run->p.max_rays : (1ll << 24);
            std::vector<ConvCheck> &checks = run->conv_checks;
            std::vector<double> capbuf((size_t)kConvChunk * 2 * kConvKinds * T);
            DevMem *live[6] = {&run->hE, &run->hP, &run->hDp, &run->hDn, &run->hAn, &run->cnt};
            long long done = 0, revs = 0;
            int chunk = 4;
            bool converged = false;
            while (!converged && done < cap && !run->cancel) {
                const long long left = (cap - done + period - 1) / period;
                const int K = (int)std::min<long long>(chunk, left);
                for (int i = 0; i < 6; ++i)
                    TRY(cudaMemcpyAsync(run->bak[i].p, live[i]->p, live[i]->bytes, cudaMemcpyDeviceToDevice, stream));
                TRY(cudaMemsetAsync(run->conv.p, 0, (size_t)K * 2 * kConvKinds * T * sizeof(double), stream));
                if (e) break;
                done_before = done;
                if ((e = run_range(rprim[0] + done, rprim[0] + done + K * period)) != cudaSuccess || status) break;
                TRY(cudaMemcpy(capbuf.data(), run->conv.p, (size_t)K * 2 * kConvKinds * T * sizeof(double),
                               cudaMemcpyDeviceToHost));
                int stop = -1;
                for (int j = 0; j < K && stop < 0; ++j) {
                    bool agree = true;
                    for (int k = 0; k < 2; ++k) {
                        ConvCheck &c = checks[(size_t)k];
                        if (c.mode < 0) continue;
                        const double *h = capbuf.data() + ((size_t)j * 2 + k) * kConvKinds * T;
                        for (int b = 0; b < T; ++b) {
                            c.E[(size_t)b] += h[b];
                            c.A0[(size_t)b] += h[T + b];
                            c.A1[(size_t)b] += h[2 * T + b];
                            c.A2[(size_t)b] += h[3 * T + b];
                        }
                        agree = c.check() && agree;  // every check runs each revolution (C# &=)
                    }
                    if (agree) stop = j;
                }
                if (stop >= 0 && stop < K - 1) {
                    for (int i = 0; i < 6; ++i)
                        TRY(cudaMemcpyAsync(live[i]->p, run->bak[i].p, live[i]->bytes, cudaMemcpyDeviceToDevice, stream));
                    if (e) break;
                    if ((e = run_range(rprim[0] + done, rprim[0] + done + (stop + 1) * period)) != cudaSuccess || status)
                        break;
                }
                done += (stop >= 0 ? stop + 1 : K) * period;
                revs = done / period;
                converged = stop >= 0;
                chunk = std::min(chunk * 2, kConvChunk);
            }
            if (e || status) break;
            run->rooms[0].rays = done;
            run->conv_revs = revs;
            run->conv_converged = converged;
            if (run->cancel) cancelled = true;
        }
        const float dev_ms = (float)dev_ms_total;
        TRY(cudaMemcpy(h_cnt, run->cnt.p, sizeof(DevCounters), cudaMemcpyDeviceToHost));
        TRY(cudaMemcpy(h_ctl, run->qctl.p, sizeof(WaveCtl), cudaMemcpyDeviceToHost));
        const HostScene &hs = sc->hs;
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
        s.queue_overflows = (int64_t)h_ctl->overflow;
        s.stack_spills = 0;
        s.lost_energy = h_cnt->lost_energy;
        s.initial_energy = h_cnt->initial_energy;
        s.percent_lost = s.initial_energy > 0 ? 100.0 * s.lost_energy / s.initial_energy : 0.0;
        s.h_oct = run->rooms[0].h_oct;
        s.bins = T;
        s.cotime_s = run->rooms[0].cotime;
        s.sound_speed = hs.c;
        s.rho_c = hs.rho_c;
        for (int o = 0; o < kBands; ++o) s.air_atten_db_per_m[o] = hs.atten[o];
        s.device_ms = dev_ms;
        s.trace_ms = t_trace;
        s.shade_ms = t_shade;
        s.broadband_ms = t_bb;
        s.sort_ms = t_sort;
        s.waves = (int64_t)h_ctl->waves;
        s.kernel_launches = timing ? launches : (long long)h_ctl->iters * ((sorting ? 9 : 6) - (fused ? 1 : 0));
        s.peak_live_rays = (int64_t)h_ctl->peak_live;
        s.bvh_nodes_visited = (int64_t)h_cnt->bvh_nodes;
        s.tri_tests = (int64_t)h_cnt->tri_tests;
        s.accel[0] = (int32_t)(n_rooms > 1 ? run->bbvh.bytes / (kBvhNodeFloats * sizeof(float)) : hs.bvh_nodes);
        s.accel[1] = hs.bvh_leaves;
        s.accel[2] = hs.bvh_depth;
        s.walk = (quant ? 4 * kBvhQNodeFloats : 4 * kBvhNodeFloats) + 1000 * (fused ? 3 : ((tr_variant & 16) ? 2 : 1));
        s.revolutions = conv_mode ? run->conv_revs : 0;
        s.converged = conv_mode && run->conv_converged ? 1 : 0;
        s.check_receivers[0] = conv_mode ? run->conv_rows[0] : -1;
        s.check_receivers[1] = conv_mode ? run->conv_rows[1] : -1;
        run->rays_done = (long long)h_cnt->primaries;
        run->segments = s.segments;
        run->end_traces = s.end_traces;
        if (h_ctl->overflow) {
            status = PACH_ERR_BOUNDS;
            msg = "ring queue full: raise ring_log2";
            final_state = PACH_RUN_FAILED;
        } else if (h_ctl->gave_up == 2) {
            status = PACH_ERR_CANCELLED;
            msg = "run cancelled; the loop stopped before every fed primary finished";
            final_state = PACH_RUN_CANCELLED;
        } else if (h_ctl->gave_up) {
            status = PACH_ERR_GAVE_UP;
            msg = "wavefront loop stopped without finishing (iteration cap or no progress)";
            final_state = PACH_RUN_FAILED;
        } else if (cancelled) {
            status = PACH_ERR_CANCELLED;
            msg = "run cancelled after " + std::to_string(s.primaries) + " primaries";
            final_state = PACH_RUN_CANCELLED;
        }
#undef TRY
    } while (0);
    run->stats.wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - wall0).count();
    if (gexec) cudaGraphExecDestroy(gexec);
    if (graph) cudaGraphDestroy(graph);
    for (cudaEvent_t ev : kev) cudaEventDestroy(ev);
    for (cudaEvent_t ev : {ev0, ev1})
        if (ev) cudaEventDestroy(ev);
    if (h_ctl) cudaFreeHost(h_ctl);
    if (h_cnt) cudaFreeHost(h_cnt);
    if (stream) cudaStreamDestroy(stream);
    if (h_mirror) cudaFreeHost(h_mirror);
    if (h_cancel) cudaFreeHost(h_cancel);
    // release the ring and the batch scene; histograms and counters stay until the run is destroyed
    for (DevMem *m : {&run->qa, &run->qs0, &run->qs1, &run->ddirs, &run->dw, &run->sortbins, &run->btri, &run->btri64,
                      &run->bnorm, &run->bmat, &run->btrans, &run->bbvh, &run->bbvhq, &run->conv, &run->bak[0],
                      &run->bak[1], &run->bak[2], &run->bak[3], &run->bak[4], &run->bak[5]})
        m->release();
    if (e != cudaSuccess) return finish(PACH_ERR_CUDA, cuda_msg(e, where.c_str()), PACH_RUN_FAILED);
    finish(status, msg, final_state);
}

pach_status check_run(pach_run *run) {
    if (!run) return fail(PACH_ERR_INVALID_ARGUMENT, "null run handle");
    return PACH_OK;
}

}  // namespace

// Checks shared by pach_trace_begin, pach_batch_begin and pach_trace_run_noalloc: the run-wide
// parameters and one room's sources and receivers (the message goes to pach_last_error).
pach_status pach::check_common(const pach_trace_params &p) {
    if (p.oct_lo < 0 || p.oct_hi > 7 || p.oct_lo > p.oct_hi) return fail(PACH_ERR_INVALID_ARGUMENT, "octave range must lie in 0..7");
    if (p.sample_rate < 1) return fail(PACH_ERR_INVALID_ARGUMENT, "sample_rate must be positive");
    if (p.traversal < 0 || p.traversal > 3) return fail(PACH_ERR_INVALID_ARGUMENT, "traversal must be 0..3");
    const long long T = (long long)((double)p.sample_rate * (p.hist_cotime_ms / 1000.0));
    if (T < 1 || T > (1ll << 24)) return fail(PACH_ERR_INVALID_ARGUMENT, "histogram length must be 1..2^24 bins");
    return PACH_OK;
}

pach_status pach::check_room(const pach_source_desc *sources, int32_t n_sources, const pach_receiver_desc *receivers,
                       int32_t n_receivers, const std::string &who) {
    if (!sources || n_sources < 1 || n_sources > kMaxSources)
        return fail(PACH_ERR_INVALID_ARGUMENT, who + "need 1.." + std::to_string(kMaxSources) + " sources");
    if (n_receivers < 0 || (n_receivers > 0 && !receivers)) return fail(PACH_ERR_INVALID_ARGUMENT, who + "bad receivers");
    for (int i = 0; i < n_receivers; ++i)
        if (!(receivers[i].radius > 0) || !std::isfinite(receivers[i].origin[0]) || !std::isfinite(receivers[i].origin[1]) ||
            !std::isfinite(receivers[i].origin[2]))
            return fail(PACH_ERR_INVALID_ARGUMENT,
                        who + "receiver " + std::to_string(i) + ": radius must be positive, origin finite");
    for (int s = 0; s < n_sources; ++s)
        if (sources[s].kind < 0 || sources[s].kind > 2) return fail(PACH_ERR_INVALID_ARGUMENT, who + "unknown source kind");
    return PACH_OK;
}


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
    return guarded([&]() -> pach_status {
        if (!atten) return fail(PACH_ERR_INVALID_ARGUMENT, "atten is null");
        if (!(pa_hpa > 0) || !(hr > 0) || air_choice < 0 || air_choice > 2)
            return fail(PACH_ERR_INVALID_ARGUMENT, "medium: pressure and humidity must be positive, air_choice 0..2");
        medium_properties(temp_c, hr, pa_hpa, air_choice, edge, atten, c, rho);
        return PACH_OK;
    }, fail);
}

pach_status pach_medium_attenuation_third_octave(double temp_c, double hr, double pa_hpa, int32_t air_choice,
                                                 int32_t edge, double *atten, double *centres_hz) {
    return guarded([&]() -> pach_status {
        if (!atten) return fail(PACH_ERR_INVALID_ARGUMENT, "atten is null");
        if (!(pa_hpa > 0) || !(hr > 0) || air_choice < 0 || air_choice > 2)
            return fail(PACH_ERR_INVALID_ARGUMENT, "medium: pressure and humidity must be positive, air_choice 0..2");
        medium_attenuation_third_octave(temp_c, hr, pa_hpa, air_choice, edge, atten);
        if (centres_hz) for (int i = 0; i < kThirdOctaveBands; ++i) centres_hz[i] = kThirdOctaveCentres[i];
        return PACH_OK;
    }, fail);
}

pach_status pach_scene_create(const pach_scene_desc *desc, pach_scene **out) {
    return guarded([&]() -> pach_status {
        if (!out) return fail(PACH_ERR_INVALID_ARGUMENT, "out is null");
        *out = nullptr;
        if (!desc) return fail(PACH_ERR_INVALID_ARGUMENT, "desc is null");
        if (!(desc->pressure_hpa > 0) || !(desc->rel_humidity > 0) || desc->air_choice < 0 || desc->air_choice > 2)
            return fail(PACH_ERR_INVALID_ARGUMENT, "scene: pressure and humidity must be positive, air_choice 0..2");
        std::unique_ptr<pach_scene> sc(new pach_scene());
        std::string err;
        if (!build_host_scene(desc, sc->hs, err)) return fail(PACH_ERR_INVALID_ARGUMENT, err);
        if (pach_device_count() <= 0)
            return fail(PACH_ERR_NO_DEVICE, "no CUDA device visible: the GB300 engine has no CPU fallback");
        cudaGetDevice(&sc->device);
        const cudaError_t e = scene_upload(sc.get());
        if (e != cudaSuccess)
            return fail(e == cudaErrorMemoryAllocation ? PACH_ERR_OUT_OF_MEMORY : PACH_ERR_CUDA, cuda_msg(e, "scene upload"));
        *out = sc.release();
        return PACH_OK;
    }, fail);
}

pach_status pach_scenes_create(const pach_scene_desc *descs, int32_t n, pach_scene **out, int32_t threads) {
    return guarded([&]() -> pach_status {
        if (!out || (n > 0 && !descs) || n < 0) return fail(PACH_ERR_INVALID_ARGUMENT, "scenes: bad arguments");
        for (int i = 0; i < n; ++i) out[i] = nullptr;
        for (int i = 0; i < n; ++i)
            if (!(descs[i].pressure_hpa > 0) || !(descs[i].rel_humidity > 0) || descs[i].air_choice < 0 ||
                descs[i].air_choice > 2)
                return fail(PACH_ERR_INVALID_ARGUMENT, "scene " + std::to_string(i) +
                                                           ": pressure and humidity must be positive, air_choice 0..2");
        if (pach_device_count() <= 0) return fail(PACH_ERR_NO_DEVICE, "no CUDA device visible: the GB300 engine has no CPU fallback");
        int device = 0;
        cudaGetDevice(&device);
        // host builds (BVH, quantised nodes, materials) on worker threads, largest scenes first
        std::vector<std::unique_ptr<pach_scene>> sc((size_t)n);
        std::vector<std::string> errs((size_t)n);
        std::vector<int> order((size_t)n);
        for (int i = 0; i < n; ++i) order[(size_t)i] = i;
        std::sort(order.begin(), order.end(), [&](int a, int b) { return descs[a].n_polys > descs[b].n_polys; });
        std::atomic<int> next{0};
        const int nt = std::max(1, std::min(n, threads > 0 ? threads : (int)std::max(1u, std::thread::hardware_concurrency())));
        std::vector<char> oom((size_t)n, 0);
        auto work = [&] {
            for (int j; (j = next.fetch_add(1)) < n;) {
                const int i = order[(size_t)j];
                try {  // nothing may leave a worker thread
                    sc[(size_t)i].reset(new pach_scene());
                    if (!build_host_scene(&descs[i], sc[(size_t)i]->hs, errs[(size_t)i])) sc[(size_t)i].reset();
                } catch (const std::exception &ex) {
                    sc[(size_t)i].reset();
                    oom[(size_t)i] = 1;
                    errs[(size_t)i] = std::string("host resources exhausted: ") + ex.what();
                }
            }
        };
        std::vector<std::thread> pool;
        for (int t = 1; t < nt; ++t) {
            try {
                pool.emplace_back(work);
            } catch (const std::exception &) {
                break;  // fewer threads: the calling thread takes the rest
            }
        }
        work();
        for (std::thread &t : pool) t.join();
        for (int i = 0; i < n; ++i)
            if (!sc[(size_t)i])
                return fail(oom[(size_t)i] ? PACH_ERR_OUT_OF_MEMORY : PACH_ERR_INVALID_ARGUMENT,
                            "scene " + std::to_string(i) + ": " + errs[(size_t)i]);
        // the scenes belong to the caller's device; each one's device copy is made on its first
        // single-room use (a batch run uploads the concatenation of its rooms, so a batch's scenes are
        // uploaded once, not twice)
        for (int i = 0; i < n; ++i) sc[(size_t)i]->device = device;
        for (int i = 0; i < n; ++i) out[i] = sc[(size_t)i].release();
        return PACH_OK;
    }, fail);
}

void pach_scene_destroy(pach_scene *scene) { delete scene; }

pach_status pach_scene_info(const pach_scene *scene, int32_t *n_polys, int32_t *n_triangles, double *sound_speed,
                            double *rho_c, double atten[PACH_BANDS], double *poly_area) {
    return guarded([&]() -> pach_status {
        if (!scene) return fail(PACH_ERR_INVALID_ARGUMENT, "null scene");
        const HostScene &hs = scene->hs;
        if (n_polys) *n_polys = hs.npoly;
        if (n_triangles) *n_triangles = hs.ntri;
        if (sound_speed) *sound_speed = hs.c;
        if (rho_c) *rho_c = hs.rho_c;
        if (atten) for (int o = 0; o < kBands; ++o) atten[o] = hs.atten[o];
        if (poly_area) for (int p = 0; p < hs.npoly; ++p) poly_area[p] = hs.area[p];
        return PACH_OK;
    }, fail);
}

pach_status pach_trace_begin(pach_scene *scene, const pach_source_desc *sources, int32_t n_sources,
                             const pach_receiver_desc *receivers, int32_t n_receivers, const pach_trace_params *params,
                             pach_run **out) {
    return guarded([&]() -> pach_status {
        if (!out) return fail(PACH_ERR_INVALID_ARGUMENT, "out is null");
        *out = nullptr;
        if (!scene || !params) return fail(PACH_ERR_INVALID_ARGUMENT, "null scene or params");
        if (pach_status st = check_room(sources, n_sources, receivers, n_receivers, "")) return st;
        if (n_receivers > 2048) return fail(PACH_ERR_INVALID_ARGUMENT, "at most 2048 receivers per run");
        const pach_trace_params &p = *params;
        const bool conv = p.ray_count < 1;  // convergence mode (SplitRayTracer rayCount < 1)
        const long long conv_cap = p.max_rays > 0 ? p.max_rays : (1ll << 24);
        if (p.ray_begin < 0 || (!conv && p.ray_begin + p.ray_count > (1ll << 32)))
            return fail(PACH_ERR_INVALID_ARGUMENT, "ray_begin must be >= 0 and ray_begin + ray_count <= 2^32");
        if (conv) {
            if (p.prim_dirs || p.prim_weights || p.proposal || p.capture || p.map)
                return fail(PACH_ERR_INVALID_ARGUMENT,
                            "convergence mode (ray_count < 1) takes no emission overrides, proposal, capture or map");
            if (p.max_rays < 0 || p.ray_begin + conv_cap + 80ll * kConvChunk * n_sources > (1ll << 32))
                return fail(PACH_ERR_INVALID_ARGUMENT, "max_rays must be >= 0 and ray_begin + max_rays < 2^32");
        }
        if (pach_status st = check_common(p)) return st;
        if (!(p.cutoff_length_m > 0)) return fail(PACH_ERR_INVALID_ARGUMENT, "cutoff_length_m must be positive");
        if (p.proposal) {
            if (p.n_proposal < 1 || p.n_proposal > 256)
                return fail(PACH_ERR_INVALID_ARGUMENT, "n_proposal must be 1..256 when proposal is given");
            if (p.prim_dirs) return fail(PACH_ERR_INVALID_ARGUMENT, "proposal and prim_dirs exclude each other");
            if (p.capture) return fail(PACH_ERR_INVALID_ARGUMENT, "capture records uniform-emission runs only");
            if (!(p.proposal_mix >= 0 && p.proposal_mix <= 1))
                return fail(PACH_ERR_INVALID_ARGUMENT, "proposal_mix must lie in [0, 1] (0 = default)");
            for (long long i = 0; i < (long long)p.n_proposal * PACH_MLP_OUT; ++i)
                if (!std::isfinite(p.proposal[i])) return fail(PACH_ERR_INVALID_ARGUMENT, "proposal holds a non-finite value");
        }
        if (p.capture && (p.capture < 0 || p.capture > 2 || n_receivers < 1))
            return fail(PACH_ERR_INVALID_ARGUMENT, "capture must be 0, 1 or 2 and needs receivers");
        if (p.capture == 2 && (double)p.ray_count * n_receivers * kCaptureWindows * 4 > 16e9)
            return fail(PACH_ERR_INVALID_ARGUMENT, "per-primary capture larger than 16 GB");
        std::unique_ptr<pach_run> run(new pach_run());
        run->scene = scene;
        run->p = p;
        if (p.map) {
            std::string err;
            if (!build_map_grid(*p.map, sources[0].origin, n_sources, scene->hs.c, run->mg, err))
                return fail(PACH_ERR_INVALID_ARGUMENT, err);
            if ((double)run->mg.M * kBands * run->mg.T * 16 > 200e9)
                return fail(PACH_ERR_INVALID_ARGUMENT, "map histograms larger than 200 GB");
            run->map_org.assign(p.map->origins, p.map->origins + 3 * (size_t)p.map->n_receivers);
            run->has_map = true;
        }
        run->p.map = nullptr;
        if (p.proposal) proposal_lobes(p.proposal, p.n_proposal, run->prop);
        if (p.prim_dirs) run->prim_dirs.assign(p.prim_dirs, p.prim_dirs + 3 * p.ray_count);
        if (p.prim_weights) run->prim_weights.assign(p.prim_weights, p.prim_weights + p.ray_count);
        run->p.proposal = nullptr;
        run->p.prim_dirs = nullptr;
        run->p.prim_weights = nullptr;
        RoomSpec rm;
        rm.scene = scene;
        rm.src.assign(sources, sources + n_sources);
        rm.rec.assign(receivers, receivers + n_receivers);
        rm.rays = p.ray_count;
        rm.prim_begin = p.ray_begin;
        rm.cutoff_len = p.cutoff_length_m;  // TaskAll:83 -- the ctor's cutoff argument is a length
        std::string err;
        if (!room_setup(rm, p, err)) return fail(PACH_ERR_INVALID_ARGUMENT, err);
        run->R = n_receivers;
        run->nsrc = n_sources;
        run->T = (int)((double)p.sample_rate * (p.hist_cotime_ms / 1000.0));
        if (conv) {
            // Revolution_Period: 80 primaries per point source, the members' sum for a cluster
            // (Classes_Sources.cs:197-200, 687); the checks' receivers as the ctor picks them, seen from
            // the source's Origin (a cluster's: the mean of its members' origins, Classes_Sources.cs:684-689)
            run->conv_mode = p.ray_count == 0 ? 0 : 1;
            run->conv_period = 80ll * n_sources;
            rm.rays = (long long)kConvChunk * run->conv_period;  // ring sizing: one chunk of revolutions
            double ctr[3] = {0, 0, 0}, dist[2];
            for (int s = 0; s < n_sources; ++s)
                for (int a = 0; a < 3; ++a) ctr[a] += sources[s].origin[a] / n_sources;
            pick_conv_receivers(scene->hs, ctr, receivers, n_receivers, run->conv_rows, dist);
            run->conv_checks.resize(2);
            for (int k = 0; k < 2; ++k)
                if (run->conv_rows[k] >= 0)
                    conv_setup(run->conv_checks[(size_t)k], run->conv_mode == 0 ? 0 : 1, run->conv_rows[k], dist[k],
                               scene->hs.c, p.sample_rate, run->T);
        }
        run->rooms.push_back(std::move(rm));
        run->worker = std::thread(run_worker, run.get());
        *out = run.release();
        return PACH_OK;
    }, fail);
}

pach_status pach_batch_begin(const pach_room_desc *rooms, int32_t n_rooms, const pach_trace_params *params,
                             pach_run **out) {
    return guarded([&]() -> pach_status {
        if (!out) return fail(PACH_ERR_INVALID_ARGUMENT, "out is null");
        *out = nullptr;
        if (!rooms || !params || n_rooms < 1 || n_rooms > kMaxRooms)
            return fail(PACH_ERR_INVALID_ARGUMENT, "need 1.." + std::to_string(kMaxRooms) + " rooms and params");
        const pach_trace_params &p = *params;
        if (pach_status st = check_common(p)) return st;
        if (p.proposal || p.prim_dirs || p.prim_weights)
            return fail(PACH_ERR_INVALID_ARGUMENT, "a batch emits from its sources: no proposal or emission overrides");
        if (p.map) return fail(PACH_ERR_INVALID_ARGUMENT, "mapping receivers need a single-room run (pach_trace_begin)");
        if (p.ray_begin < 0) return fail(PACH_ERR_INVALID_ARGUMENT, "ray_begin must be >= 0");
        std::unique_ptr<pach_run> run(new pach_run());
        run->p = p;
        run->p.map = nullptr;
        long long prim = p.ray_begin;
        int R = 0, nsrc = 0;
        for (int i = 0; i < n_rooms; ++i) {
            const pach_room_desc &d = rooms[i];
            const std::string who = "room " + std::to_string(i) + ": ";
            if (!d.scene) return fail(PACH_ERR_INVALID_ARGUMENT, who + "null scene");
            if (d.scene->device != rooms[0].scene->device) return fail(PACH_ERR_INVALID_ARGUMENT, who + "scenes on different devices");
            if (pach_status st = check_room(d.sources, d.n_sources, d.receivers, d.n_receivers, who)) return st;
            if (d.ray_count < 1) return fail(PACH_ERR_INVALID_ARGUMENT, who + "ray_count must be >= 1");
            if (!(d.cutoff_length_m > 0)) return fail(PACH_ERR_INVALID_ARGUMENT, who + "cutoff_length_m must be positive");
            RoomSpec rm;
            rm.scene = const_cast<pach_scene *>(d.scene);
            rm.src.assign(d.sources, d.sources + d.n_sources);
            rm.rec.assign(d.receivers, d.receivers + d.n_receivers);
            rm.rays = d.ray_count;
            rm.prim_begin = prim;
            rm.cutoff_len = d.cutoff_length_m;
            std::string err;
            if (!room_setup(rm, p, err)) return fail(PACH_ERR_INVALID_ARGUMENT, who + err);
            prim += d.ray_count;
            R += d.n_receivers;
            nsrc += d.n_sources;
            run->rooms.push_back(std::move(rm));
        }
        if (prim > (1ll << 32)) return fail(PACH_ERR_INVALID_ARGUMENT, "ray_begin + the rooms' rays must be <= 2^32");
        if (R > 2048) return fail(PACH_ERR_INVALID_ARGUMENT, "at most 2048 receivers over the rooms of a batch");
        if (p.capture && (p.capture != 1 || R < 1))
            return fail(PACH_ERR_INVALID_ARGUMENT, "a batch captures per direction bin only (capture 1) and needs receivers");
        run->scene = run->rooms[0].scene;
        run->p.ray_count = prim - p.ray_begin;
        run->p.cutoff_length_m = run->rooms[0].cutoff_len;
        run->R = R;
        run->nsrc = nsrc;
        run->T = (int)((double)p.sample_rate * (p.hist_cotime_ms / 1000.0));
        run->worker = std::thread(run_worker, run.get());
        *out = run.release();
        return PACH_OK;
    }, fail);
}

pach_status pach_trace_poll(pach_run *run, pach_progress *pr) {
    return guarded([&]() -> pach_status {
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
    }, fail);
}

pach_status pach_trace_cancel(pach_run *run) {
    return guarded([&]() -> pach_status {
        if (pach_status s = check_run(run)) return s;
        run->cancel = true;
        return PACH_OK;
    }, fail);
}

pach_status pach_trace_wait(pach_run *run, int64_t timeout_ms) {
    return guarded([&]() -> pach_status {
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
    }, fail);
}

pach_status pach_trace_get_histograms(pach_run *run, int32_t scaled, double *energy, double *pressure, double *dir_pos,
                                      double *dir_neg, double *analysis, size_t cap_bins) {
    return guarded([&]() -> pach_status {
        if (pach_status s = check_run(run)) return s;
        {
            std::lock_guard<std::mutex> lk(run->mu);
            if (!run->finished) return fail(PACH_ERR_NOT_READY, "run still in progress");
            if (run->status != PACH_OK && run->status != PACH_ERR_CANCELLED) return fail(run->status, run->err);
        }
        const size_t nE = (size_t)run->R * kBands * run->T, nD = nE * 3;
        if (cap_bins < nE) return fail(PACH_ERR_INVALID_ARGUMENT, "cap_bins < receivers * 8 * bins");
        cudaSetDevice(run->scene->device);
        struct Item { double *dst; DevMem *src; size_t n; int lanes; bool pressure; };
        const Item items[5] = {{energy, &run->hE, nE, 1, false}, {pressure, &run->hP, nE, 1, true},
                               {dir_pos, &run->hDp, nD, 3, false}, {dir_neg, &run->hDn, nD, 3, false},
                               {analysis, &run->hAn, nD, 3, false}};
        const long long done = run->rays_done.load();
        for (const Item &it : items) {
            if (!it.dst || it.n == 0) continue;
            cudaError_t e = cudaMemcpy(it.dst, it.src->p, it.n * sizeof(double), cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) return fail(PACH_ERR_CUDA, cuda_msg(e, "histogram copy"));
            if (!scaled) continue;
            // Receiver_Bank.Scale(N) then, for a cluster, Scale(1/n_sources) (TaskAll:770-771), with N the
            // primaries the receiver's room completed (rooms are fed in order)
            const size_t per_rec = (size_t)it.lanes * kBands * run->T;
            double *dst = it.dst;
            for (const RoomSpec &rm : run->rooms) {
                const long long off = rm.prim_begin - run->rooms[0].prim_begin;
                const double N = (double)std::max(1ll, std::min(rm.rays, done - off));
                const double ns = (double)rm.src.size();
                const double f = it.pressure ? std::sqrt(ns) / std::sqrt(N) : ns / N;
                for (size_t i = 0; i < rm.rec.size() * per_rec; ++i) dst[i] *= f;
                dst += rm.rec.size() * per_rec;
            }
        }
        return PACH_OK;
    }, fail);
}

pach_status pach_trace_get_filters(pach_run *run, int32_t directional, const double *swl, double *out, size_t cap) {
    return guarded([&]() -> pach_status {
        if (pach_status s = check_run(run)) return s;
        {
            std::lock_guard<std::mutex> lk(run->mu);
            if (!run->finished) return fail(PACH_ERR_NOT_READY, "run still in progress");
            if (run->status != PACH_OK && run->status != PACH_ERR_CANCELLED) return fail(run->status, run->err);
        }
        if (run->R == 0) return fail(PACH_ERR_INVALID_ARGUMENT, "the run has no receivers");
        const int kinds = directional ? 7 : 1;
        const size_t n_out = (size_t)run->R * kinds * ((size_t)run->T + 16383 - 4096);
        if (!out || cap < n_out) return fail(PACH_ERR_INVALID_ARGUMENT, "cap < receivers x filters x (T + 12287)");
        cudaSetDevice(run->scene->device);
        // each receiver's pressure factor of the scaled histograms, sqrt(n_sources / N) (P Dir / E keeps it)
        std::vector<double> scale;
        const long long done = run->rays_done.load();
        for (const RoomSpec &rm : run->rooms) {
            const long long off = rm.prim_begin - run->rooms[0].prim_begin;
            const double N = (double)std::max(1ll, std::min(rm.rays, done - off));
            scale.insert(scale.end(), rm.rec.size(), std::sqrt((double)rm.src.size()) / std::sqrt(N));
        }
        const size_t wsb = filters_workspace_bytes(run->R * kinds, run->T);
        DevMem dscale, dout, ws;
        cudaError_t e;
        if ((e = dscale.alloc(scale.size() * sizeof(double))) != cudaSuccess ||
            (e = dout.alloc(n_out * sizeof(double))) != cudaSuccess || (e = ws.alloc(wsb)) != cudaSuccess)
            return fail(PACH_ERR_OUT_OF_MEMORY, cuda_msg(e, "filter buffers"));
        if ((e = cudaMemcpy(dscale.p, scale.data(), scale.size() * sizeof(double), cudaMemcpyHostToDevice)) != cudaSuccess)
            return fail(PACH_ERR_CUDA, cuda_msg(e, "filter scale copy"));
        pach_status s = filters_device(run->hE.as<double>(), run->hP.as<double>(), run->hDp.as<double>(),
                                       run->hDn.as<double>(), dscale.as<double>(), run->R, run->T, kinds,
                                       run->p.sample_rate, swl, 4096, dout.as<double>(), ws.p, wsb, nullptr);
        if (s != PACH_OK) return s;
        if ((e = cudaMemcpy(out, dout.p, n_out * sizeof(double), cudaMemcpyDeviceToHost)) != cudaSuccess)
            return fail(PACH_ERR_CUDA, cuda_msg(e, "filters"));
        return PACH_OK;
    }, fail);
}

pach_status pach_trace_get_capture(pach_run *run, float *out, size_t cap) {
    return guarded([&]() -> pach_status {
        if (pach_status s = check_run(run)) return s;
        {
            std::lock_guard<std::mutex> lk(run->mu);
            if (!run->finished) return fail(PACH_ERR_NOT_READY, "run still in progress");
            if (run->status != PACH_OK && run->status != PACH_ERR_CANCELLED) return fail(run->status, run->err);
        }
        if (!run->p.capture) return fail(PACH_ERR_INVALID_ARGUMENT, "the run was made without capture");
        const size_t per = run->p.capture == 2 ? (size_t)rprim_total(run) : (size_t)kDirBins;
        const size_t n = (size_t)run->R * kCaptureWindows * per;
        if (!out || cap < n) return fail(PACH_ERR_INVALID_ARGUMENT, "cap < receivers * 4 * (1536 bins or primaries)");
        cudaSetDevice(run->scene->device);
        cudaError_t e = cudaMemcpy(out, run->dcap.p, n * sizeof(float), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return fail(PACH_ERR_CUDA, cuda_msg(e, "capture copy"));
        return PACH_OK;
    }, fail);
}

pach_status pach_trace_get_map(pach_run *run, int32_t scaled, double *energy, double *pressure, double *direct_time,
                               int32_t *sizes, size_t cap_bins) {
    return guarded([&]() -> pach_status {
        if (pach_status s = check_run(run)) return s;
        if (!run->has_map) return fail(PACH_ERR_INVALID_ARGUMENT, "the run has no mapping receivers");
        const MapGrid &g = run->mg;
        if (sizes) { sizes[0] = g.M; sizes[1] = g.T; }
        if (direct_time) std::memcpy(direct_time, g.direct.data(), g.direct.size() * sizeof(double));
        if (!energy && !pressure) return PACH_OK;
        {
            std::lock_guard<std::mutex> lk(run->mu);
            if (!run->finished) return fail(PACH_ERR_NOT_READY, "run still in progress");
            if (run->status != PACH_OK && run->status != PACH_ERR_CANCELLED) return fail(run->status, run->err);
        }
        const size_t n = (size_t)g.M * kBands * g.T;
        if (cap_bins < n) return fail(PACH_ERR_INVALID_ARGUMENT, "cap_bins < map receivers * 8 * bins");
        cudaSetDevice(run->scene->device);
        // Histogram.Scale(N) divides energy and pressure by N (Directional_Histogram.Scale: pressure by
        // sqrt(N)); a cluster's Scale(1 / n_sources) multiplies back
        const double N = (double)std::max(1ll, run->rays_done.load());
        const double f = (double)run->nsrc / N;
        const double fp = g.directional ? std::sqrt((double)run->nsrc / N) : f;
        for (auto [dst, src, k] : {std::tuple<double *, DevMem *, double>{energy, &run->mE, f}, {pressure, &run->mP, fp}}) {
            if (!dst) continue;
            cudaError_t e = cudaMemcpy(dst, src->p, n * sizeof(double), cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) return fail(PACH_ERR_CUDA, cuda_msg(e, "map copy"));
            if (scaled)
                for (size_t i = 0; i < n; ++i) dst[i] *= k;
        }
        return PACH_OK;
    }, fail);
}

pach_status pach_trace_get_map_directions(pach_run *run, int32_t scaled, double *dir_pos, double *dir_neg,
                                          size_t cap_bins) {
    return guarded([&]() -> pach_status {
        if (pach_status s = check_run(run)) return s;
        if (!run->has_map || !run->mg.directional) return fail(PACH_ERR_INVALID_ARGUMENT, "the run has no directional map");
        {
            std::lock_guard<std::mutex> lk(run->mu);
            if (!run->finished) return fail(PACH_ERR_NOT_READY, "run still in progress");
            if (run->status != PACH_OK && run->status != PACH_ERR_CANCELLED) return fail(run->status, run->err);
        }
        const MapGrid &g = run->mg;
        const size_t n = (size_t)g.M * 3 * kBands * g.T;
        if (cap_bins < n) return fail(PACH_ERR_INVALID_ARGUMENT, "cap_bins < map receivers * 3 * 8 * bins");
        cudaSetDevice(run->scene->device);
        const double f = (double)run->nsrc / (double)std::max(1ll, run->rays_done.load());
        for (auto [dst, src] : {std::pair<double *, DevMem *>{dir_pos, &run->mDp}, {dir_neg, &run->mDn}}) {
            if (!dst) continue;
            cudaError_t e = cudaMemcpy(dst, src->p, n * sizeof(double), cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) return fail(PACH_ERR_CUDA, cuda_msg(e, "map direction copy"));
            if (scaled)
                for (size_t i = 0; i < n; ++i) dst[i] *= f;
        }
        return PACH_OK;
    }, fail);
}

pach_status pach_map_parameters(pach_run *run, int32_t decay_depth, int32_t clarity_ms, double *t_x, double *edt,
                                double *clarity, double *definition, double *energy_sum) {
    return guarded([&]() -> pach_status {
        if (pach_status s = check_run(run)) return s;
        if (!run->has_map) return fail(PACH_ERR_INVALID_ARGUMENT, "the run has no mapping receivers");
        {
            std::lock_guard<std::mutex> lk(run->mu);
            if (!run->finished) return fail(PACH_ERR_NOT_READY, "run still in progress");
            if (run->status != PACH_OK && run->status != PACH_ERR_CANCELLED) return fail(run->status, run->err);
        }
        const MapGrid &g = run->mg;
        const int n = g.M * kBands;
        cudaSetDevice(run->scene->device);
        DevMem out;
        struct Release {
            DevMem &m;
            ~Release() { m.release(); }
        } release_out{out};
        cudaError_t e = out.alloc((size_t)5 * n * sizeof(double));
        if (e != cudaSuccess) return fail(PACH_ERR_OUT_OF_MEMORY, cuda_msg(e, "parameter map buffers"));
        double *d = out.as<double>();
        const double scale = (double)run->nsrc / (double)std::max(1ll, run->rays_done.load());
        e = launch_map_params(run->mE.as<double>(), n, g.T, 1000.0, scale, decay_depth, clarity_ms / 1000.0, d, d + n,
                              d + 2 * (size_t)n, d + 3 * (size_t)n, d + 4 * (size_t)n, nullptr);
        if (e == cudaSuccess) e = cudaDeviceSynchronize();
        if (e != cudaSuccess) return fail(PACH_ERR_CUDA, cuda_msg(e, "parameter map kernel"));
        double *dst[5] = {t_x, edt, clarity, definition, energy_sum};
        for (int i = 0; i < 5; ++i) {
            if (!dst[i]) continue;
            e = cudaMemcpy(dst[i], d + (size_t)i * n, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) return fail(PACH_ERR_CUDA, cuda_msg(e, "parameter map copy"));
        }
        return PACH_OK;
    }, fail);
}

pach_status pach_etc_parameters(const double *etc, int32_t n, int32_t T, int32_t sample_rate, int32_t decay_depth,
                                double clarity_s, double *t_x, double *edt, double *clarity, double *definition,
                                double *energy_sum) {
    return guarded([&]() -> pach_status {
        if (n < 0 || T < 1 || sample_rate < 1 || (n > 0 && !etc))
            return fail(PACH_ERR_INVALID_ARGUMENT, "etc_parameters: need n >= 0 curves of T >= 1 bins at a positive rate");
        if (n == 0) return PACH_OK;
        if (pach_device_count() <= 0) return fail(PACH_ERR_NO_DEVICE, "no CUDA device visible");
        DevMem in, out;
        struct Release {
            DevMem &a, &b;
            ~Release() { a.release(); b.release(); }
        } release_bufs{in, out};
        const size_t bytes = (size_t)n * T * sizeof(double);
        cudaError_t e = upload(in, etc, bytes);
        if (e == cudaSuccess) e = out.alloc((size_t)5 * n * sizeof(double));
        if (e != cudaSuccess) return fail(PACH_ERR_OUT_OF_MEMORY, cuda_msg(e, "etc_parameters buffers"));
        double *d = out.as<double>();
        e = launch_map_params(in.as<double>(), n, T, (double)sample_rate, 1.0, decay_depth, clarity_s, d, d + n,
                              d + 2 * (size_t)n, d + 3 * (size_t)n, d + 4 * (size_t)n, nullptr);
        if (e == cudaSuccess) e = cudaDeviceSynchronize();
        if (e != cudaSuccess) return fail(PACH_ERR_CUDA, cuda_msg(e, "etc_parameters kernel"));
        double *dst[5] = {t_x, edt, clarity, definition, energy_sum};
        for (int i = 0; i < 5; ++i) {
            if (!dst[i]) continue;
            e = cudaMemcpy(dst[i], d + (size_t)i * n, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) return fail(PACH_ERR_CUDA, cuda_msg(e, "etc_parameters copy"));
        }
        return PACH_OK;
    }, fail);
}

pach_status pach_trace_get_stats(pach_run *run, pach_stats *stats) {
    return guarded([&]() -> pach_status {
        if (pach_status s = check_run(run)) return s;
        if (!stats) return fail(PACH_ERR_INVALID_ARGUMENT, "stats is null");
        std::lock_guard<std::mutex> lk(run->mu);
        if (!run->finished) return fail(PACH_ERR_NOT_READY, "run still in progress");
        *stats = run->stats;
        return PACH_OK;
    }, fail);
}

void pach_run_destroy(pach_run *run) { delete run; }

pach_status pach_trace_run(pach_scene *scene, const pach_source_desc *sources, int32_t n_sources,
                           const pach_receiver_desc *receivers, int32_t n_receivers, const pach_trace_params *params,
                           int32_t scaled, double *energy, double *pressure, double *dir_pos, double *dir_neg,
                           double *analysis, size_t cap_bins, pach_stats *stats) {
    return guarded([&]() -> pach_status {
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
    }, fail);
}

pach_status pach_trace_specular_paths(pach_scene *scene, int32_t n, const double *origins, const double *dirs,
                                      int32_t max_bounces, int32_t *poly_out, double *t_out, double *pts_out) {
    return guarded([&]() -> pach_status {
        if (!scene || n < 0 || max_bounces < 1 || !origins || !dirs || !poly_out || !t_out || !pts_out)
            return fail(PACH_ERR_INVALID_ARGUMENT, "bad arguments");
        if (n == 0) return PACH_OK;
        cudaSetDevice(scene->device);
        DevMem o, d, pl, t, pt;
        const size_t k = (size_t)n * max_bounces;
        cudaError_t e;
        if ((e = scene_upload(scene)) || (e = upload(o, origins, sizeof(double) * 3 * n)) || (e = upload(d, dirs, sizeof(double) * 3 * n)) ||
            (e = pl.alloc(sizeof(int32_t) * k)) || (e = t.alloc(sizeof(double) * k)) || (e = pt.alloc(sizeof(double) * 3 * k)) ||
            (e = launch_paths(scene->dev, n, o.as<double>(), d.as<double>(), max_bounces, pl.as<int>(), t.as<double>(),
                              pt.as<double>(), 0)) ||
            (e = cudaMemcpy(poly_out, pl.p, sizeof(int32_t) * k, cudaMemcpyDeviceToHost)) ||
            (e = cudaMemcpy(t_out, t.p, sizeof(double) * k, cudaMemcpyDeviceToHost)) ||
            (e = cudaMemcpy(pts_out, pt.p, sizeof(double) * 3 * k, cudaMemcpyDeviceToHost)))
            return fail(PACH_ERR_CUDA, cuda_msg(e, "specular paths"));
        return PACH_OK;
    }, fail);
}

pach_status pach_scene_shoot_host(const pach_scene_desc *desc, int32_t n, const double *origins, const double *dirs,
                                  int32_t *poly_out, double *t_out) {
    return guarded([&]() -> pach_status {
        if (n < 0 || (n > 0 && (!origins || !dirs || !poly_out || !t_out))) return fail(PACH_ERR_INVALID_ARGUMENT, "bad arguments");
        HostScene hs;
        std::string err;
        if (!build_host_scene(desc, hs, err)) return fail(PACH_ERR_INVALID_ARGUMENT, err);
        for (int i = 0; i < n; ++i) {
            const double o[3] = {origins[3 * i], origins[3 * i + 1], origins[3 * i + 2]};
            double d[3] = {dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]};
            const double l = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            for (double &x : d) x /= l;
            int tri = -1;
            double t = 0;
            if (bvh_shoot_host(hs, o, d, 1e-10, tri, t)) {
                poly_out[i] = hs.tri_poly[tri];
                t_out[i] = t;
            } else {
                poly_out[i] = -1;
                t_out[i] = 0;
            }
        }
        return PACH_OK;
    }, fail);
}

pach_status pach_emit_directions(uint64_t seed, int64_t ray_begin, int32_t n, int32_t n_sources, int32_t kind,
                                 double *dirs_out) {
    return guarded([&]() -> pach_status {
        if (n < 0 || n_sources < 1 || n_sources > kMaxSources || kind < 0 || kind > 2 || !dirs_out)
            return fail(PACH_ERR_INVALID_ARGUMENT, "bad arguments");
        if (n == 0) return PACH_OK;
        if (pach_device_count() <= 0) return fail(PACH_ERR_NO_DEVICE, "no CUDA device visible");
        std::vector<float4> src(n_sources, make_float4(0, 0, 0, (float)kind));
        std::vector<double> gf;
        geodesic_faces(gf);
        std::vector<float4> geo(kGeoFaces * 3);
        for (int i = 0; i < kGeoFaces * 3; ++i) geo[i] = make_float4((float)gf[3 * i], (float)gf[3 * i + 1], (float)gf[3 * i + 2], 0.f);
        DevMem ds, dg, dout, droom;
        cudaError_t e;
        DevRun r{};
        r.seed = seed;
        RoomParams room{};
        room.nsrc = n_sources;
        if ((e = upload(ds, src.data(), src.size() * sizeof(float4))) || (e = upload(dg, geo.data(), geo.size() * sizeof(float4))) ||
            (e = upload(droom, &room, sizeof(room))) || (e = dout.alloc(sizeof(double) * 3 * n)))
            return fail(PACH_ERR_CUDA, cuda_msg(e, "emit setup"));
        r.src = ds.as<float4>();
        r.geo = dg.as<float4>();
        r.rooms = droom.as<RoomParams>();
        r.n_rooms = 1;
        if ((e = launch_emit(r, ray_begin, n, dout.as<double>(), 0)) ||
            (e = cudaMemcpy(dirs_out, dout.p, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost)))
            return fail(PACH_ERR_CUDA, cuda_msg(e, "emit"));
        return PACH_OK;
    }, fail);
}

int32_t pach_direction_bin(double x, double y, double z) { return dir_bin((float)x, (float)y, (float)z); }

pach_status pach_direct_sound(pach_scene *scene, const pach_source_desc *sources, int32_t n_sources,
                              const pach_receiver_desc *receivers, int32_t n_receivers, int32_t *valid,
                              double *distance, double *energy) {
    return guarded([&]() -> pach_status {
        if (!scene || !sources || n_sources < 1 || n_receivers < 0 || (n_receivers > 0 && (!receivers || !valid)))
            return fail(PACH_ERR_INVALID_ARGUMENT, "bad arguments");
        if ((long long)n_sources * n_receivers > (1ll << 30)) return fail(PACH_ERR_INVALID_ARGUMENT, "too many pairs");
        if (n_receivers == 0) return PACH_OK;
        cudaSetDevice(scene->device);
        const HostScene &hs = scene->hs;
        std::vector<double> s3(3 * (size_t)n_sources), r3(3 * (size_t)n_receivers);
        for (int s = 0; s < n_sources; ++s)
            for (int a = 0; a < 3; ++a) s3[3 * s + a] = sources[s].origin[a];
        for (int k = 0; k < n_receivers; ++k)
            for (int a = 0; a < 3; ++a) r3[3 * k + a] = receivers[k].origin[a];
        const size_t npair = (size_t)n_sources * n_receivers;
        DevMem ds, dr, dv, dt;
        std::vector<int> v(npair);
        std::vector<double> tm(npair * kBands);
        cudaError_t e;
        if ((e = scene_upload(scene)) || (e = upload(ds, s3.data(), s3.size() * sizeof(double))) ||
            (e = upload(dr, r3.data(), r3.size() * sizeof(double))) ||
            (e = dv.alloc(npair * sizeof(int))) || (e = dt.alloc(npair * kBands * sizeof(double))) ||
            (e = launch_direct(scene->dev, ds.as<double>(), n_sources, dr.as<double>(), n_receivers, 64, dv.as<int>(),
                               dt.as<double>(), 0)) ||
            (e = cudaMemcpy(v.data(), dv.p, npair * sizeof(int), cudaMemcpyDeviceToHost)) ||
            (e = cudaMemcpy(tm.data(), dt.p, npair * kBands * sizeof(double), cudaMemcpyDeviceToHost)))
            return fail(PACH_ERR_CUDA, cuda_msg(e, "direct sound"));
        for (int k = 0; k < n_receivers; ++k)
            for (int s = 0; s < n_sources; ++s) {
                const size_t p = (size_t)k * n_sources + s;
                const double dx = r3[3 * k] - s3[3 * s], dy = r3[3 * k + 1] - s3[3 * s + 1], dz = r3[3 * k + 2] - s3[3 * s + 2];
                const double L = std::sqrt(dx * dx + dy * dy + dz * dz);
                valid[p] = v[p];
                if (distance) distance[p] = L;
                if (energy)
                    for (int o = 0; o < kBands; ++o) {
                        const double P = 1e-12 * std::pow(10.0, .1 * sources[s].power_db[o]);
                        energy[p * kBands + o] = P * std::pow(10.0, -.1 * hs.atten[o] * L) * tm[p * kBands + o] / (4 * M_PI * L * L);
                    }
            }
        return PACH_OK;
    }, fail);
}

pach_status pach_proposal_sample(const float *proposal, int32_t n_prop, double mix, uint64_t seed, int64_t ray_begin,
                                 int32_t n, float *dirs, float *weights) {
    return guarded([&]() -> pach_status {
        if (!proposal || n_prop < 1 || n_prop > 256 || !(mix >= 0 && mix <= 1) || n < 0 || ray_begin < 0 ||
            ray_begin + n > (1ll << 32) || (n > 0 && (!dirs || !weights)))
            return fail(PACH_ERR_INVALID_ARGUMENT, "bad arguments");
        if (n == 0) return PACH_OK;
        if (pach_device_count() <= 0) return fail(PACH_ERR_NO_DEVICE, "no CUDA device visible");
        std::vector<float> lobes;
        proposal_lobes(proposal, n_prop, lobes);
        DevMem dl, dd, dw;
        cudaError_t e;
        if ((e = upload(dl, lobes.data(), lobes.size() * sizeof(float))) || (e = dd.alloc(sizeof(float) * 3 * n)) ||
            (e = dw.alloc(sizeof(float) * n)))
            return fail(PACH_ERR_CUDA, cuda_msg(e, "proposal sample setup"));
        DevRun r{};
        r.seed = seed;
        r.prop = dl.as<float4>();
        r.n_prop = n_prop;
        r.prop_mix = (float)(mix > 0 ? mix : 0.3);
        if ((e = launch_prop_sample(r, ray_begin, n, dd.as<float>(), dw.as<float>(), 0)) ||
            (e = cudaMemcpy(dirs, dd.p, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost)) ||
            (e = cudaMemcpy(weights, dw.p, sizeof(float) * n, cudaMemcpyDeviceToHost)))
            return fail(PACH_ERR_CUDA, cuda_msg(e, "proposal sample"));
        return PACH_OK;
    }, fail);
}

}  // extern "C"

// Read access to scene handles for entry points defined in other translation units.
namespace pach {
const HostScene *scene_host(const pach_scene *s) { return s ? &s->hs : nullptr; }
const DevScene *scene_dev(const pach_scene *s) { return s && s->on_device ? &s->dev : nullptr; }
int scene_device(const pach_scene *s) { return s ? s->device : -1; }
void set_last_error(const char *msg) { g_err = msg; }
}  // namespace pach
