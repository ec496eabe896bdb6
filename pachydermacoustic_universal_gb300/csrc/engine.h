// engine.h -- internal structures shared by the host side (scene build, C ABI) and the kernels.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <exception>
#include <future>
#include <memory>
#include <new>
#include <string>
#include <thread>
#include <utility>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/pach_gpu.h"
#include "../../include/pach_proposal.h"

namespace pach {

constexpr int kBands = 8;
constexpr int kMaxSources = 64;
constexpr int kGeoFaces = 80;

// Allocator whose resize() leaves elements default-initialised (no zero fill): the large host arrays
// of a scene are sized first and then filled by parallel chunks, which also spreads the first-touch
// page faults over the threads.
template <class T>
struct UninitAlloc : std::allocator<T> {
    template <class U>
    struct rebind { using other = UninitAlloc<U>; };
    UninitAlloc() = default;
    template <class U>
    UninitAlloc(const UninitAlloc<U> &) noexcept {}
    template <class U>
    void construct(U *p) noexcept { ::new ((void *)p) U; }
    template <class U, class... A>
    void construct(U *p, A &&...a) { ::new ((void *)p) U(std::forward<A>(a)...); }
};
template <class T>
using hvec = std::vector<T, UninitAlloc<T>>;

// Runs an entry point's body so that no C++ exception crosses the C ABI: a failed host allocation or
// thread creation becomes PACH_ERR_OUT_OF_MEMORY with a message stored by `report` (the entry
// point's last-error setter).
template <class F, class R>
pach_status guarded(F &&body, R &&report) noexcept {
    try {
        return body();
    } catch (const std::bad_alloc &) {
        return report(PACH_ERR_OUT_OF_MEMORY, std::string("out of host memory"));
    } catch (const std::exception &e) {
        return report(PACH_ERR_OUT_OF_MEMORY, std::string("host resources exhausted: ") + e.what());
    } catch (...) {
        return report(PACH_ERR_OUT_OF_MEMORY, std::string("host resources exhausted"));
    }
}

// Runs f(c0, c1) over [0, n) in chunks of `grain` elements on up to hardware_concurrency() threads;
// inline when one chunk covers the range.  Chunk c is [c * grain, min(n, (c + 1) * grain)).
template <class F>
void parallel_chunks(size_t n, size_t grain, F &&f) {
    const size_t nch = (n + grain - 1) / grain;
    if (nch <= 1) {
        if (n) f((size_t)0, n);
        return;
    }
    const size_t nt = std::min(nch, (size_t)std::max(1u, std::thread::hardware_concurrency()));
    auto run = [&](size_t t) {
        for (size_t c = t; c < nch; c += nt) f(c * grain, std::min(n, (c + 1) * grain));
    };
    std::vector<std::future<void>> parts;
    for (size_t t = 1; t < nt; ++t) parts.push_back(std::async(std::launch::async, run, t));
    run(0);
    for (auto &p : parts) p.get();
}

// Host-side prepared scene (FP64 master copy + FP32 device layout sources).
struct HostScene {
    int npoly = 0, ntri = 0;
    hvec<double> tri64;              // [ntri][9]: v0, e1, e2
    hvec<int32_t> tri_poly;          // [ntri]
    hvec<int32_t> tri_plane;         // [ntri] coplanar group id
    hvec<double> normal;             // [npoly][3]
    hvec<double> area;               // [npoly]
    hvec<double> alpha, scat, trans;  // [npoly][8]
    bool has_trans = false;
    double bmin[3], bmax[3];
    // BVH: 4-wide, collapsed from an SAH binary tree; triangles above are stored in leaf order.
    // node n = 8 float4 (128 B): lo.x[4], hi.x[4], lo.y[4], hi.y[4], lo.z[4], hi.z[4], child[4] (int
    // bits), unused; a child >= 0 is an inner node, < 0 the leaf ~(first * 16 + count - 1); an
    // empty slot has an inverted box.
    hvec<float> bvh;                 // [nodes*32]
    hvec<float> bvhq;                // [nodes*12]: the same tree with 8-bit child boxes (48-byte nodes; empty
                                     // when the triangle ids need more than 24 bits)
    int bvh_nodes = 0, bvh_leaves = 0, bvh_depth = 0;
    double c = 343, rho = 1.2, rho_c = 411.6, atten[kBands] = {0};
    double scale = 1;                // largest box extent
};

constexpr int kBvhStack = 64;
constexpr int kBvhNodeFloats = 32;
constexpr int kBvhQNodeFloats = 12;  // 48-byte quantised nodes
constexpr int kLeafMax = 8;      // largest leaf the node encoding holds
constexpr int kLeafDefault = 3;  // leaf size used when the scene does not ask for one (measured best of 2..8)

// Device scene view (passed by value to kernels).
struct DevScene {
    const float4 *tri;          // [ntri*3]: (v0, plane bits) (e1, poly bits) (e2, grazing threshold)
    const double *tri64;        // [ntri*9]
    const float4 *pnormal;      // [npoly]
    const float4 *mat;          // [npoly*8]: (1-alpha, s_lo, s_mid, s_hi)
    const float *trans;         // [npoly*8]
    const float4 *bvh;          // [nodes*8] 128-byte nodes
    const float4 *bvhq;         // [nodes*3] 48-byte quantised nodes (null: walk the 128-byte ones)
    int ntri;
    float t_eps;
    int has_trans;
};

// One octave ray in a device queue: 64 bytes, 16-byte aligned.
struct __align__(16) ORayItem {
    float px, py, pz, I;        // position, intensity relative to the primary's initial band energy
    float dx, dy, dz, scale;    // direction, absolute energy of I = 1 (E0[band] x emission weight)
    double t_sum;               // seconds travelled
    uint32_t prim;              // primary ray index
    uint32_t nb;                // draw blocks used on this stream
    unsigned long long sid;     // stream identity in the split tree
    uint32_t meta;              // bits 0-2 band, 3-4 Scatter_Mask, 5 phase (0 B, 1 C), 6-31 room
    int32_t plane;              // coplanar group of the surface the ray leaves (-1 none)
};

// Counters accumulated by the kernels (one instance in device memory).
struct DevCounters {
    unsigned long long primaries, seg_broad, seg_b, seg_c, octave_rays, end_traces, detections, capped,
        retests, queue_overflow, stack_spills, lost_items, bvh_nodes, tri_tests;
    double lost_energy, initial_energy;
};

// Device-side schedule of the wavefront loop (one instance in device memory).
struct WaveCtl {
    unsigned long long head, tail;  // ring indices, monotonic
    unsigned long long m;           // items in the current wave
    long long next_prim, prim_end;  // primaries still to feed: [next_prim, prim_end)
    long long pa_begin, pa_count;   // phase-A batch of the current iteration
    unsigned long long waves, overflow, peak_live;
    long long prim_first;           // first primary of the run
    unsigned long long per_prim;    // peak ring footprint per primary measured by the pilot batch (0 = not yet)
    unsigned long long trace_next;  // next wave item a trace thread takes (dynamic fetch)
    unsigned long long last_live;   // live count at the previous feed decision
    unsigned long long iters;       // loop iterations run (graph mode)
    unsigned long long idle;        // consecutive iterations that neither traced nor fed
    int done, gave_up;
    long long pilot_count;          // primaries of the pilot in flight (0: none)
    unsigned long long pilot_peak;  // peak live count while the pilot runs
    int pilot_room;                 // first room whose ring footprint has not been measured by a pilot
    int pressure;                   // the ring passed three quarters full since the last batch was fed
};

// Progress mirror in mapped host memory, written by the device every iteration in graph mode.
struct HostMirror {
    long long next_prim;
    unsigned long long iters, segments, end_traces;
    int done, gave_up;
};

// One room of a run (a plain run is a batch of one room).  Rooms share the run's device scene (the
// concatenation of their scenes), receiver, source and histogram tables; a room owns the ranges below.
struct RoomParams {
    long long prim_begin, prim_end;  // its primaries in the run's global primary numbering
    double inv_c_d, cotime;          // 1 / c, COTime = cutoff length / c (s)
    float inv_c, rho_c;
    float atten_k[kBands];           // exp2 factor per second of travel: -0.1 log2(10) m c
    float t_eps;                     // smallest hit distance (2e-7 x the room's scale)
    int bvh_root;                    // root node of its BVH in the run's node array
    int rec_begin, R;                // its receivers [rec_begin, rec_begin + R) (run-wide receiver index)
    int src_begin, nsrc;             // its sources
    int h_oct, oct_lo, oct_hi, is_order, pure_specular, max_broad;
};
constexpr int kMaxRooms = 4096;
// Receiver tables up to this size are staged in shared memory by the detection kernels.
constexpr int kSmemReceivers = 256;
// staged: the float4 table, then the original index of each sorted slot
inline int receiver_smem_bytes(int R) { return 20 * (R > 0 && R <= kSmemReceivers ? R : 1); }

constexpr long long kPilotPrimaries = 256;

// Mapping receivers on the device (PachMapReceiver).  The grid is the reference's: cells of
// BoxDims / ceil(BoxDims / (4, 4, 2.5 increments)) over the spheres' bounding box; cell c lists
// the receivers whose sphere overlaps it (FP64 sphere-box test on the host), each entry with a
// 27-bit mask of the neighbouring cells (bit (dx+1)*9 + (dy+1)*3 + (dz+1)) that list it too, so a
// walk tests a receiver once (the reference's Ray_ID mailbox).
struct MapDev {
    const float4 *rec;        // [M] (x, y, z, r^2)
    const double *direct;     // [M] direct arrival time (s)
    const int *cell;          // [cells + 1] entry offsets, cell = (x * ny + y) * nz + z
    const uint2 *entry;       // (receiver, neighbour mask)
    double *E, *P;            // [M][8][T]
    double *Dp, *Dn;          // [M][3][8][T] (directional maps)
    float lo[3], hi[3];       // grid box (OBox)
    float vd[3];              // cell size
    int n[3];                 // cells per axis
    int M, T;
    int one_pt;               // Histogram_1Pt: every arrival in bin 0, no pressure
    int walk;                 // 0 the reference's walks, 1 every crossed cell
    int directional;          // Directional_Histogram: pressure sqrt(E rho c) and arrival directions
    float rho_c;
    float size_mod;           // 1 / (pi r^2)
    float atten_k[kBands];    // exp2 factor per second after the direct arrival: -0.1 log2(10) m
};

// Host side of the mapping receivers (map_grid.cpp): the grid in FP64 and its cell lists.
struct MapGrid {
    int M = 0, T = 1, walk = 0;
    bool one_pt = false, directional = false;
    double r = 0, r2 = 0;
    double mn[3] = {0, 0, 0}, mx[3] = {0, 0, 0}, vd[3] = {1, 1, 1};
    int n[3] = {1, 1, 1};
    std::vector<int> cell_off;      // [cells + 1]
    std::vector<uint2> entry;       // (receiver, neighbour mask)
    std::vector<double> direct;     // [M] s
};
bool build_map_grid(const pach_map_desc &d, const double src[3], int nsrc, double c, MapGrid &g, std::string &err);

// Launch-wide parameters (kernel argument).
struct DevRun {
    DevScene S;
    // rooms: room i holds primaries [room_prim[i], room_prim[i + 1])
    const RoomParams *rooms;    // [n_rooms]
    const long long *room_prim; // [n_rooms + 1]
    int n_rooms;
    // receivers of every room
    // each room's receivers ordered by the coordinate of their widest spread (measured 0.7-4.8 % faster
    // detection than the given order on a shoebox, a hall and an arena)
    const float4 *rec;          // [R] (x, y, z, r^2)
    const int *rec_id;          // [R] histogram row of each slot (null: slot = row)
    int R, T;
    double fs;                  // histogram rate (Hz)
    // sources of every room
    const float4 *src;          // [sources] origin (w = kind)
    const float *e0;            // [sources*8] band powers (W)
    const float4 *geo;          // [80*3] geodesic face vertices
    const double *prim_dirs;    // optional, indexed by prim - prim_base
    const double *prim_weights;
    long long prim_base;
    unsigned long long seed;
    long long max_seg;
    volatile int *cancel;       // mapped host flag: stop feeding (graph mode; null otherwise)
    HostMirror *mirror;         // mapped host progress (graph mode; null otherwise)
    unsigned long long max_iters;  // graph mode: iteration cap
    // outputs
    double *hE, *hP, *hDp, *hDn, *hAn;
    DevCounters *cnt;
    // wavefront ring of octave rays (live items are [head, tail) modulo ring_cap)
    ORayItem *ring;
    unsigned long long ring_cap;   // power of two
    WaveCtl *ctl;
    int4 *hits;                    // per wave slot: (triangle, t bits, polygon, coplanar group); triangle -1 =
                                   // miss.  The walk writes the hit's polygon and group so that the shading
                                   // pass loads normal and material directly, one dependent load fewer
    unsigned long long max_wave;   // items per wave at most
    long long feed_batch;          // primaries per phase-A launch at most
    unsigned long long feed_bound; // ring slots one primary can fill in phase A
    unsigned long long low_water;  // feed new primaries when fewer live items remain
    // per-wave ray order (counting sort by direction octant and origin cell)
    ORayItem *wave_buf;            // the wave, sorted (null: trace and shade read the ring in place)
    unsigned *bin_count;           // [kSortBins], zero between waves
    unsigned *bin_cursor;          // [kSortBins]
    float sort_lo[3], sort_inv[3]; // origin grid: cell = (p - lo) * inv, 0..kSortGrid-1 per axis
    // learned emission proposal (null: the source's own emission)
    const float4 *prop;            // [n_prop][kLobes][2]: (mu xyz, kappa), (log pi + log norm, cdf, 0, 0)
    int n_prop;
    float prop_mix;                // probability of the uniform component
    // training capture (null: off).  Mode 1: energy per receiver, time window and emission-direction
    // bin, [R][kCaptureWindows][kDirBins].  Mode 2: energy per primary, receiver and time window,
    // [primaries][R][kCaptureWindows] (primary index - prim_base).
    float *capture;
    int capture_mode;
    float cap_edge[3];             // window edges, ms after the direct arrival
    // mapping receivers (used by the map variants of the broadband and shading kernels)
    MapDev map;
    // convergence mode (null: off): each revolution's contribution to the check receivers' band-conv_oct
    // histograms, [kConvChunk][2][kConvKinds][T]; revolution = (primary - ctl->prim_first) / conv_period
    double *conv;
    int conv_row[2];               // histogram rows of the check receivers (-1: none)
    int conv_oct;
    long long conv_period;         // primaries per revolution
    int count_work;                // 1: the walk counts its node visits and triangle tests (kernel-timing runs)
};

constexpr int kLobes = PACH_MLP_LOBES;
constexpr int kDirBins = PACH_DIR_BINS;
constexpr int kCaptureWindows = PACH_CAPTURE_WINDOWS;

// Emission-direction bin: cube map with faces +x -x +y -y +z -z, 16 x 16 cells each; a face's cell
// (i, j) covers u, v in [i/8 - 1, (i+1)/8 - 1) x [j/8 - 1, (j+1)/8 - 1) of the face's two other
// axes in x, y, z order (u = second / major, v = third / major).
__host__ __device__ inline int dir_bin(float x, float y, float z) {
    const float ax = fabsf(x), ay = fabsf(y), az = fabsf(z);
    int f;
    float u, v;
    if (ax >= ay && ax >= az) {
        f = x > 0.f ? 0 : 1;
        u = y / ax;
        v = z / ax;
    } else if (ay >= az) {
        f = y > 0.f ? 2 : 3;
        u = x / ay;
        v = z / ay;
    } else {
        f = z > 0.f ? 4 : 5;
        u = x / az;
        v = y / az;
    }
    int i = (int)((u + 1.f) * 8.f), j = (int)((v + 1.f) * 8.f);
    i = i < 0 ? 0 : (i > 15 ? 15 : i);
    j = j < 0 ? 0 : (j > 15 ? 15 : j);
    return f * 256 + j * 16 + i;
}

// mlp.cu: raw network outputs [n][160] -> the lobe table DevRun::prop holds ([n][kLobes][8] floats)
void proposal_lobes(const float *raw, int n, std::vector<float> &out);

constexpr int kSortGrid = 8;                       // origin cells per axis
constexpr int kSortBins = 8 * kSortGrid * kSortGrid * kSortGrid;  // x 8 direction octants

// trace.cu entry points (host wrappers).  One wavefront iteration:
//   feed (1 thread) -> broadband (phase A of the fed primaries) -> wave (1 thread: size the wave)
//   -> trace (BVH walk of every ray of the wave) -> shade (detect, absorb, scatter, append).
cudaError_t launch_feed(const DevRun &r, cudaStream_t s);
cudaError_t launch_cond(const DevRun &r, cudaGraphConditionalHandle h, cudaStream_t s);
// small: every room has at most kFuseMaxTris triangles (walk with the plain stack)
cudaError_t launch_broadband(const DevRun &r, int blocks, int threads, cudaStream_t s, bool map = false,
                             bool small = false);
cudaError_t launch_wave(const DevRun &r, cudaStream_t s);
cudaError_t launch_sort(const DevRun &r, int blocks, cudaStream_t s);  // count -> scan -> scatter
// variant: 256-thread blocks per SM the trace kernel is compiled for (3..6; others -> 4), plus 16 for the
// speculative BVH walk (compiled for 4 and 6 blocks per SM).  traversal 0 picks the speculative walk for
// scenes of more than kSpecMinTris triangles: measured on a 20k-triangle hall it walks 1.5x faster than
// one leaf at a time, while on a 12-triangle shoebox (a two-level tree) it is 10 % slower.
constexpr int kSpecMinTris = 64;
// quantised: walk the 48-byte nodes (variants for 4 and 6 blocks per SM), + 32.
inline int trace_variant(int blocks_per_sm, int traversal, int ntri, bool quantised = false) {
    // default: 6 blocks of 256 (40 registers) on the smaller quantised nodes (+2.5 % on a 20k-triangle
    // hall), 4 (64 registers) on 128-byte nodes (+23 %)
    const int minb = blocks_per_sm > 0 ? blocks_per_sm : (quantised ? 6 : 4);
    const bool spec = traversal == 2 || (traversal == 0 && ntri > kSpecMinTris);
    if (quantised) return 32 + (spec ? 16 : 0) + (minb >= 6 ? 6 : 4);
    if (spec) return 16 + (minb >= 6 ? 6 : 4);
    return minb;
}
// bvh_format of pach_trace_params: 0 default, 1 128-byte float nodes, 2 48-byte quantised nodes.
// The default walks quantised nodes above kQuantMinTris triangles: measured +6 % walk rate on a
// 20k-triangle hall and +8 % on a 500k-triangle arena (L1-bound walks), -37 % on a 12-triangle
// shoebox (a two-node tree: the decode costs, the smaller nodes save nothing).
constexpr int kQuantMinTris = 1024;
inline bool use_quantised_nodes(int bvh_format, int ntri) {
    return bvh_format == 2 || (bvh_format == 0 && ntri > kQuantMinTris);
}
cudaError_t launch_trace(const DevRun &r, int variant, int blocks, int threads, cudaStream_t s);
// fused: k_shade walks the rays itself (no k_trace launch) -- the default for scenes of at most
// kFuseMaxTris triangles, or traversal = 3
// map: also detect the run's mapping receivers (kernel variants compiled with the grid walk)
// wide: the shading variant with 4 blocks per SM, for rooms of at least kShadeWideReceivers receivers
constexpr int kShadeWideReceivers = 48;
cudaError_t launch_shade(const DevRun &r, int blocks, int threads, cudaStream_t s, bool fused = false, bool map = false,
                         bool wide = false);
// Room-acoustic parameters of n energy-time curves etc [n][T] x scale at fs Hz on the device (map_params.cu).
cudaError_t launch_map_params(const double *etc, int n, int T, double fs, double scale, int decay_depth,
                              double clarity_s, double *t_x, double *edt, double *clarity, double *definition,
                              double *sum, cudaStream_t s);
constexpr int kFuseMaxTris = 64;
inline bool fused_walk(int traversal, int ntri) { return traversal == 3 || (traversal == 0 && ntri <= kFuseMaxTris); }
cudaError_t wave_kernel_occupancy(int variant, int threads, int smem_shade, int *bpsm_trace, int *bpsm_shade,
                                  bool fused = false, bool wide = false);
cudaError_t launch_paths(const DevScene &S, int n, const double *o, const double *d, int max_bounces, int *poly,
                         double *t, double *pts, cudaStream_t s);
cudaError_t launch_emit(const DevRun &r, long long p0, int n, double *out, cudaStream_t s);
cudaError_t launch_prop_sample(const DevRun &r, long long p0, int n, float *dirs, float *weights, cudaStream_t s);
cudaError_t launch_direct(const DevScene &S, const double *src, int nsrc, const double *rec, int nrec, int max_cross,
                          int *valid, double *transmod, cudaStream_t s);

// Convergence mode (rayCount < 1, convergence.cpp): one of the reference's convergence checks on one
// receiver's cumulative raw histograms of band h_oct (energy, and the three Reflection_Analysis_Data
// kinds); check() is its Check() after each revolution.
struct ConvCheck {
    int mode = -1;            // 0 SpecMin_Convergence_Check (rayCount == 0), 1 Minimum_Convergence_Check (< 0)
    int row = -1;             // histogram row of the receiver
    int T = 0, fs = 1000;
    int s_start = 0, s50 = 0, s80 = 0, s_inf = 0;   // Minimum: sample windows
    double snap50 = 0, snap80 = 0, snapinf = 0;
    int step = 0, binct = 0;  // SpecMin: 50 ms blocks
    long long rayct = 0, nmin = 0;
    std::vector<double> snapshot;
    int count = 0;
    std::vector<double> E, A0, A1, A2;  // [T] energy; specular, diffuse, specular-after-scatter
    bool check();
};
void conv_setup(ConvCheck &c, int mode, int row, double dist_m, double c_mps, int fs, int T);
void pick_conv_receivers(const HostScene &hs, const double src[3], const pach_receiver_desc *rec, int R, int rows[2],
                         double dist[2]);
// Per-revolution capture of the two check receivers, [kConvChunk revolutions][2][4][T] doubles.
constexpr int kConvChunk = 64;       // revolutions traced per device loop at most
constexpr int kConvKinds = 4;        // energy, analysis 0..2

// capi.cpp: read access to a scene handle (for entry points in other translation units)
const HostScene *scene_host(const pach_scene *s);
const DevScene *scene_dev(const pach_scene *s);
int scene_device(const pach_scene *s);
void set_last_error(const char *msg);
// argument checks of the tracing entry points (who prefixes the message, e.g. "room 3: ")
pach_status check_common(const pach_trace_params &p);
pach_status check_room(const pach_source_desc *sources, int32_t n_sources, const pach_receiver_desc *receivers,
                       int32_t n_receivers, const std::string &who);

// filters.cu: receiver filters (ETCToFilter of the band pressures and of P Dir / E) on the device.
// kinds 1 (pressure) or 7 (pressure, then -x +x -y +y -z +z from Dir_Rec_Neg / Dir_Rec_Pos); cut 0 or
// 4096 samples; scale [R] multiplies each receiver's envelopes (NULL: 1); asynchronous on st.
size_t filters_workspace_bytes(int n_filters, int T);
pach_status filters_device(const double *E, const double *P, const double *Dp, const double *Dn, const double *scale,
                           int R, int T, int kinds, int fs, const double *swl, int cut, double *out, void *ws,
                           size_t ws_bytes, cudaStream_t st);

// scene.cpp
bool build_host_scene(const pach_scene_desc *d, HostScene &hs, std::string &err);
void medium_properties(double temp_c, double hr, double pa_hpa, int air_choice, int edge, double atten[kBands],
                       double *c, double *rho);
constexpr int kThirdOctaveBands = 23;  // the reference's third-octave table (50 Hz .. 10 kHz without 2500 Hz)
extern const double kThirdOctaveCentres[kThirdOctaveBands];
void medium_attenuation_third_octave(double temp_c, double hr, double pa_hpa, int air_choice, int edge,
                                     double atten[kThirdOctaveBands]);
void geodesic_faces(std::vector<double> &faces);  // [80][3][3]
void geodesic_faces_fixed(double out[kGeoFaces * 9]);
unsigned long long derived_broadband_bound(const HostScene &hs, int h_oct, bool pure_specular);
// Host walk of hs.bvh with the device's box test and FP64 triangle tests (t > t_min).
bool bvh_shoot_host(const HostScene &hs, const double o[3], const double d[3], double t_min, int &tri, double &t);

}  // namespace pach
