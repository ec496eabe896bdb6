// engine.h -- internal structures shared by the host side (scene build, C ABI) and the kernels.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/pach_gpu.h"

namespace pach {

constexpr int kBands = 8;
constexpr int kMaxSources = 64;
constexpr int kGeoFaces = 80;

// Host-side prepared scene (FP64 master copy + FP32 device layout sources).
struct HostScene {
    int npoly = 0, ntri = 0;
    std::vector<double> tri64;       // [ntri][9]: v0, e1, e2
    std::vector<int32_t> tri_poly;   // [ntri]
    std::vector<int32_t> tri_plane;  // [ntri] coplanar group id
    std::vector<double> normal;      // [npoly][3]
    std::vector<double> area;        // [npoly]
    std::vector<double> alpha, scat, trans;  // [npoly][8]
    bool has_trans = false;
    double bmin[3], bmax[3];
    int dims[3];
    std::vector<uint32_t> cell_start;  // [ncell+1]
    std::vector<uint32_t> cell_tris;
    double c = 343, rho = 1.2, rho_c = 411.6, atten[kBands] = {0};
    double scale = 1;                // largest box extent
};

// Device scene view (passed by value to kernels).
struct DevScene {
    const float4 *tri;          // [ntri*3]: (v0, plane bits) (e1, poly bits) (e2, 0)
    const double *tri64;        // [ntri*9]
    const float4 *pnormal;      // [npoly]
    const float4 *mat;          // [npoly*8]: (1-alpha, s_lo, s_mid, s_hi)
    const float *trans;         // [npoly*8]
    const uint32_t *cell_start; // [ncell+1]
    const uint32_t *cell_tris;
    int nx, ny, nz, ntri;
    float bminx, bminy, bminz;
    float cellx, celly, cellz;
    float icellx, icelly, icellz;
    float bmaxx, bmaxy, bmaxz;
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
    uint32_t meta;              // bits 0-2 band, 3-4 Scatter_Mask, 5 phase (0 B, 1 C)
    int32_t plane;              // coplanar group of the surface the ray leaves (-1 none)
};

// Counters accumulated by the kernels (one instance in device memory).
struct DevCounters {
    unsigned long long primaries, seg_broad, seg_b, seg_c, octave_rays, end_traces, detections, capped,
        retests, queue_overflow, stack_spills, lost_items;
    double lost_energy, initial_energy;
};

// Launch-wide parameters (kernel argument).
struct DevRun {
    DevScene S;
    // receivers
    const float4 *rec;          // [R] (x, y, z, r^2)
    int R, T;
    double fs;                  // histogram rate (Hz)
    float inv_c;
    double inv_c_d;
    float atten_k[kBands];      // exp2 factor per second of travel: -0.1 log2(10) m c
    float rho_c;
    double cotime;
    // sources
    int nsrc;
    const float4 *src;          // [nsrc] origin (w = kind)
    const float *e0;            // [nsrc*8] band powers (W)
    const float4 *geo;          // [80*3] geodesic face vertices
    const double *prim_dirs;    // optional, indexed by prim - prim_base
    const double *prim_weights;
    long long prim_base;
    int h_oct, oct_lo, oct_hi, is_order, pure_specular, max_broad;
    unsigned long long seed;
    long long max_seg;
    // outputs
    double *hE, *hP, *hDp, *hDn, *hAn;
    DevCounters *cnt;
    // queues
    ORayItem *q_in;             // input of the octave kernel
    const unsigned long long *q_in_count;
    unsigned long long q_in_cap;
    unsigned long long *q_in_head;
    ORayItem *q_out;            // spill / phase-A output
    unsigned long long *q_out_count;
    unsigned long long q_out_cap;
};

// trace.cu entry points (host wrappers)
cudaError_t launch_broadband(const DevRun &r, long long p0, long long p1, int blocks, int threads, cudaStream_t s);
cudaError_t launch_octave(const DevRun &r, int blocks, int threads, cudaStream_t s);
cudaError_t launch_paths(const DevScene &S, int n, const double *o, const double *d, int max_bounces, int *poly,
                         double *t, double *pts, cudaStream_t s);
cudaError_t launch_emit(const DevRun &r, long long p0, int n, double *out, cudaStream_t s);
cudaError_t octave_kernel_occupancy(int threads, int *blocks_per_sm);

// scene.cpp
bool build_host_scene(const pach_scene_desc *d, HostScene &hs, std::string &err);
void medium_properties(double temp_c, double hr, double pa_hpa, int air_choice, int edge, double atten[kBands],
                       double *c, double *rho);
void geodesic_faces(std::vector<double> &faces);  // [80][3][3]
unsigned long long derived_broadband_bound(const HostScene &hs, int h_oct, bool pure_specular);

}  // namespace pach
