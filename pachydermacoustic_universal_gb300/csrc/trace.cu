// trace.cu -- sm_103a kernels of the stochastic split ray tracer.
//
// Hot path of SplitRayTracer.cast_ray_distributed / End_Trace ("Classes_Complete_Trace -
// TaskAll.cs":335-536) on the GPU:
//   k_broadband  phase A: one thread per primary ray -- emission (Classes_Sources.cs:256-265,
//                390-403), grid traversal, broadband receiver detection (Classes_Receivers.cs:803-829),
//                absorption (Classes_Materials.cs:166-178) and Scatter_Early (4498-4570); the band
//                children of every bounce and the final split go to a device queue.
//   k_octave     phases B and C: a persistent kernel whose threads pull octave rays from the queue
//                (warp-aggregated tickets) and advance one bounce per loop iteration, so that every
//                lane of a warp traverses in lock-step whatever phase its ray is in (Scatter_Late
//                4629-4701, Scatter_VeryLate 4572-4627, Spherical_Receiver.CheckRay 837-877).
//                Scatter_Late's specular children go to a per-thread stack: the lower-energy branch
//                continues and the other is pushed, which keeps the depth near log2 of the subtree;
//                a full stack spills to a device queue that the host drains with another launch.
// Geometry is FP32 (Moller-Trumbore) with an FP64 re-test of candidates whose barycentric margin
// lies in an epsilon band or whose determinant is near grazing.  Histograms accumulate in FP64 with
// global atomics.  Random numbers: Philox4x32-10 keyed by (seed, primary, stream id, block) -- the
// streams the CPU oracle draws -- so a ray's decisions do not depend on scheduling.
#include <cfloat>
#include <cstdint>

#include "engine.h"

namespace pach {
namespace {

constexpr int kStack = 16;
constexpr float kInvPi = 0.318309886183790671538f;
constexpr float kBaryEps = 2e-5f;
constexpr float kTP1 = 1e-2f;                  // TaskAll:351
constexpr float kTP2 = 3.16227766016837933e-5f;  // 10^-4.5, TaskAll:331, 355
constexpr float kTP3 = 1e-9f;                  // TaskAll:356

// ------------------------------------------------------------------------------------------
// RNG (Philox4x32-10, Salmon et al. SC'11) and stream identities
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ uint4 philox(uint4 c, uint32_t k0, uint32_t k1) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r) { k0 += W0; k1 += W1; }
        const uint32_t hi0 = __umulhi(M0, c.x), lo0 = M0 * c.x;
        const uint32_t hi1 = __umulhi(M1, c.z), lo1 = M1 * c.z;
        c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
    }
    return c;
}

__device__ __forceinline__ float u24(uint32_t x) { return (float)(x >> 8) * (1.0f / 16777216.0f); }

__device__ __forceinline__ float4 draw(unsigned long long seed, uint32_t prim, unsigned long long sid, uint32_t b) {
    const uint4 c = philox(make_uint4(b, prim, (uint32_t)sid, (uint32_t)(sid >> 32)), (uint32_t)seed,
                           (uint32_t)(seed >> 32));
    return make_float4(u24(c.x), u24(c.y), u24(c.z), u24(c.w));
}

__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__device__ __forceinline__ unsigned long long sid_early(int k, int o, int q) {
    return (1ull << 62) | ((unsigned long long)k << 5) | ((unsigned long long)o << 2) | (unsigned long long)q;
}
__device__ __forceinline__ unsigned long long sid_final(int o) { return (2ull << 62) | (unsigned long long)o; }
__device__ __forceinline__ unsigned long long sid_late(unsigned long long parent, uint32_t nb) {
    return (3ull << 62) |
           (mix64(parent + 0x9E3779B97F4A7C15ull * (unsigned long long)(nb + 1)) & ((1ull << 62) - 1));
}

// ------------------------------------------------------------------------------------------
// small vector helpers
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ float3 f3(float4 a) { return make_float3(a.x, a.y, a.z); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator*(float3 a, float s) { return make_float3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float dot3(float3 a, float3 b) { return fmaf(a.x, b.x, fmaf(a.y, b.y, a.z * b.z)); }
__device__ __forceinline__ float3 cross3(float3 a, float3 b) {
    return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float3 unit3(float3 a) { return a * rsqrtf(dot3(a, a)); }

// Uniform-hemisphere direction about n (Lambert_Scattering, Classes_Materials.cs:4521-4552): frame
// z = n, x from (0,0,1) unless |n.z| in (0.99, 1.01) then (1,0,0); azimuth 2 pi U1; cos(zenith) = U2.
__device__ __forceinline__ float3 lambert(float3 n, float U1, float U2) {
    float3 dx = make_float3(0.f, 0.f, 1.f);
    const float proj = fabsf(n.z);
    if (0.99f < proj && proj < 1.01f) dx = make_float3(1.f, 0.f, 0.f);
    float3 dy = cross3(n, dx);
    dx = cross3(dy, n);
    dx = unit3(dx);
    dy = unit3(dy);
    float s, c;
    sincospif(2.0f * U1, &s, &c);
    const float sz = sqrtf(fmaxf(0.f, 1.f - U2 * U2));
    return unit3(dx * (c * sz) + dy * (s * sz) + n * U2);
}

// ------------------------------------------------------------------------------------------
// geometry
// ------------------------------------------------------------------------------------------
// FP64 re-test of triangle i (the FP32 ray converted exactly).
__device__ __noinline__ bool retest64(const DevScene &S, int i, float3 of, float3 df, double &t) {
    const double *T = S.tri64 + 9 * (size_t)i;
    const double ox = of.x, oy = of.y, oz = of.z, dx = df.x, dy = df.y, dz = df.z;
    const double e1x = T[3], e1y = T[4], e1z = T[5], e2x = T[6], e2y = T[7], e2z = T[8];
    const double px = dy * e2z - dz * e2y, py = dz * e2x - dx * e2z, pz = dx * e2y - dy * e2x;
    const double det = e1x * px + e1y * py + e1z * pz;
    if (det == 0.0) return false;
    const double inv = 1.0 / det;
    const double sx = ox - T[0], sy = oy - T[1], sz = oz - T[2];
    const double u = (sx * px + sy * py + sz * pz) * inv;
    if (u < 0.0 || u > 1.0) return false;
    const double qx = sy * e1z - sz * e1y, qy = sz * e1x - sx * e1z, qz = sx * e1y - sy * e1x;
    const double v = (dx * qx + dy * qy + dz * qz) * inv;
    if (v < 0.0 || u + v > 1.0) return false;
    t = (e2x * qx + e2y * qy + e2z * qz) * inv;
    return true;
}

// Nearest hit along o + t d with t > t_eps, skipping triangles of plane `skip` (the surface the ray
// leaves).  Uniform-grid DDA; a candidate is accepted once the walk has passed its distance.
__device__ __forceinline__ bool trace_ray(const DevScene &S, float3 o, float3 d, int skip, float &t_best,
                                          int &tri_best, unsigned long long &retests) {
    const float idx_ = 1.0f / d.x, idy_ = 1.0f / d.y, idz_ = 1.0f / d.z;
    float rx = (o.x - S.bminx) * S.icellx, ry = (o.y - S.bminy) * S.icelly, rz = (o.z - S.bminz) * S.icellz;
    if (rx < 0.f || ry < 0.f || rz < 0.f || rx >= (float)S.nx || ry >= (float)S.ny || rz >= (float)S.nz) {
        // origin outside the grid: clip to the box (Hare OBox.Intersect)
        const float tx1 = (S.bminx - o.x) * idx_, tx2 = (S.bmaxx - o.x) * idx_;
        const float ty1 = (S.bminy - o.y) * idy_, ty2 = (S.bmaxy - o.y) * idy_;
        const float tz1 = (S.bminz - o.z) * idz_, tz2 = (S.bmaxz - o.z) * idz_;
        const float tn = fmaxf(fmaxf(fminf(tx1, tx2), fminf(ty1, ty2)), fminf(tz1, tz2));
        const float tf = fminf(fminf(fmaxf(tx1, tx2), fmaxf(ty1, ty2)), fmaxf(tz1, tz2));
        if (!(tn <= tf) || tf < 0.f) return false;
        const float t0 = fmaxf(tn, 0.f);
        rx = (o.x + d.x * t0 - S.bminx) * S.icellx;
        ry = (o.y + d.y * t0 - S.bminy) * S.icelly;
        rz = (o.z + d.z * t0 - S.bminz) * S.icellz;
    }
    int ix = min(max((int)floorf(rx), 0), S.nx - 1);
    int iy = min(max((int)floorf(ry), 0), S.ny - 1);
    int iz = min(max((int)floorf(rz), 0), S.nz - 1);
    const int sx = d.x < 0.f ? -1 : 1, sy = d.y < 0.f ? -1 : 1, sz = d.z < 0.f ? -1 : 1;
    float tmx = d.x != 0.f ? (S.bminx + (float)(ix + (sx > 0)) * S.cellx - o.x) * idx_ : FLT_MAX;
    float tmy = d.y != 0.f ? (S.bminy + (float)(iy + (sy > 0)) * S.celly - o.y) * idy_ : FLT_MAX;
    float tmz = d.z != 0.f ? (S.bminz + (float)(iz + (sz > 0)) * S.cellz - o.z) * idz_ : FLT_MAX;
    const float tdx = d.x != 0.f ? S.cellx * fabsf(idx_) : FLT_MAX;
    const float tdy = d.y != 0.f ? S.celly * fabsf(idy_) : FLT_MAX;
    const float tdz = d.z != 0.f ? S.cellz * fabsf(idz_) : FLT_MAX;
    float best = FLT_MAX;
    int bi = -1;
    const int max_steps = S.nx + S.ny + S.nz + 3;
    for (int step = 0; step < max_steps; ++step) {
        const uint32_t cell = ((uint32_t)iz * S.ny + iy) * S.nx + ix;
        const uint32_t beg = __ldg(S.cell_start + cell), end = __ldg(S.cell_start + cell + 1);
        for (uint32_t k = beg; k < end; ++k) {
            const int i = (int)__ldg(S.cell_tris + k);
            const float4 A = __ldg(S.tri + 3 * i);
            if (__float_as_int(A.w) == skip) continue;
            const float4 B = __ldg(S.tri + 3 * i + 1);
            const float4 C = __ldg(S.tri + 3 * i + 2);
            const float3 e1 = f3(B), e2 = f3(C);
            const float3 p = cross3(d, e2);
            const float det = dot3(e1, p);
            const float3 s = o - f3(A);
            const float inv = 1.0f / det;
            const float u = dot3(s, p) * inv;
            const float3 q = cross3(s, e1);
            const float v = dot3(d, q) * inv;
            const float t = dot3(e2, q) * inv;
            const float margin = fminf(fminf(u, v), 1.0f - u - v);
            if (fabsf(det) < C.w || !(fabsf(margin) > kBaryEps)) {
                // near grazing, near an edge, or not finite: decide in FP64
                double td;
                ++retests;
                if (retest64(S, i, o, d, td)) {
                    const float tf = (float)td;
                    if (tf > S.t_eps && tf < best) { best = tf; bi = i; }
                }
            } else if (margin > 0.f && t > S.t_eps && t < best) {
                best = t;
                bi = i;
            }
        }
        const float texit = fminf(fminf(tmx, tmy), tmz);
        if (best <= texit) break;
        if (tmx < tmy) {
            if (tmx < tmz) { ix += sx; if (ix < 0 || ix >= S.nx) break; tmx += tdx; }
            else { iz += sz; if (iz < 0 || iz >= S.nz) break; tmz += tdz; }
        } else {
            if (tmy < tmz) { iy += sy; if (iy < 0 || iy >= S.ny) break; tmy += tdy; }
            else { iz += sz; if (iz < 0 || iz >= S.nz) break; tmz += tdz; }
        }
    }
    if (bi < 0) return false;
    t_best = best;
    tri_best = bi;
    return true;
}

// ------------------------------------------------------------------------------------------
// receivers
// ------------------------------------------------------------------------------------------
// Sphere test of segment [o, o + tseg d] (Classes_Receivers.cs:839-849).  The discriminant is
// formed as r^2 - |m - b d|^2 (equal to b^2 - c for a unit d) to avoid cancellation in FP32.
__device__ __forceinline__ bool sphere_hit(float4 c, float3 o, float3 d, float tseg, float &t, float &half) {
    const float3 m = make_float3(o.x - c.x, o.y - c.y, o.z - c.z);
    const float b = dot3(m, d);
    const float cc = dot3(m, m) - c.w;
    if (cc > 0.f && b > 0.f) return false;
    const float3 perp = m - d * b;
    const float disc = c.w - dot3(perp, perp);
    if (disc < 0.f) return false;
    t = -b;  // chord midpoint (t1 + t2) / 2
    if (!(t > 0.f && t < tseg)) return false;
    half = sqrtf(disc);  // (t2 - t1) / 2
    return true;
}

// Directional_Histogram.Add (Classes_Receivers.cs:1813-1825) + Reflection_Analysis_Data.
__device__ __forceinline__ void hist_add(const DevRun &r, int k, int oct, long long bin, float e, float3 d, int kind) {
    const size_t base = ((size_t)k * kBands + oct) * r.T + bin;
    atomicAdd(r.hE + base, (double)e);
    atomicAdd(r.hP + base, (double)sqrtf(e * r.rho_c));
    const float ca[3] = {-d.x, -d.y, -d.z};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const size_t j = (((size_t)k * 3 + a) * kBands + oct) * r.T + bin;
        atomicAdd((ca[a] > 0.f ? r.hDp : r.hDn) + j, (double)(ca[a] * e));
    }
    atomicAdd(r.hAn + (((size_t)k * 3 + kind) * kBands + oct) * r.T + bin, (double)e);
}

// Spherical_Receiver.CheckRay (Classes_Receivers.cs:837-877): energy I 10^(-0.1 m c time) / pi * half.
__device__ __forceinline__ uint32_t detect_octave(const DevRun &r, const float4 *rec, float3 o, float3 d, float tseg,
                                                  double t_sum, float Iabs, int oct, int mask) {
    uint32_t n = 0;
    for (int k = 0; k < r.R; ++k) {
        float t, half;
        if (!sphere_hit(rec[k], o, d, tseg, t, half)) continue;
        ++n;
        const double time = t_sum + (double)(t * r.inv_c);
        const long long bin = (long long)(time * r.fs);
        if (!(time >= 0.0) || bin < 0 || bin >= r.T) continue;
        const float e = Iabs * exp2f(r.atten_k[oct] * (float)time) * kInvPi * half;
        hist_add(r, k, oct, bin, e, d, (mask & 1) ? 1 : ((mask & 2) ? 2 : 0));
    }
    return n;
}

// Spherical_Receiver.CheckBroadbandRay (Classes_Receivers.cs:803-829): every band of the range,
// analysis bin 0 (specular).
__device__ __forceinline__ uint32_t detect_broad(const DevRun &r, const float4 *rec, float3 o, float3 d, float tseg,
                                                 double t_sum, const float (&E)[kBands], const float (&sc)[kBands]) {
    uint32_t n = 0;
    for (int k = 0; k < r.R; ++k) {
        float t, half;
        if (!sphere_hit(rec[k], o, d, tseg, t, half)) continue;
        ++n;
        const double time = t_sum + (double)(t * r.inv_c);
        const long long bin = (long long)(time * r.fs);
        if (!(time >= 0.0) || bin < 0 || bin >= r.T) continue;
#pragma unroll
        for (int oct = 0; oct < kBands; ++oct) {
            if (oct < r.oct_lo || oct > r.oct_hi) continue;
            const float e = E[oct] * sc[oct] * exp2f(r.atten_k[oct] * (float)time) * kInvPi * half;
            hist_add(r, k, oct, bin, e, d, 0);
        }
    }
    return n;
}

// ------------------------------------------------------------------------------------------
// emission
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ float3 emit_dir(const DevRun &r, long long prim, int kind) {
    const float4 U = draw(r.seed, (uint32_t)prim, 0ull, 0u);
    if (kind == PACH_SOURCE_RANDOM) {  // RandomSource (Classes_Sources.cs:256-265)
        float st, ct, sp, cp;
        sincospif(2.0f * U.x, &st, &ct);
        sincospif(2.0f * U.y, &sp, &cp);
        return make_float3(st * cp, st * sp, ct);
    }
    if (kind == PACH_SOURCE_UNIFORM) {
        const float z = 1.0f - 2.0f * U.x;
        const float rr = sqrtf(fmaxf(0.f, 1.f - z * z));
        float sp, cp;
        sincospif(2.0f * U.y, &sp, &cp);
        return make_float3(rr * cp, rr * sp, z);
    }
    // GeodesicSource (Classes_Sources.cs:390-403): face (per-source ray count) mod 80, point on face
    const long long j = prim / r.nsrc;
    const int f = (int)(j % kGeoFaces);
    float u = U.x, v = U.y;
    if (u + v > 1.f) { u = 1.f - u; v = 1.f - v; }
    const float3 a = f3(r.geo[3 * f]), b = f3(r.geo[3 * f + 1]), c = f3(r.geo[3 * f + 2]);
    return unit3(a + (b - a) * u + (c - a) * v);
}

// ------------------------------------------------------------------------------------------
// queue items
// ------------------------------------------------------------------------------------------
struct Ray {
    float3 p, d;
    float I, scale;
    double t_sum;
    uint32_t prim, nb;
    unsigned long long sid;
    int oct, mask, phase, plane;
};

__device__ __forceinline__ ORayItem to_item(const Ray &R) {
    ORayItem it;
    it.px = R.p.x; it.py = R.p.y; it.pz = R.p.z; it.I = R.I;
    it.dx = R.d.x; it.dy = R.d.y; it.dz = R.d.z; it.scale = R.scale;
    it.t_sum = R.t_sum; it.prim = R.prim; it.nb = R.nb; it.sid = R.sid;
    it.meta = (uint32_t)R.oct | ((uint32_t)R.mask << 3) | ((uint32_t)R.phase << 5);
    it.plane = R.plane;
    return it;
}

__device__ __forceinline__ Ray to_ray(const ORayItem &it) {
    Ray R;
    R.p = make_float3(it.px, it.py, it.pz);
    R.d = make_float3(it.dx, it.dy, it.dz);
    R.I = it.I; R.scale = it.scale; R.t_sum = it.t_sum; R.prim = it.prim; R.nb = it.nb; R.sid = it.sid;
    R.oct = (int)(it.meta & 7u); R.mask = (int)((it.meta >> 3) & 3u); R.phase = (int)((it.meta >> 5) & 1u);
    R.plane = it.plane;
    return R;
}

__device__ __forceinline__ Ray new_ray(float3 p, float3 d, float I, float scale, double t_sum, uint32_t prim,
                                       unsigned long long sid, int oct, int mask, int plane) {
    Ray R;
    R.p = p; R.d = d; R.I = I; R.scale = scale; R.t_sum = t_sum; R.prim = prim; R.nb = 0; R.sid = sid;
    R.oct = oct; R.mask = mask; R.phase = 0; R.plane = plane;
    return R;
}

__device__ __forceinline__ void store_item(ORayItem *q, unsigned long long slot, const ORayItem &it) {
    float4 *dst = reinterpret_cast<float4 *>(q + slot);
    const float4 *src = reinterpret_cast<const float4 *>(&it);
    dst[0] = src[0]; dst[1] = src[1]; dst[2] = src[2]; dst[3] = src[3];
}

__device__ __forceinline__ ORayItem load_item(const ORayItem *q, unsigned long long i) {
    const float4 *s = reinterpret_cast<const float4 *>(q + i);
    ORayItem it;
    float4 *d = reinterpret_cast<float4 *>(&it);
    d[0] = __ldcs(s); d[1] = __ldcs(s + 1); d[2] = __ldcs(s + 2); d[3] = __ldcs(s + 3);
    return it;
}

// ------------------------------------------------------------------------------------------
// counters
// ------------------------------------------------------------------------------------------
struct LocalCounters {
    unsigned long long v[11] = {0};  // prim, seg_broad, seg_b, seg_c, oct, end_traces, det, capped, retests, overflow, spills
    double lost = 0, init = 0;
};
enum { C_PRIM, C_SEGA, C_SEGB, C_SEGC, C_OCT, C_END, C_DET, C_CAP, C_RET, C_OVF, C_SPILL };

__device__ void flush_counters(const DevRun &r, const LocalCounters &L) {
    __shared__ unsigned long long s_u[11];
    __shared__ double s_d[2];
    if (threadIdx.x < 11) s_u[threadIdx.x] = 0;
    if (threadIdx.x < 2) s_d[threadIdx.x] = 0;
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 11; ++i)
        if (L.v[i]) atomicAdd(&s_u[i], L.v[i]);
    if (L.lost != 0) atomicAdd(&s_d[0], L.lost);
    if (L.init != 0) atomicAdd(&s_d[1], L.init);
    __syncthreads();
    if (threadIdx.x == 0) {
        DevCounters *c = r.cnt;
        unsigned long long *dst[11] = {&c->primaries, &c->seg_broad, &c->seg_b, &c->seg_c, &c->octave_rays,
                                       &c->end_traces, &c->detections, &c->capped, &c->retests, &c->queue_overflow,
                                       &c->stack_spills};
        for (int i = 0; i < 11; ++i)
            if (s_u[i]) atomicAdd(dst[i], s_u[i]);
        if (s_d[0] != 0) atomicAdd(&c->lost_energy, s_d[0]);
        if (s_d[1] != 0) atomicAdd(&c->initial_energy, s_d[1]);
    }
}

__device__ __forceinline__ void load_receivers(const DevRun &r, float4 *rec) {
    for (int i = threadIdx.x; i < r.R; i += blockDim.x) rec[i] = r.rec[i];
    __syncthreads();
}

// ------------------------------------------------------------------------------------------
// phase A: broadband rays (cast_ray_distributed, TaskAll:347-424)
// ------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_broadband(DevRun r, long long p0, long long p1) {
    extern __shared__ float4 s_rec[];
    load_receivers(r, s_rec);
    LocalCounters L;
    const DevScene &S = r.S;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long prim = p0 + (long long)blockIdx.x * blockDim.x + threadIdx.x; prim < p1; prim += stride) {
        const int s = (int)((prim + 1) % r.nsrc);  // SourceCluster round robin (Classes_Sources.cs:712-722)
        const float4 src = r.src[s];
        float3 d;
        float w = 1.f;
        if (r.prim_dirs) {
            const double *pd = r.prim_dirs + 3 * (prim - r.prim_base);
            d = make_float3((float)pd[0], (float)pd[1], (float)pd[2]);
        } else {
            d = emit_dir(r, prim, (int)src.w);
        }
        if (r.prim_weights) w = (float)r.prim_weights[prim - r.prim_base];
        float E[kBands], sc[kBands];
#pragma unroll
        for (int o = 0; o < kBands; ++o) {
            E[o] = 1.f;
            sc[o] = r.e0[s * kBands + o] * w;
            L.init += (double)sc[o];
        }
        float3 pos = f3(src);
        double t_sum = 0.0;
        int order = 0, plane = -1;
        bool lost = false;
        float eh;
        do {
            float t;
            int tri;
            const bool hit = trace_ray(S, pos, d, plane, t, tri, L.v[C_RET]);
            ++L.v[C_SEGA];
            if (!hit) {
                if (order > r.is_order) L.v[C_DET] += detect_broad(r, s_rec, pos, d, 1e6f, t_sum, E, sc);
#pragma unroll
                for (int o = 0; o < kBands; ++o) L.lost += (double)(E[o] * sc[o]);
                lost = true;
                break;
            }
            if (order > r.is_order) L.v[C_DET] += detect_broad(r, s_rec, pos, d, t, t_sum, E, sc);
            t_sum += (double)t * r.inv_c_d;
            pos = pos + d * t;
            const float4 A = __ldg(S.tri + 3 * tri), B = __ldg(S.tri + 3 * tri + 1);
            plane = __float_as_int(A.w);
            const int poly = __float_as_int(B.w);
            const int k = order++;
            float3 n = f3(__ldg(S.pnormal + poly));
            float cos_t = dot3(d, n);
            float smid[kBands], tau[kBands];
#pragma unroll
            for (int o = 0; o < kBands; ++o) {
                const float4 m = __ldg(S.mat + poly * kBands + o);
                E[o] *= m.x;  // Basic_Material.Absorb
                smid[o] = r.pure_specular ? 0.f : m.z;
                tau[o] = (S.has_trans && !r.pure_specular) ? __ldg(S.trans + poly * kBands + o) : 0.f;
            }
            // Scatter_Early
            if (cos_t > 0.f) { n = n * -1.f; cos_t = -cos_t; }
            int nchild = 0;
#pragma unroll
            for (int o = 0; o < kBands; ++o) nchild += (E[o] != 0.f) ? (tau[o] > 0.f ? 3 : 1) : 0;
            unsigned long long slot = 0;
            bool room = false;
            if (nchild) {
                slot = atomicAdd(r.q_out_count, (unsigned long long)nchild);
                room = slot + nchild <= r.q_out_cap;
                if (!room) ++L.v[C_OVF];
            }
#pragma unroll
            for (int o = 0; o < kBands; ++o) {
                if (E[o] == 0.f) continue;
                Ray ch = new_ray(pos, d, E[o] * smid[o], sc[o], t_sum, (uint32_t)prim, sid_early(k, o, 0), o, 3, plane);
                E[o] *= (1.f - smid[o]);
                const float4 U = draw(r.seed, (uint32_t)prim, ch.sid, 0u);
                ch.d = lambert(n, U.x, U.y);
                if (tau[o] > 0.f) {
                    const Ray tr = new_ray(pos, d, E[o] * tau[o], sc[o], t_sum, (uint32_t)prim, sid_early(k, o, 1), o, 0, plane);
                    E[o] *= (1.f - tau[o]);
                    Ray td = ch;
                    td.I = ch.I * tau[o];
                    ch.I *= (1.f - tau[o]);
                    td.d = ch.d * -1.f;
                    td.sid = sid_early(k, o, 2);
                    if (room) { store_item(r.q_out, slot++, to_item(tr)); store_item(r.q_out, slot++, to_item(td)); }
                    L.v[C_OCT] += 2;
                }
                if (room) store_item(r.q_out, slot++, to_item(ch));
                ++L.v[C_OCT];
            }
            d = d - n * (2.f * cos_t);
            eh = 0.f;
#pragma unroll
            for (int o = 0; o < kBands; ++o) eh = (o == r.h_oct) ? E[o] : eh;
            if (order >= r.max_broad && eh > kTP1) { ++L.v[C_CAP]; break; }
        } while (eh > kTP1);
        if (!lost) {
            const int nfin = r.oct_hi - r.oct_lo + 1;
            unsigned long long slot = atomicAdd(r.q_out_count, (unsigned long long)nfin);
            const bool room = slot + nfin <= r.q_out_cap;
            if (!room) ++L.v[C_OVF];
#pragma unroll
            for (int o = 0; o < kBands; ++o) {
                if (o < r.oct_lo || o > r.oct_hi) continue;
                const Ray it = new_ray(pos, d, E[o], sc[o], t_sum, (uint32_t)prim, sid_final(o), o, 0, plane);
                if (room) store_item(r.q_out, slot++, to_item(it));
                ++L.v[C_OCT];
            }
        }
        ++L.v[C_PRIM];
    }
    flush_counters(r, L);
}

// ------------------------------------------------------------------------------------------
// phases B and C: octave rays (TaskAll:429-536)
// ------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_octave(DevRun r) {
    extern __shared__ float4 s_rec[];
    load_receivers(r, s_rec);
    LocalCounters L;
    const DevScene &S = r.S;
    const unsigned long long n_in = min(*r.q_in_count, r.q_in_cap);
    ORayItem stack[kStack];
    int sp = 0;
    bool have = false;
    Ray R;
    const int lane = threadIdx.x & 31;
    while (true) {
        // ---- acquire work: own stack first, then the shared queue (one ticket atomic per warp) ----
        const unsigned act = __activemask();
        const bool need = !have && sp == 0;
        const unsigned want = __ballot_sync(act, need);
        if (want) {
            const int leader = __ffs(want) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(r.q_in_head, (unsigned long long)__popc(want));
            base = __shfl_sync(act, base, leader);
            if (need) {
                const unsigned long long idx = base + __popc(want & ((1u << lane) - 1u));
                if (idx >= n_in) break;
                R = to_ray(load_item(r.q_in, idx));
                have = true;
            }
        }
        if (!have) {
            R = to_ray(stack[--sp]);
            have = true;
        }
        // ---- one bounce ----
        float t;
        int tri;
        const bool hit = trace_ray(S, R.p, R.d, R.plane, t, tri, L.v[C_RET]);
        ++L.v[R.phase == 0 ? C_SEGB : C_SEGC];
        L.v[C_DET] += detect_octave(r, s_rec, R.p, R.d, hit ? t : 1e6f, R.t_sum, R.I * R.scale, R.oct, R.mask);
        if (!hit) {  // lost ray: no End_Trace after a miss in phase B (TaskAll:437-443)
            L.lost += (double)(R.I * R.scale);
            have = false;
            continue;
        }
        R.t_sum += (double)t * r.inv_c_d;
        R.p = R.p + R.d * t;
        const float4 A = __ldg(S.tri + 3 * tri), B = __ldg(S.tri + 3 * tri + 1);
        R.plane = __float_as_int(A.w);
        const int poly = __float_as_int(B.w);
        const float3 n = f3(__ldg(S.pnormal + poly));
        const float cos_t = dot3(n, R.d);
        const float4 m = __ldg(S.mat + poly * kBands + R.oct);  // (1-alpha, s_lo, s_mid, s_hi)
        R.I *= m.x;
        const float4 U = draw(r.seed, R.prim, R.sid, 1u + R.nb);
        const uint32_t nb = R.nb++;
        const bool transmit = S.has_trans && !r.pure_specular && U.x < __ldg(S.trans + poly * kBands + R.oct);
        const float3 spec = R.d - n * (2.f * cos_t);
        const float3 nn = cos_t > 0.f ? n * -1.f : n;
        bool test_loop = true;
        if (R.phase == 0) {
            // Scatter_Late
            if (r.pure_specular || U.y > m.w) {
                R.d = transmit ? spec * -1.f : spec;
                R.mask &= ~1;
            } else {
                const bool split = U.y > m.y;
                Ray C;
                if (split) {
                    C = R;
                    C.I = R.I * (1.f - m.z);
                    R.I *= m.z;
                    C.mask &= ~1;
                    C.d = transmit ? spec * -1.f : spec;
                    C.sid = sid_late(R.sid, nb);
                    C.nb = 0;
                    C.phase = 0;
                    ++L.v[C_OCT];
                }
                const float3 ld = lambert(nn, U.z, U.w);
                R.d = transmit ? ld * -1.f : ld;
                R.mask |= 3;
                if (split) {
                    if (C.I < R.I) {
                        // continue with the lower-energy child; the parent is mid-loop, settle its phase
                        const Ray tmp = R;
                        R = C;
                        C = tmp;
                        test_loop = false;
                        if (!(C.t_sum < r.cotime && C.I > kTP2)) { C.phase = 1; ++L.v[C_END]; }
                    }
                    if (sp < kStack) {
                        stack[sp++] = to_item(C);
                    } else {
                        const unsigned long long slot = atomicAdd(r.q_out_count, 1ull);
                        if (slot < r.q_out_cap) store_item(r.q_out, slot, to_item(C));
                        else ++L.v[C_OVF];
                        ++L.v[C_SPILL];
                    }
                }
            }
            if (test_loop && !(R.t_sum < r.cotime && R.I > kTP2)) { R.phase = 1; ++L.v[C_END]; }
        } else {
            // Scatter_VeryLate
            if (!r.pure_specular && U.y < m.z) {
                R.d = lambert(nn, U.z, U.w);
                R.mask |= 3;
            } else {
                R.d = spec;
                R.mask &= ~1;
            }
            if (transmit) R.d = R.d * -1.f;
            if (!(R.t_sum < r.cotime && R.I > kTP3)) have = false;
        }
        if (have && (long long)R.nb >= r.max_seg) { ++L.v[C_CAP]; have = false; }
    }
    flush_counters(r, L);
}

// ------------------------------------------------------------------------------------------
// pure-specular paths and emission directions (parity probes)
// ------------------------------------------------------------------------------------------
__global__ void k_paths(DevScene S, int n, const double *o, const double *dd, int maxb, int *poly, double *tout,
                        double *pts) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float3 p = make_float3((float)o[3 * i], (float)o[3 * i + 1], (float)o[3 * i + 2]);
    float3 d = unit3(make_float3((float)dd[3 * i], (float)dd[3 * i + 1], (float)dd[3 * i + 2]));
    int plane = -1;
    unsigned long long rt = 0;
    for (int b = 0; b < maxb; ++b) {
        const size_t k = (size_t)i * maxb + b;
        poly[k] = -1; tout[k] = 0; pts[3 * k] = pts[3 * k + 1] = pts[3 * k + 2] = 0;
    }
    for (int b = 0; b < maxb; ++b) {
        float t;
        int tri;
        if (!trace_ray(S, p, d, plane, t, tri, rt)) break;
        const size_t k = (size_t)i * maxb + b;
        const float4 A = __ldg(S.tri + 3 * tri), B = __ldg(S.tri + 3 * tri + 1);
        const int pl = __float_as_int(B.w);
        p = p + d * t;
        poly[k] = pl;
        tout[k] = t;
        pts[3 * k] = p.x; pts[3 * k + 1] = p.y; pts[3 * k + 2] = p.z;
        const float3 nrm = f3(__ldg(S.pnormal + pl));
        d = d - nrm * (2.f * dot3(d, nrm));
        plane = __float_as_int(A.w);
    }
}

__global__ void k_emit(DevRun r, long long p0, int n, double *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const long long prim = p0 + i;
    const int s = (int)((prim + 1) % r.nsrc);
    const float3 d = emit_dir(r, prim, (int)r.src[s].w);
    out[3 * i] = d.x; out[3 * i + 1] = d.y; out[3 * i + 2] = d.z;
}

}  // namespace

// ------------------------------------------------------------------------------------------
// host wrappers
// ------------------------------------------------------------------------------------------
cudaError_t launch_broadband(const DevRun &r, long long p0, long long p1, int blocks, int threads, cudaStream_t s) {
    k_broadband<<<blocks, threads, sizeof(float4) * (size_t)(r.R > 0 ? r.R : 1), s>>>(r, p0, p1);
    return cudaGetLastError();
}

cudaError_t launch_octave(const DevRun &r, int blocks, int threads, cudaStream_t s) {
    k_octave<<<blocks, threads, sizeof(float4) * (size_t)(r.R > 0 ? r.R : 1), s>>>(r);
    return cudaGetLastError();
}

cudaError_t octave_kernel_occupancy(int threads, int *blocks_per_sm) {
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_octave, threads, sizeof(float4) * 64);
}

cudaError_t launch_paths(const DevScene &S, int n, const double *o, const double *d, int max_bounces, int *poly,
                         double *t, double *pts, cudaStream_t s) {
    k_paths<<<(n + 127) / 128, 128, 0, s>>>(S, n, o, d, max_bounces, poly, t, pts);
    return cudaGetLastError();
}

cudaError_t launch_emit(const DevRun &r, long long p0, int n, double *out, cudaStream_t s) {
    k_emit<<<(n + 127) / 128, 128, 0, s>>>(r, p0, n, out);
    return cudaGetLastError();
}

}  // namespace pach
