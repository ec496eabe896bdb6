// device_common.cuh -- device helpers shared by the tracer kernels: Philox streams, vector math,
// the Lambert direction, the FP32/FP64 triangle test, the BVH walk, receiver detection with FP64
// histogram accumulation, emission directions and the octave-ray queue item.
#pragma once
#include <cfloat>
#include <cstdint>

#include "engine.h"

namespace pach {
namespace {

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

// Traversal work of one thread in one launch: FP64 re-tests, inner BVH nodes visited, triangles
// tested (32-bit: a thread walks a few thousand rays per launch at most; launches sum them in 64 bits).
struct TraceWork {
    unsigned retests = 0;
    unsigned nodes = 0, tris = 0;
};

// One candidate triangle: FP32 Moller-Trumbore, FP64 re-test inside the epsilon band.
__device__ __forceinline__ void test_tri(const DevScene &S, float t_eps, int i, float3 o, float3 d, int skip,
                                         float &best, int &bi, TraceWork &w) {
    const float4 A = __ldg(S.tri + 3 * i);
    if (__float_as_int(A.w) == skip) return;
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
    const bool grazing = fabsf(det) < C.w;
    if (grazing || !(fabsf(margin) > kBaryEps)) {
        // near grazing, near an edge, or not finite: decide in FP64.  Away from grazing the FP32
        // distance is accurate, so a candidate well outside (t_eps, best) needs no re-test.
        if (!grazing && isfinite(t) && (t < 0.5f * t_eps || t > 1.0001f * best)) return;
        double td;
        ++w.retests;
        if (retest64(S, i, o, d, td)) {
            const float tf = (float)td;
            if (tf > t_eps && tf < best) { best = tf; bi = i; }
        }
    } else if (margin > 0.f && t > t_eps && t < best) {
        best = t;
        bi = i;
    }
}

// Empty child slot of a 4-wide node (no leaf can have this code below 2^27 triangles).
constexpr int kEmptyChild = (int)0x80000000;

// Walk stack entries.  int2: (node or leaf code, entry distance of its box when it was pushed); a
// pop skips the entries whose box starts beyond the best hit found since -- the test a parent
// applies before pushing, applied again with the smaller best, so the walk's result is unchanged.
// Measured +1.8 % on a 20k-triangle hall, -4.5 % on a 12-triangle shoebox (a two-level tree culls
// nothing and pays for the wider entries): int, no distance, for the small-scene walk.
__device__ __forceinline__ void stack_push(int2 *stack, int &sp, int id, float t) {
    stack[sp++] = make_int2(id, __float_as_int(t));
}
__device__ __forceinline__ void stack_push(int *stack, int &sp, int id, float) { stack[sp++] = id; }
__device__ __forceinline__ int stack_pop(const int2 *stack, int &sp, float best) {
    while (sp > 0) {
        const int2 e = stack[--sp];
        if (__int_as_float(e.y) <= best) return e.x;
    }
    return kEmptyChild;
}
__device__ __forceinline__ int stack_pop(const int *stack, int &sp, float) { return sp > 0 ? stack[--sp] : kEmptyChild; }

__device__ __forceinline__ void cswap(float &ka, int &va, float &kb, int &vb) {
    if (kb < ka) {
        const float k = ka; ka = kb; kb = k;
        const int v = va; va = vb; vb = v;
    }
}

// One 4-wide node: slab-test the children against [0, best], order the hit ones by entry distance
// (5-exchange sorting network), push all but the nearest (farthest first), return the nearest in
// `next`.  Returns false when no child is hit.
template <typename E>
__device__ __forceinline__ bool bvh4_step(const float4 *__restrict__ bvh, int node, float ix, float iy, float iz,
                                          float ox, float oy, float oz, float best, E *stack, int &sp, int &next) {
    const float4 *N = bvh + (kBvhNodeFloats / 4) * node;
    // the near plane of each axis is the low bound for a positive direction, the high one otherwise:
    // choosing it per node leaves one max and one min per axis and child
    const float4 lx = __ldg(N), hx = __ldg(N + 1), ly = __ldg(N + 2), hy = __ldg(N + 3);
    const float4 lz = __ldg(N + 4), hz = __ldg(N + 5);
    const int4 ch = __ldg(reinterpret_cast<const int4 *>(N + 6));
    const float4 nx = ix < 0.f ? hx : lx, fx = ix < 0.f ? lx : hx;
    const float4 ny = iy < 0.f ? hy : ly, fy = iy < 0.f ? ly : hy;
    const float4 nz = iz < 0.f ? hz : lz, fz = iz < 0.f ? lz : hz;
    const float anx[4] = {nx.x, nx.y, nx.z, nx.w}, afx[4] = {fx.x, fx.y, fx.z, fx.w};
    const float any_[4] = {ny.x, ny.y, ny.z, ny.w}, afy[4] = {fy.x, fy.y, fy.z, fy.w};
    const float anz[4] = {nz.x, nz.y, nz.z, nz.w}, afz[4] = {fz.x, fz.y, fz.z, fz.w};
    int id[4] = {ch.x, ch.y, ch.z, ch.w};
    float tk[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float tn = fmaxf(fmaxf(fmaf(anx[k], ix, -ox), fmaf(any_[k], iy, -oy)), fmaxf(fmaf(anz[k], iz, -oz), 0.f));
        const float tf = fminf(fminf(fmaf(afx[k], ix, -ox), fmaf(afy[k], iy, -oy)), fminf(fmaf(afz[k], iz, -oz), best));
        tk[k] = (tn <= tf && id[k] != kEmptyChild) ? tn : FLT_MAX;
    }
    cswap(tk[0], id[0], tk[1], id[1]);
    cswap(tk[2], id[2], tk[3], id[3]);
    cswap(tk[0], id[0], tk[2], id[2]);
    cswap(tk[1], id[1], tk[3], id[3]);
    cswap(tk[1], id[1], tk[2], id[2]);
    if (tk[0] == FLT_MAX) return false;
#pragma unroll
    for (int k = 3; k >= 1; --k)
        if (tk[k] != FLT_MAX && sp < kBvhStack) stack_push(stack, sp, id[k], tk[k]);
    next = id[0];
    return true;
}

// The same step on a 48-byte quantised node: child bounds are 8-bit steps from the node's origin,
// a power-of-two step s per axis, so the slab distance q (s / d) + (origin - o) / d is one FMA per
// bound as with float nodes (s / d is exact: s is a power of two); (origin - o) / d is formed per node
// from the ray origin (px, py, pz), which keeps three fewer values live through the walk.  One byte permute makes the float
// 2^23 + 256 q; with the node's scale s / 256 the 2^15 steps it carries are taken off the slab offset
// once per node and axis (one rounding, at most 2^-9 of a step, inside the builder's s / 256 margin)
// instead of a subtraction per bound.
template <typename E>
__device__ __forceinline__ bool bvh4q_step(const float4 *__restrict__ bvhq, int node, float ix, float iy, float iz,
                                           float px, float py, float pz, float best, E *stack, int &sp, int &next) {
    const float4 *N = bvhq + (kBvhQNodeFloats / 4) * node;
    const float4 H = __ldg(N);
    const uint4 A = __ldg(reinterpret_cast<const uint4 *>(N + 1));
    const uint4 B = __ldg(reinterpret_cast<const uint4 *>(N + 2));
    const uint32_t e = __float_as_uint(H.w);
    // children from the slot codes (0 inner, 1-8 leaf of that many triangles, 15 empty): inner ids
    // count up from B.z, leaf triangles from the low 24 bits of B.w
    const uint32_t slots = (e >> 24) | ((B.w >> 24) << 8);
    int id[4];
    {
        int inner = (int)B.z, tri = (int)(B.w & 0xFFFFFFu);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int v = (int)((slots >> (4 * k)) & 15u);
            id[k] = v == 0 ? inner : (v <= 8 ? ~(tri * 16 + v - 1) : kEmptyChild);
            inner += v == 0;
            tri += v <= 8 ? v : 0;
        }
    }
    const float sx = __uint_as_float((e & 255u) << 23) * ix, sy = __uint_as_float(((e >> 8) & 255u) << 23) * iy,
                sz = __uint_as_float(((e >> 16) & 255u) << 23) * iz;
    const float bx = fmaf(-8388608.0f, sx, (H.x - px) * ix), by = fmaf(-8388608.0f, sy, (H.y - py) * iy),
                bz = fmaf(-8388608.0f, sz, (H.z - pz) * iz);
    float tk[4];
    // byte k of w as the float 2^23 + 256 byte (bits 0x4B00bb00): one byte permute
    auto q = [](uint32_t w, int k) {
        return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7504u + 16u * (uint32_t)k));
    };
    // near / far bound words of each axis, chosen by the direction's sign (as for float nodes)
    const uint32_t nwx = ix < 0.f ? A.y : A.x, fwx = ix < 0.f ? A.x : A.y;
    const uint32_t nwy = iy < 0.f ? A.w : A.z, fwy = iy < 0.f ? A.z : A.w;
    const uint32_t nwz = iz < 0.f ? B.y : B.x, fwz = iz < 0.f ? B.x : B.y;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float tn = fmaxf(fmaxf(fmaf(q(nwx, k), sx, bx), fmaf(q(nwy, k), sy, by)), fmaxf(fmaf(q(nwz, k), sz, bz), 0.f));
        const float tf = fminf(fminf(fmaf(q(fwx, k), sx, bx), fmaf(q(fwy, k), sy, by)), fminf(fmaf(q(fwz, k), sz, bz), best));
        tk[k] = tn <= tf ? tn : FLT_MAX;  // an empty slot's box is inverted on every axis: never hit
    }
    cswap(tk[0], id[0], tk[1], id[1]);
    cswap(tk[2], id[2], tk[3], id[3]);
    cswap(tk[0], id[0], tk[2], id[2]);
    cswap(tk[1], id[1], tk[3], id[3]);
    cswap(tk[1], id[1], tk[2], id[2]);
    if (tk[0] == FLT_MAX) return false;
#pragma unroll
    for (int k = 3; k >= 1; --k)
        if (tk[k] != FLT_MAX && sp < kBvhStack) stack_push(stack, sp, id[k], tk[k]);
    next = id[0];
    return true;
}

// Nearest hit along o + t d with t > t_eps, skipping triangles of plane `skip` (the surface the ray
// leaves).  4-wide BVH, nearest-child-first walk with a per-thread stack of the other hit
// children; a child box is entered only if the ray meets it before the best hit so far.
// E: the stack entry (int2 culls on pop, int does not; see stack_push).
template <typename E = int2>
__device__ __forceinline__ bool trace_ray(const DevScene &S, int root, float t_eps, float3 o, float3 d, int skip,
                                          float &t_best, int &tri_best, TraceWork &w) {
    const float dx = fabsf(d.x) < 1e-20f ? copysignf(1e-20f, d.x) : d.x;
    const float dy = fabsf(d.y) < 1e-20f ? copysignf(1e-20f, d.y) : d.y;
    const float dz = fabsf(d.z) < 1e-20f ? copysignf(1e-20f, d.z) : d.z;
    const float ix = 1.0f / dx, iy = 1.0f / dy, iz = 1.0f / dz;
    const float ox = o.x * ix, oy = o.y * iy, oz = o.z * iz;
    E stack[kBvhStack];
    int sp = 0;
    int node = root;
    float best = FLT_MAX;
    int bi = -1;
    if constexpr (sizeof(E) == sizeof(int2)) {
        while (node != kEmptyChild) {
            if (node >= 0) {
                ++w.nodes;
                int next;
                node = (S.bvhq ? bvh4q_step(S.bvhq, node, ix, iy, iz, o.x, o.y, o.z, best, stack, sp, next)
                               : bvh4_step(S.bvh, node, ix, iy, iz, ox, oy, oz, best, stack, sp, next))
                           ? next
                           : stack_pop(stack, sp, best);
                continue;
            }
            // leaf ~(first * 16 + count - 1)
            const int code = ~node;
            const int f0 = code >> 4, cnt = (code & 15) + 1;
            w.tris += (unsigned)cnt;
            for (int k = 0; k < cnt; ++k) test_tri(S, t_eps, f0 + k, o, d, skip, best, bi, w);
            node = stack_pop(stack, sp, best);
        }
    } else {
        // the small-scene walk: inner nodes until a leaf, then the leaf (measured 4 % faster on a
        // two-level tree than the loop above)
        for (;;) {
            bool done = false;
            while (node >= 0) {
                ++w.nodes;
                int next;
                if (!(S.bvhq ? bvh4q_step(S.bvhq, node, ix, iy, iz, o.x, o.y, o.z, best, stack, sp, next)
                             : bvh4_step(S.bvh, node, ix, iy, iz, ox, oy, oz, best, stack, sp, next))) {
                    if (sp == 0) { done = true; break; }
                    node = stack[--sp];
                    continue;
                }
                node = next;
            }
            if (done) break;
            const int code = ~node;
            const int f0 = code >> 4, cnt = (code & 15) + 1;
            w.tris += (unsigned)cnt;
            for (int k = 0; k < cnt; ++k) test_tri(S, t_eps, f0 + k, o, d, skip, best, bi, w);
            if (sp == 0) break;
            node = stack[--sp];
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
__device__ __forceinline__ void hist_add(const DevRun &r, float rho_c, int k, int oct, long long bin, float e, float3 d,
                                         int kind) {
    const size_t base = ((size_t)k * kBands + oct) * r.T + bin;
    atomicAdd(r.hE + base, (double)e);
    atomicAdd(r.hP + base, (double)sqrtf(e * rho_c));
    const float ca[3] = {-d.x, -d.y, -d.z};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const size_t j = (((size_t)k * 3 + a) * kBands + oct) * r.T + bin;
        atomicAdd((ca[a] > 0.f ? r.hDp : r.hDn) + j, (double)(ca[a] * e));
    }
    atomicAdd(r.hAn + (((size_t)k * 3 + kind) * kBands + oct) * r.T + bin, (double)e);
}

__device__ __forceinline__ void capture_add(const DevRun &r, const RoomParams &P, float4 rc, int k, uint32_t prim,
                                            double time, float e);

// Convergence mode: the detection also goes to its revolution's copy of the check receiver's energy
// and analysis histograms (the checks replay the revolutions on the host).
__device__ __forceinline__ void conv_add(const DevRun &r, int row, int oct, long long bin, float e, int kind,
                                         uint32_t prim) {
    if (oct != r.conv_oct) return;
    const int k = row == r.conv_row[0] ? 0 : (row == r.conv_row[1] ? 1 : -1);
    if (k < 0) return;
    const long long rev = ((long long)prim - r.ctl->prim_first) / r.conv_period;
    if (rev < 0 || rev >= kConvChunk) return;
    double *h = r.conv + ((size_t)rev * 2 + k) * kConvKinds * r.T;
    atomicAdd(h + bin, (double)e);
    atomicAdd(h + (size_t)(1 + kind) * r.T + bin, (double)e);
}

// A cheap superset of sphere_hit: the centre's squared distance from the ray's line, |m|^2 - b^2,
// within the squared radius plus a margin far above its FP32 rounding (a few ulps of |m|^2 away from
// sphere_hit's |m - b d|^2; tests/test_receiver_prefilter.py checks in float32 that no sphere the
// exact test accepts is rejected here).  The chord's position along the
// segment is left to the exact test: a receiver near the line but beyond the segment is rare.
__device__ __forceinline__ bool sphere_near(float4 c, float3 o, float3 d) {
    const float mx = o.x - c.x, my = o.y - c.y, mz = o.z - c.z;
    const float b = fmaf(mx, d.x, fmaf(my, d.y, mz * d.z));
    const float mm = fmaf(mx, mx, fmaf(my, my, mz * mz));
    return fmaf(-b, b, mm) <= fmaf(1e-5f, mm, c.w + 1e-6f);
}

// One octave detection (Spherical_Receiver.CheckRay, Classes_Receivers.cs:837-877) of the receiver in
// slot s, whose sphere the segment's chord (midpoint t, half-length half) crosses: energy
// I 10^(-0.1 m c time) / pi * half into its histograms.
__device__ __forceinline__ void detect_octave_one(const DevRun &r, const RoomParams &P, const int *rid, int s, float4 c,
                                                  float3 d, float t, float half, double t_sum, float Iabs, int oct,
                                                  int mask, uint32_t prim) {
    const int row = rid ? rid[s] : s;
    const double time = t_sum + (double)(t * P.inv_c);
    const long long bin = (long long)(time * r.fs);
    if (!(time >= 0.0) || bin < 0 || bin >= r.T) return;
    const float e = Iabs * exp2f(P.atten_k[oct] * (float)time) * kInvPi * half;
    const int kind = (mask & 1) ? 1 : ((mask & 2) ? 2 : 0);
    hist_add(r, P.rho_c, row, oct, bin, e, d, kind);
    if (r.capture) capture_add(r, P, c, row, prim, time, e);
    if (r.conv) conv_add(r, row, oct, bin, e, kind, prim);
}

// Spherical_Receiver.CheckRay over the receivers of the ray's room (rec: the run's receiver table in
// shared memory).  Returns the spheres hit.  GROUPED: receivers go four at a time through sphere_near
// (four independent chains, no branch while none is near; the remainder of the room's receivers one
// at a time) and the exact sphere_hit decides for the near ones.
template <bool GROUPED>
__device__ __forceinline__ uint32_t detect_octave(const DevRun &r, const RoomParams &P, const float4 *rec,
                                                  const int *rid, float3 o, float3 d, float tseg, double t_sum,
                                                  float Iabs, int oct, int mask, uint32_t prim) {
    uint32_t n = 0;
    if constexpr (!GROUPED) {
        for (int s = P.rec_begin; s < P.rec_begin + P.R; ++s) {
            const float4 c = rec[s];
            float t, half;
            if (!sphere_hit(c, o, d, tseg, t, half)) continue;
            ++n;
            detect_octave_one(r, P, rid, s, c, d, t, half, t_sum, Iabs, oct, mask, prim);
        }
        return n;
    }
    const int s1 = P.rec_begin + P.R;
    int s0 = P.rec_begin;
    for (; s0 + 4 <= s1; s0 += 4) {
        bool near[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) near[k] = sphere_near(rec[s0 + k], o, d);
        if (!(near[0] | near[1] | near[2] | near[3])) continue;
#pragma unroll 1
        for (int k = 0; k < 4; ++k) {
            if (!near[k]) continue;
            const float4 c = rec[s0 + k];
            float t, half;
            if (!sphere_hit(c, o, d, tseg, t, half)) continue;
            ++n;
            detect_octave_one(r, P, rid, s0 + k, c, d, t, half, t_sum, Iabs, oct, mask, prim);
        }
    }
    for (; s0 < s1; ++s0) {
        const float4 c = rec[s0];
        float t, half;
        if (!sphere_hit(c, o, d, tseg, t, half)) continue;
        ++n;
        detect_octave_one(r, P, rid, s0, c, d, t, half, t_sum, Iabs, oct, mask, prim);
    }
    return n;
}

// Spherical_Receiver.CheckBroadbandRay (Classes_Receivers.cs:803-829): every band of the range,
// analysis bin 0 (specular).
__device__ __forceinline__ uint32_t detect_broad(const DevRun &r, const RoomParams &P, const float4 *rec,
                                                 const int *rid, float3 o, float3 d, float tseg, double t_sum,
                                                 const float (&E)[kBands], const float (&sc)[kBands], uint32_t prim) {
    uint32_t n = 0;
    for (int s = P.rec_begin; s < P.rec_begin + P.R; ++s) {
        const float4 c = rec[s];
        float t, half;
        if (!sphere_hit(c, o, d, tseg, t, half)) continue;
        ++n;
        const int k = rid ? rid[s] : s;
        const double time = t_sum + (double)(t * P.inv_c);
        const long long bin = (long long)(time * r.fs);
        if (!(time >= 0.0) || bin < 0 || bin >= r.T) continue;
        float esum = 0.f;
#pragma unroll
        for (int oct = 0; oct < kBands; ++oct) {
            if (oct < P.oct_lo || oct > P.oct_hi) continue;
            const float e = E[oct] * sc[oct] * exp2f(P.atten_k[oct] * (float)time) * kInvPi * half;
            hist_add(r, P.rho_c, k, oct, bin, e, d, 0);
            if (r.conv) conv_add(r, k, oct, bin, e, 0, prim);
            esum += e;
        }
        if (r.capture) capture_add(r, P, c, k, prim, time, esum);
    }
    return n;
}

// ------------------------------------------------------------------------------------------
// mapping receivers (PachMapReceiver, Pach_Map_Receiver.cs)
// ------------------------------------------------------------------------------------------
// Histogram.Add / Histogram_1Pt.Add (Classes_Receivers.cs:1159-1166, 1393-1396) at 1000 Hz: the
// sample is (int)(time * 1000), a truncation, so arrivals up to 1 ms before the direct arrival
// land in bin 0; samples outside [0, T) are dropped.  Histogram_1Pt keeps every arrival in bin 0
// and no pressure.
// Directional_Histogram.Add (1813-1825) for a directional map: pressure sqrt(E rho c), and the
// arrival direction -d split by sign into the +/- component histograms, each term rounded to float
// as the reference rounds it.  (The reference has no lower bound there; an arrival more than 1 ms
// before the direct one cannot occur at a receiver the direct path reaches, and is dropped.)
__device__ __forceinline__ void map_add(const MapDev &M, int k, int oct, double time, float e, float3 d) {
    long long s = 0;
    if (!M.one_pt) {
        const double x = time * 1000.0;
        if (!(x > -1.0) || x >= (double)M.T) return;
        s = (long long)x;
    }
    const size_t i = ((size_t)k * kBands + oct) * M.T + s;
    atomicAdd(M.E + i, (double)e);
    if (M.one_pt) return;
    if (!M.directional) {
        atomicAdd(M.P + i, (double)sqrtf(e));
        return;
    }
    atomicAdd(M.P + i, (double)sqrtf(e * M.rho_c));
    const float ca[3] = {-d.x, -d.y, -d.z};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const size_t j = (((size_t)k * 3 + a) * kBands + oct) * M.T + s;
        atomicAdd((ca[a] > 0.f ? M.Dp : M.Dn) + j, (double)(ca[a] * e));
    }
}

// OBox.IsPointInBox and OBox.Intersect (Hare AABB, not in the reference tree), restated as
// inclusive bounds and the slab test of the half-line o + t d, t >= 0.
__device__ __forceinline__ bool map_box_entry(const MapDev &M, float3 o, float3 d, float &t0) {
    const float oo[3] = {o.x, o.y, o.z}, dd[3] = {d.x, d.y, d.z};
    float tn = 0.f, tf = 3.0e38f;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (dd[a] == 0.f) {
            if (oo[a] < M.lo[a] || oo[a] > M.hi[a]) return false;
            continue;
        }
        const float inv = 1.f / dd[a];
        float ta = (M.lo[a] - oo[a]) * inv, tb = (M.hi[a] - oo[a]) * inv;
        if (ta > tb) { const float x = ta; ta = tb; tb = x; }
        tn = fmaxf(tn, ta);
        tf = fminf(tf, tb);
    }
    t0 = tn;
    return tn <= tf;
}

__device__ __forceinline__ int map_cell_index(float p, float lo, float vd) {
    return (int)floorf(fminf(fmaxf((p - lo) / vd, -1.0e9f), 1.0e9f));
}

// The receiver-grid walk of one segment [o, end] (CheckBroadbandRay / CheckRay,
// Pach_Map_Receiver.cs:1359-1631), calling visit(k) once for every receiver listed in a visited
// cell.  walk 0 keeps the reference's two walks as written: the broadband walk starts from the
// ray's origin even when it lies outside the grid, takes its step signs, first crossings and
// increments from the ray's POSITION (R.x where R.dx is meant) and stops as soon as ANY cell index
// equals the end cell's; the octave walk starts at the grid entry point and stops on reaching the
// end cell without visiting it (after a segment that starts and ends in one cell it runs on to the
// grid's edge).  walk 1 visits every cell the segment crosses, the end cell included.
template <typename Visit>
__device__ __forceinline__ void map_walk(const MapDev &M, float3 o, float3 d, float3 end, bool broadband, Visit visit) {
    const bool quirk = broadband && M.walk == 0;
    float3 s = o;
    const bool inside = o.x >= M.lo[0] && o.x <= M.hi[0] && o.y >= M.lo[1] && o.y <= M.hi[1] && o.z >= M.lo[2] &&
                        o.z <= M.hi[2];
    if (!inside) {
        float t0;
        if (!map_box_entry(M, o, d, t0)) return;
        if (!quirk) s = o + d * t0;
    }
    const float sp[3] = {s.x, s.y, s.z}, ep[3] = {end.x, end.y, end.z};
    // the quantity whose sign and size steer the walk: the direction, or the reference broadband walk's
    // position; a direction component of -0 walks as +0 (its crossing time is +inf, never -inf)
    float g[3] = {quirk ? o.x : d.x, quirk ? o.y : d.y, quirk ? o.z : d.z};
    if (!quirk)
        for (int a = 0; a < 3; ++a) g[a] = g[a] == 0.f ? 0.f : g[a];
    int c[3], ce[3], step[3];
    float tmax[3], tdel[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        c[a] = map_cell_index(sp[a], M.lo[a], M.vd[a]);
        ce[a] = map_cell_index(ep[a], M.lo[a], M.vd[a]);
        c[a] = c[a] < 0 ? 0 : (c[a] >= M.n[a] ? M.n[a] - 1 : c[a]);
        if ((g[a] < 0.f && c[a] < ce[a]) || (g[a] >= 0.f && c[a] > ce[a])) return;
        step[a] = g[a] < 0.f ? -1 : 1;
        const float bound = (float)(g[a] < 0.f ? c[a] : c[a] + 1) * M.vd[a] + M.lo[a];
        tmax[a] = (bound - sp[a]) / g[a];
        tdel[a] = M.vd[a] / g[a] * (float)step[a];
    }
    // the last three cells visited: a receiver listed in an earlier cell of this walk is listed in one
    // of them (a sphere spans at most two cells per axis and every step moves one axis by one cell)
    int3 p0 = make_int3(-4, -4, -4), p1 = p0, p2 = p0;  // far from every cell until visited
    auto near_bit = [&](int3 p) -> uint32_t {
        const int dx = p.x - c[0], dy = p.y - c[1], dz = p.z - c[2];
        return (dx >= -1 && dx <= 1 && dy >= -1 && dy <= 1 && dz >= -1 && dz <= 1)
                   ? 1u << ((dx + 1) * 9 + (dy + 1) * 3 + (dz + 1))
                   : 0u;
    };
    const int max_steps = M.n[0] + M.n[1] + M.n[2] + 1;
    for (int it = 0; it <= max_steps; ++it) {
        const uint32_t seen = near_bit(p0) | near_bit(p1) | near_bit(p2);
        const int ci = (c[0] * M.n[1] + c[1]) * M.n[2] + c[2];
        const int e1 = __ldg(M.cell + ci + 1);
        for (int e = __ldg(M.cell + ci); e < e1; ++e) {
            const uint2 en = __ldg(M.entry + e);
            if (en.y & seen) continue;
            visit((int)en.x);
        }
        p2 = p1;
        p1 = p0;
        p0 = make_int3(c[0], c[1], c[2]);
        if (M.walk && c[0] == ce[0] && c[1] == ce[1] && c[2] == ce[2]) return;
        // the reference's comparison order (ties go to z, then y)
        const bool sx = tmax[0] < tmax[1] && tmax[0] < tmax[2];
        const bool sy = !(tmax[0] < tmax[1]) && tmax[1] < tmax[2];
        if (sx) {
            c[0] += step[0];
            if (c[0] < 0 || c[0] >= M.n[0]) return;  // outside the grid
            tmax[0] += tdel[0];
        } else if (sy) {
            c[1] += step[1];
            if (c[1] < 0 || c[1] >= M.n[1]) return;
            tmax[1] += tdel[1];
        } else {
            c[2] += step[2];
            if (c[2] < 0 || c[2] >= M.n[2]) return;
            tmax[2] += tdel[2];
        }
        if (quirk) {
            if (!(c[0] != ce[0] && c[1] != ce[1] && c[2] != ce[2])) return;
        } else if (M.walk == 0) {
            if (c[0] == ce[0] && c[1] == ce[1] && c[2] == ce[2]) return;
        }
    }
}

// Map_Receiver.CheckRay (Pach_Map_Receiver.cs:1810-1826) over the grid: energy
// I 10^(-0.1 m t) / (pi r^2), t = arrival time after the receiver's direct arrival (s).
__device__ __forceinline__ uint32_t map_detect_octave(const MapDev &M, const RoomParams &P, float3 o, float3 d,
                                                      float tseg, double t_sum, float Iabs, int oct) {
    uint32_t n = 0;
    map_walk(M, o, d, o + d * tseg, false, [&](int k) {
        float t, half;
        if (!sphere_hit(__ldg(M.rec + k), o, d, tseg, t, half)) return;
        ++n;
        const double time = t_sum + (double)(t * P.inv_c) - __ldg(M.direct + k);
        map_add(M, k, oct, time, Iabs * exp2f(M.atten_k[oct] * (float)time) * M.size_mod, d);
    });
    return n;
}

// Map_Receiver.CheckBroadbandRay (Pach_Map_Receiver.cs:1780-1808): all eight bands, whatever the
// octave range.
__device__ __forceinline__ uint32_t map_detect_broad(const MapDev &M, const RoomParams &P, float3 o, float3 d,
                                                     float tseg, double t_sum, const float (&E)[kBands],
                                                     const float (&sc)[kBands]) {
    uint32_t n = 0;
    map_walk(M, o, d, o + d * tseg, true, [&](int k) {
        float t, half;
        if (!sphere_hit(__ldg(M.rec + k), o, d, tseg, t, half)) return;
        ++n;
        const double time = t_sum + (double)(t * P.inv_c) - __ldg(M.direct + k);
#pragma unroll
        for (int oct = 0; oct < kBands; ++oct)
            map_add(M, k, oct, time, E[oct] * sc[oct] * exp2f(M.atten_k[oct] * (float)time) * M.size_mod, d);
    });
    return n;
}

// ------------------------------------------------------------------------------------------
// emission
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ float3 emit_dir(const DevRun &r, int nsrc, long long prim, int kind) {
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
    const long long j = prim / nsrc;
    const int f = (int)(j % kGeoFaces);
    float u = U.x, v = U.y;
    if (u + v > 1.f) { u = 1.f - u; v = 1.f - v; }
    const float3 a = f3(r.geo[3 * f]), b = f3(r.geo[3 * f + 1]), c = f3(r.geo[3 * f + 2]);
    return unit3(a + (b - a) * u + (c - a) * v);
}

// ------------------------------------------------------------------------------------------
// learned emission proposal and training capture (no counterpart in the reference)
// ------------------------------------------------------------------------------------------
constexpr float kInv4Pi = 0.0795774715459476679f;

// Defensive mixture: uniform on the sphere with probability prop_mix, else a lobe of one of the n_prop
// receiver mixtures (receiver uniform, lobe by its weight).  w = (1 / 4 pi) / q(d), the density ratio of
// uniform emission to the mixture, keeps the estimate unbiased.
__device__ __forceinline__ float3 proposal_dir(const DevRun &r, uint32_t prim, float &w) {
    const float4 U = draw(r.seed, prim, 0ull, 1u);
    const float4 V = draw(r.seed, prim, 0ull, 2u);
    float3 d;
    if (U.x < r.prop_mix) {
        const float z = 1.0f - 2.0f * V.x;
        const float rr = sqrtf(fmaxf(0.f, 1.f - z * z));
        float sp, cp;
        sincospif(2.0f * V.y, &sp, &cp);
        d = make_float3(rr * cp, rr * sp, z);
    } else {
        const int j = min(r.n_prop - 1, (int)(U.y * (float)r.n_prop));
        const float4 *L = r.prop + (size_t)j * kLobes * 2;
        int k = 0;
        while (k < kLobes - 1 && U.z >= __ldg(L + 2 * k + 1).y) ++k;
        const float4 a = __ldg(L + 2 * k);
        const float kap = a.w;
        // Wood (1994) for the 2-sphere: cosine to the mean c = 1 + log(u + (1 - u) e^(-2 kappa)) / kappa
        const float c = fminf(1.f, fmaxf(-1.f, 1.f + logf(V.x + (1.f - V.x) * expf(-2.f * kap)) / kap));
        const float sn = sqrtf(fmaxf(0.f, 1.f - c * c));
        float sp, cp;
        sincospif(2.0f * V.y, &sp, &cp);
        const float3 mu = make_float3(a.x, a.y, a.z);
        const float3 t = fabsf(mu.x) < 0.9f ? make_float3(1.f, 0.f, 0.f) : make_float3(0.f, 1.f, 0.f);
        const float3 e1 = unit3(cross3(mu, t));
        const float3 e2 = cross3(mu, e1);
        d = unit3(mu * c + (e1 * cp + e2 * sp) * sn);
    }
    float qs = 0.f;
    for (int j = 0; j < r.n_prop; ++j) {
        const float4 *L = r.prop + (size_t)j * kLobes * 2;
        for (int k = 0; k < kLobes; ++k) {
            const float4 a = __ldg(L + 2 * k), b = __ldg(L + 2 * k + 1);
            qs += expf(b.x + a.w * (a.x * d.x + a.y * d.y + a.z * d.z - 1.f));
        }
    }
    const float q = r.prop_mix * kInv4Pi + (1.f - r.prop_mix) * qs / (float)r.n_prop;
    w = kInv4Pi / q;
    return d;
}

// Emission direction of primary prim and its weight (1 unless importance sampled).
__device__ __forceinline__ float3 primary_dir(const DevRun &r, int nsrc, uint32_t prim, int kind, float &w) {
    w = 1.f;
    if (r.prim_dirs) {
        const double *pd = r.prim_dirs + 3 * ((long long)prim - r.prim_base);
        if (r.prim_weights) w = (float)r.prim_weights[(long long)prim - r.prim_base];
        return make_float3((float)pd[0], (float)pd[1], (float)pd[2]);
    }
    if (r.prop) return proposal_dir(r, prim, w);
    if (r.prim_weights) w = (float)r.prim_weights[(long long)prim - r.prim_base];
    return emit_dir(r, nsrc, prim, kind);
}

// Training capture: energy e detected at receiver k at time (s) from primary prim, added to the bin
// of the primary's emission direction in the window of (time - direct arrival).
// rc: the receiver (x, y, z, r^2), k: its histogram row
__device__ __forceinline__ void capture_add(const DevRun &r, const RoomParams &P, float4 rc, int k, uint32_t prim,
                                            double time, float e) {
    const int s = P.src_begin + (int)((prim + 1ull) % (unsigned long long)P.nsrc);
    const float4 src = r.src[s];
    const double dx = rc.x - src.x, dy = rc.y - src.y, dz = rc.z - src.z;
    const float ms = (float)((time - sqrt(dx * dx + dy * dy + dz * dz) * P.inv_c_d) * 1000.0);
    const int win = (ms >= r.cap_edge[0]) + (ms >= r.cap_edge[1]) + (ms >= r.cap_edge[2]);
    if (r.capture_mode == 2) {
        atomicAdd(r.capture + (((size_t)((long long)prim - r.prim_base)) * r.R + k) * kCaptureWindows + win, e);
        return;
    }
    float w;
    const float3 d0 = primary_dir(r, P.nsrc, prim, (int)src.w, w);
    const int b = dir_bin(d0.x, d0.y, d0.z);
    atomicAdd(r.capture + ((size_t)k * kCaptureWindows + win) * kDirBins + b, e);
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
    int oct, mask, phase, plane, room;
};

__device__ __forceinline__ ORayItem to_item(const Ray &R) {
    ORayItem it;
    it.px = R.p.x; it.py = R.p.y; it.pz = R.p.z; it.I = R.I;
    it.dx = R.d.x; it.dy = R.d.y; it.dz = R.d.z; it.scale = R.scale;
    it.t_sum = R.t_sum; it.prim = R.prim; it.nb = R.nb; it.sid = R.sid;
    it.meta = (uint32_t)R.oct | ((uint32_t)R.mask << 3) | ((uint32_t)R.phase << 5) | ((uint32_t)R.room << 6);
    it.plane = R.plane;
    return it;
}

__device__ __forceinline__ Ray to_ray(const ORayItem &it) {
    Ray R;
    R.p = make_float3(it.px, it.py, it.pz);
    R.d = make_float3(it.dx, it.dy, it.dz);
    R.I = it.I; R.scale = it.scale; R.t_sum = it.t_sum; R.prim = it.prim; R.nb = it.nb; R.sid = it.sid;
    R.oct = (int)(it.meta & 7u); R.mask = (int)((it.meta >> 3) & 3u); R.phase = (int)((it.meta >> 5) & 1u);
    R.room = (int)(it.meta >> 6);
    R.plane = it.plane;
    return R;
}

__device__ __forceinline__ Ray new_ray(float3 p, float3 d, float I, float scale, double t_sum, uint32_t prim,
                                       unsigned long long sid, int oct, int mask, int plane, int room) {
    Ray R;
    R.p = p; R.d = d; R.I = I; R.scale = scale; R.t_sum = t_sum; R.prim = prim; R.nb = 0; R.sid = sid;
    R.oct = oct; R.mask = mask; R.phase = 0; R.plane = plane; R.room = room;
    return R;
}

// Room of a primary: the last room whose first primary is <= prim (binary search of room_prim).
__device__ __forceinline__ int room_of(const DevRun &r, long long prim) {
    int lo = 0, hi = r.n_rooms - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(r.room_prim + mid) <= prim) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Reserves n consecutive queue slots only if they all fit; bounded retries under contention.
__device__ __forceinline__ bool reserve(unsigned long long *count, unsigned long long n, unsigned long long cap,
                                        unsigned long long &slot) {
    unsigned long long old = *reinterpret_cast<volatile unsigned long long *>(count);
    for (int tries = 0; tries < 64; ++tries) {
        if (old + n > cap) return false;
        const unsigned long long prev = atomicCAS(count, old, old + n);
        if (prev == old) { slot = old; return true; }
        old = prev;
    }
    return false;
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

// Receiver table for detection: staged in shared memory when it is small (the common case), else read
// through L1 (a batch of many rooms: each ray tests only its room's receivers).
// The run's receiver table (and the row of each sorted slot) in shared memory when it fits.
__device__ __forceinline__ const float4 *stage_receivers(const DevRun &r, float4 *smem, const int *&rid) {
    if (r.R > kSmemReceivers) {
        rid = r.rec_id;
        return r.rec;
    }
    int *sid = reinterpret_cast<int *>(smem + (r.R > 0 ? r.R : 1));
    for (int i = threadIdx.x; i < r.R; i += blockDim.x) {
        smem[i] = r.rec[i];
        if (r.rec_id) sid[i] = r.rec_id[i];
    }
    __syncthreads();
    rid = r.rec_id ? sid : nullptr;
    return smem;
}

}  // namespace
}  // namespace pach
