// trace.cu -- sm_103a kernels of the stochastic split ray tracer, as a wavefront pipeline.
//
// Hot path of SplitRayTracer.cast_ray_distributed / End_Trace ("Classes_Complete_Trace -
// TaskAll.cs":335-536).  Octave rays live in a ring queue in HBM; every iteration of the device
// loop runs five kernels on one stream:
//   k_feed       1 thread: retire the last wave, hand the next batch of primaries to phase A while
//                the ring runs low (primaries stream in until the run is done, so no launch tail).
//   k_broadband  phase A, one thread per fed primary: emission (Classes_Sources.cs:256-265,
//                390-403), BVH walk, broadband detection (Classes_Receivers.cs:803-829), absorption
//                (Classes_Materials.cs:166-178) and Scatter_Early (4498-4570); the band children of
//                every bounce and the final split are appended to the ring (TaskAll:347-424).
//   k_wave       1 thread: size the wave -- as many ring items as leave room for their outputs.
//   k_trace      one thread per wave item: the BVH walk only, a lean kernel that keeps many warps
//                resident to hide L1/L2 latency; writes (triangle, t) per item.
//   k_shade      one thread per wave item: receiver detection into FP64 histograms (837-877),
//                absorption, one Philox draw block, Scatter_Late (phase B, 4629-4701) or
//                Scatter_VeryLate (phase C, 4572-4627), then the surviving ray and a split child are
//                appended to the ring with one atomic per warp (TaskAll:429-536).
// Random numbers are Philox4x32-10 streams keyed by (seed, primary, stream id, block): the streams
// the CPU oracle draws, so a ray's decisions do not depend on scheduling.
#include "device_common.cuh"

namespace pach {
namespace {

constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ ORayItem ring_load(const DevRun &r, unsigned long long i) {
    return load_item(r.ring, i & (r.ring_cap - 1));
}

__device__ __forceinline__ void ring_store(const DevRun &r, unsigned long long i, const ORayItem &it) {
    store_item(r.ring, i & (r.ring_cap - 1), it);
}

// Item j of the current wave: the sorted copy when the wave was sorted, else the ring in place.
__device__ __forceinline__ const ORayItem *wave_item(const DevRun &r, unsigned long long head, unsigned long long j) {
    return r.wave_buf ? r.wave_buf + j : r.ring + ((head + j) & (r.ring_cap - 1));
}

// All 32 lanes call: lane gets the first of its n ring slots; one atomic per warp.
__device__ __forceinline__ unsigned long long warp_append(unsigned long long *tail, int n) {
    const int lane = threadIdx.x & 31;
    int incl = n;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(FULL, incl, o);
        if (lane >= o) incl += v;
    }
    const int total = __shfl_sync(FULL, incl, 31);
    unsigned long long base = 0;
    if (lane == 31 && total) base = atomicAdd(tail, (unsigned long long)total);
    base = __shfl_sync(FULL, base, 31);
    return base + (unsigned long long)(incl - n);
}

// ------------------------------------------------------------------------------------------
// scheduling (single thread)
// ------------------------------------------------------------------------------------------
__global__ void k_feed(DevRun r) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    WaveCtl *c = r.ctl;
    c->head += c->m;  // retire the previous wave
    c->m = 0;
    c->pa_count = 0;
    if (c->done) return;
    // cancellation (graph mode): stop feeding; the primaries already fed run to completion
    if (r.cancel && *r.cancel && c->prim_end > c->next_prim) c->prim_end = c->next_prim;
    const unsigned long long live = c->tail - c->head;
    // Pilots: the first kPilotPrimaries primaries of every room (of a plain run: of the run) are fed
    // alone; once their split trees are done, their peak live count per primary (x 3) is the ring
    // footprint the feed plans batches with -- the largest over the rooms measured so far, so a room
    // whose split trees outgrow an earlier room's cannot overfill the ring.  The margin: a pilot fits
    // in one wave, so each wave advances its trees by a whole level, while a batch larger than a wave
    // is traced first-in-first-out across two levels at once and peaks higher per primary (measured
    // up to 2.7x on 12-receiver shoeboxes at 20k primaries); k_wave doubles the figure again when the
    // ring passes three quarters full.
    if (c->pilot_count > 0) {
        if (live != 0) return;
        unsigned long long pp = c->pilot_peak * 3 / (unsigned long long)c->pilot_count + 1;
        if (pp < r.feed_bound) pp = r.feed_bound;
        if (pp > c->per_prim) c->per_prim = pp;
        c->pilot_count = 0;
    }
    if (c->next_prim >= c->prim_end) return;
    const int room = room_of(r, c->next_prim);
    if (room >= c->pilot_room) {
        if (live != 0) return;  // the pilot runs alone: the ring drains first
        const long long room_end = room + 1 < r.n_rooms ? __ldg(r.room_prim + room + 1) : c->prim_end;
        long long n = room_end - c->next_prim;
        if (n > kPilotPrimaries) n = kPilotPrimaries;
        if (n > r.feed_batch) n = r.feed_batch;
        if (n > c->prim_end - c->next_prim) n = c->prim_end - c->next_prim;
        const long long fit = (long long)(r.ring_cap / r.feed_bound);  // >= 4: checked at set-up
        if (n > fit) n = fit;
        if (n < 1) n = 1;
        c->pa_begin = c->next_prim;
        c->pa_count = n;
        c->next_prim += n;
        c->pilot_count = n;
        c->pilot_peak = 0;
        c->pilot_room = room + 1;
        c->last_live = 0;
        return;
    }
    // Split trees grow for many waves after phase A, so a batch is fed only once the previous one
    // has peaked: the live count is low and no longer rising (generations of primaries).
    const bool decaying = live <= c->last_live;
    c->last_live = live;
    if (live <= r.low_water && (decaying || live == 0)) {
        // Hard limit: the phase-A output of every fed primary must fit.  Soft limit: the new batch's
        // peak keeps the ring at most half full.
        unsigned long long room_n = (r.ring_cap - live) / r.feed_bound;
        const unsigned long long per_prim = c->per_prim ? c->per_prim : r.feed_bound;
        const unsigned long long half = r.ring_cap / 2;
        const unsigned long long soft = live < half ? (half - live) / per_prim : 0;
        if (soft < room_n) room_n = soft > 0 ? soft : (live == 0 ? 1 : 0);
        long long n = c->prim_end - c->next_prim;
        if (n > r.feed_batch) n = r.feed_batch;
        // a batch never reaches into a room whose pilot has not run
        if (c->pilot_room < r.n_rooms) {
            const long long lim = __ldg(r.room_prim + c->pilot_room) - c->next_prim;
            if (n > lim) n = lim;
        }
        if ((unsigned long long)n > room_n) n = (long long)room_n;
        if (n > 0) {
            c->pa_begin = c->next_prim;
            c->pa_count = n;
            c->next_prim += n;
            c->pressure = 0;
        }
    }
}

__global__ void k_wave(DevRun r) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    WaveCtl *c = r.ctl;
    if (c->done) { c->m = 0; return; }
    const unsigned long long live = c->tail - c->head;
    if (live > c->peak_live) c->peak_live = live;
    if (c->pilot_count > 0 && live > c->pilot_peak) c->pilot_peak = live;
    // the batches outgrew their plan: plan the next ones with twice the footprint per primary
    if (live > r.ring_cap / 4 * 3 && !c->pressure && c->per_prim) {
        c->pressure = 1;
        c->per_prim *= 2;
    }
    unsigned long long m = (r.ring_cap - live) / 2;  // each item leaves at most two
    if (m > live) m = live;
    if (m > r.max_wave) m = r.max_wave;
    c->m = m;
    c->trace_next = 0;
    if (m) ++c->waves;
    if (live == 0 && c->next_prim >= c->prim_end) c->done = 1;
    if (live > 0 && m == 0) { ++c->overflow; c->done = 1; }  // ring full: cannot make progress
}

// Last node of a graph-mode iteration: decides whether the while loop runs again.  The loop ends
// when the run is done, and also -- as a failure -- after max_iters iterations or 4096 consecutive
// iterations that neither traced nor fed, so it always terminates.  Progress goes to mapped host
// memory for the polling host thread.
__global__ void k_cond(DevRun r, cudaGraphConditionalHandle h) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    WaveCtl *c = r.ctl;
    ++c->iters;
    if (c->m == 0 && c->pa_count == 0 && !c->done) ++c->idle;
    else c->idle = 0;
    bool stop = c->done != 0;
    if (!stop && (c->iters >= r.max_iters || c->idle >= 4096)) {
        c->gave_up = 1;
        stop = true;
    }
    if (!stop && r.cancel && *r.cancel >= 2) {  // abort: the host stops waiting for fed primaries
        c->gave_up = 2;
        stop = true;
    }
    if (r.mirror) {
        HostMirror *hm = r.mirror;
        hm->next_prim = c->next_prim;
        hm->iters = c->iters;
        hm->segments = r.cnt->seg_broad + r.cnt->seg_b + r.cnt->seg_c;
        hm->end_traces = r.cnt->end_traces;
        hm->gave_up = c->gave_up;
        __threadfence_system();
        hm->done = stop ? 1 : 0;
    }
    cudaGraphSetConditional(h, stop ? 0u : 1u);
}

// ------------------------------------------------------------------------------------------
// phase A: broadband rays (cast_ray_distributed, TaskAll:347-424)
// ------------------------------------------------------------------------------------------
// SMALL: scenes of at most kFuseMaxTris triangles walk with the plain stack (see stack_push).
template <bool MAP, bool SMALL>
__global__ void __launch_bounds__(128) k_broadband(DevRun r) {
    extern __shared__ float4 s_rec_buf[];
    const int *s_rid;
    const float4 *s_rec = stage_receivers(r, s_rec_buf, s_rid);
    LocalCounters L;
    const DevScene &S = r.S;
    WaveCtl *c = r.ctl;
    const long long p0 = c->pa_begin, cnt = c->pa_count;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += stride) {
        const long long prim = p0 + i;
        const int room = room_of(r, prim);
        const RoomParams &P = r.rooms[room];
        // SourceCluster round robin (Classes_Sources.cs:712-722)
        const int s = P.src_begin + (int)((prim + 1) % P.nsrc);
        const float4 src = r.src[s];
        float w;
        float3 d = primary_dir(r, P.nsrc, (uint32_t)prim, (int)src.w, w);
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
            TraceWork tw;
            const bool hit = SMALL ? trace_ray<int>(S, P.bvh_root, P.t_eps, pos, d, plane, t, tri, tw)
                                   : trace_ray<int2>(S, P.bvh_root, P.t_eps, pos, d, plane, t, tri, tw);
            L.v[C_RET] += tw.retests;
            ++L.v[C_SEGA];
            if (!hit) {
                if (order > P.is_order) {
                    L.v[C_DET] += detect_broad(r, P, s_rec, s_rid, pos, d, 1e6f, t_sum, E, sc, (uint32_t)prim);
                    if constexpr (MAP) L.v[C_DET] += map_detect_broad(r.map, P, pos, d, 1e6f, t_sum, E, sc);
                }
#pragma unroll
                for (int o = 0; o < kBands; ++o) L.lost += (double)(E[o] * sc[o]);
                lost = true;
                break;
            }
            if (order > P.is_order) {
                L.v[C_DET] += detect_broad(r, P, s_rec, s_rid, pos, d, t, t_sum, E, sc, (uint32_t)prim);
                if constexpr (MAP) L.v[C_DET] += map_detect_broad(r.map, P, pos, d, t, t_sum, E, sc);
            }
            t_sum += (double)t * P.inv_c_d;
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
                smid[o] = P.pure_specular ? 0.f : m.z;
                tau[o] = (S.has_trans && !P.pure_specular) ? __ldg(S.trans + poly * kBands + o) : 0.f;
            }
            // Scatter_Early
            if (cos_t > 0.f) { n = n * -1.f; cos_t = -cos_t; }
            int nchild = 0;
#pragma unroll
            for (int o = 0; o < kBands; ++o) nchild += (E[o] != 0.f) ? (tau[o] > 0.f ? 3 : 1) : 0;
            unsigned long long slot = nchild ? atomicAdd(&c->tail, (unsigned long long)nchild) : 0ull;
#pragma unroll
            for (int o = 0; o < kBands; ++o) {
                if (E[o] == 0.f) continue;
                Ray ch = new_ray(pos, d, E[o] * smid[o], sc[o], t_sum, (uint32_t)prim, sid_early(k, o, 0), o, 3, plane,
                                 room);
                E[o] *= (1.f - smid[o]);
                const float4 U = draw(r.seed, (uint32_t)prim, ch.sid, 0u);
                ch.d = lambert(n, U.x, U.y);
                if (tau[o] > 0.f) {
                    const Ray tr = new_ray(pos, d, E[o] * tau[o], sc[o], t_sum, (uint32_t)prim, sid_early(k, o, 1), o, 0,
                                           plane, room);
                    E[o] *= (1.f - tau[o]);
                    Ray td = ch;
                    td.I = ch.I * tau[o];
                    ch.I *= (1.f - tau[o]);
                    td.d = ch.d * -1.f;
                    td.sid = sid_early(k, o, 2);
                    ring_store(r, slot++, to_item(tr));
                    ring_store(r, slot++, to_item(td));
                    L.v[C_OCT] += 2;
                }
                ring_store(r, slot++, to_item(ch));
                ++L.v[C_OCT];
            }
            d = d - n * (2.f * cos_t);
            eh = 0.f;
#pragma unroll
            for (int o = 0; o < kBands; ++o) eh = (o == P.h_oct) ? E[o] : eh;
            if (order >= P.max_broad && eh > kTP1) { ++L.v[C_CAP]; break; }
        } while (eh > kTP1);
        if (!lost) {
            const int nfin = P.oct_hi - P.oct_lo + 1;
            unsigned long long slot = atomicAdd(&c->tail, (unsigned long long)nfin);
#pragma unroll
            for (int o = 0; o < kBands; ++o) {
                if (o < P.oct_lo || o > P.oct_hi) continue;
                const Ray it = new_ray(pos, d, E[o], sc[o], t_sum, (uint32_t)prim, sid_final(o), o, 0, plane, room);
                ring_store(r, slot++, to_item(it));
                ++L.v[C_OCT];
            }
        }
        ++L.v[C_PRIM];
    }
    flush_counters(r, L);
}

// ------------------------------------------------------------------------------------------
// wave ordering: counting sort by (direction octant, Morton code of the origin cell) so that the
// rays of a warp start close together heading the same way and walk similar BVH paths
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ unsigned spread3(unsigned x) {  // 3 bits -> every third bit
    return (x & 1u) | ((x & 2u) << 2) | ((x & 4u) << 4);
}

__device__ __forceinline__ unsigned sort_key(const DevRun &r, float4 P, float4 D) {
    const int cx = min(max((int)((P.x - r.sort_lo[0]) * r.sort_inv[0]), 0), kSortGrid - 1);
    const int cy = min(max((int)((P.y - r.sort_lo[1]) * r.sort_inv[1]), 0), kSortGrid - 1);
    const int cz = min(max((int)((P.z - r.sort_lo[2]) * r.sort_inv[2]), 0), kSortGrid - 1);
    const unsigned morton = spread3((unsigned)cx) | (spread3((unsigned)cy) << 1) | (spread3((unsigned)cz) << 2);
    const unsigned oct = (D.x < 0.f ? 1u : 0u) | (D.y < 0.f ? 2u : 0u) | (D.z < 0.f ? 4u : 0u);
    return (oct << 9) | morton;
}

__global__ void __launch_bounds__(256) k_sort_count(DevRun r) {
    __shared__ unsigned h[kSortBins];
    for (int i = threadIdx.x; i < kSortBins; i += blockDim.x) h[i] = 0;
    __syncthreads();
    const unsigned long long m = r.ctl->m, head = r.ctl->head;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long j = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; j < m; j += stride) {
        const float4 *q = reinterpret_cast<const float4 *>(r.ring + ((head + j) & (r.ring_cap - 1)));
        atomicAdd(&h[sort_key(r, __ldg(q), __ldg(q + 1))], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kSortBins; i += blockDim.x)
        if (h[i]) atomicAdd(&r.bin_count[i], h[i]);
}

// One block of 1024 threads, 4 bins each: exclusive scan into the cursors; clears the counts.
__global__ void __launch_bounds__(1024) k_sort_scan(DevRun r) {
    __shared__ unsigned warp_sum[32];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    unsigned c[4], s = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        c[k] = r.bin_count[4 * t + k];
        r.bin_count[4 * t + k] = 0;
        s += c[k];
    }
    unsigned incl = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned v = __shfl_up_sync(FULL, incl, o);
        if (lane >= o) incl += v;
    }
    if (lane == 31) warp_sum[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        unsigned w = warp_sum[lane], wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned v = __shfl_up_sync(FULL, wi, o);
            if (lane >= o) wi += v;
        }
        warp_sum[lane] = wi - w;  // exclusive warp offsets
    }
    __syncthreads();
    unsigned run = warp_sum[warp] + incl - s;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        r.bin_cursor[4 * t + k] = run;
        run += c[k];
    }
}

__global__ void __launch_bounds__(256) k_sort_scatter(DevRun r) {
    const unsigned long long m = r.ctl->m, head = r.ctl->head;
    const unsigned long long m32 = (m + 31) & ~31ull;
    const int lane = threadIdx.x & 31;
    const unsigned long long warp0 = ((unsigned long long)blockIdx.x * blockDim.x + threadIdx.x) & ~31ull;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long base = warp0; base < m32; base += stride) {
        const unsigned long long j = base + lane;
        const bool act = j < m;
        const unsigned amask = __ballot_sync(FULL, act);
        if (!act) continue;
        const ORayItem it = load_item(r.ring, (head + j) & (r.ring_cap - 1));
        const float4 *f = reinterpret_cast<const float4 *>(&it);
        const unsigned key = sort_key(r, f[0], f[1]);
        const unsigned peers = __match_any_sync(amask, key);
        const int leader = __ffs(peers) - 1;
        unsigned pos = 0;
        if (lane == leader) pos = atomicAdd(&r.bin_cursor[key], (unsigned)__popc(peers));
        pos = __shfl_sync(amask, pos, leader) + __popc(peers & ((1u << lane) - 1u));
        store_item(r.wave_buf, pos, it);
    }
}

// ------------------------------------------------------------------------------------------
// phases B and C, split into the BVH walk and the surface interaction
// ------------------------------------------------------------------------------------------
// The walk's result for wave slot j: the nearest triangle (-1: none), its distance, and the polygon and
// coplanar group the shading pass needs (read from the triangle record, which the walk has just tested).
__device__ __forceinline__ void write_hit(const DevRun &r, const DevScene &S, unsigned j, int tri, float t) {
    int poly = -1, plane = -1;
    if (tri >= 0) {
        plane = __ldg(reinterpret_cast<const int *>(S.tri + 3 * tri) + 3);
        poly = __ldg(reinterpret_cast<const int *>(S.tri + 3 * tri + 1) + 3);
    }
    r.hits[j] = make_int4(tri, __float_as_int(t), poly, plane);
}

// The speculative walk tests the warp's leaves once at most kSpecSlack lanes are still looking for
// their first leaf (and some lane holds one) instead of waiting for the last: leaves tested sooner
// shrink the best hit sooner (fewer nodes and triangles per ray) and the warp idles less.  Measured
// on the arena (500k triangles) for 0 / 2 / 8 / 10 / 12 / 16 / 24 / 31: 1.65 / 1.73 / 1.78 / 1.80 /
// 1.79 / 1.76 / 1.58 / 1.23 G segments/s; on the 20k-triangle hall 0 / 8 / 12: 1.82 / 1.99 / 1.97.
constexpr int kSpecSlack = 10;

// Persistent BVH walk with dynamic ray fetch: every loop iteration a lane descends inner nodes to
// its next leaf and tests it; a lane whose walk has ended writes its hit and takes the next wave
// item at once (one ticket atomic per warp), so a warp does not idle on its slowest lane.
// Values the walk needs only when a ray starts or ends, once per leaf or once per warp iteration live
// in shared memory (each lane's wave index, the plane it leaves and its hit tolerance; each warp's node
// and triangle counts), not in registers: the walk's 40 registers already spill.  The counts are taken
// in kernel-timing runs only (r.count_work): they cost a ballot and a shared-memory update per pass.
template <int MINB, bool SPEC, bool QUANT>
__global__ void __launch_bounds__(256, MINB) k_trace(DevRun r) {
    __shared__ unsigned s_item[256];
    __shared__ int s_skip[256];
    __shared__ float s_teps[256];
    __shared__ unsigned long long s_cnt[8][2];
    WaveCtl *c = r.ctl;
    const unsigned long long m = c->m, head = c->head;
    const DevScene &S = r.S;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) s_cnt[wid][0] = s_cnt[wid][1] = 0;
    __syncwarp();
    TraceWork w;
    bool have = false, exhausted = false;
    unsigned j = 0;  // index in the wave (a wave holds at most half the ring: < 2^31 items)
    float3 o = make_float3(0.f, 0.f, 0.f), d = o;
    float ix = 0.f, iy = 0.f, iz = 0.f, ox = 0.f, oy = 0.f, oz = 0.f, best = FLT_MAX;
    int skip = -1, node = 0, sp = 0, bi = -1, leaf = 0;
    float teps = S.t_eps;
    int2 stack[kBvhStack];
    for (;;) {
        const unsigned need = __ballot_sync(FULL, !have && !exhausted);
        if (need) {
            const int leader = __ffs(need) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(&c->trace_next, (unsigned long long)__popc(need));
            base = __shfl_sync(FULL, base, leader);
            if (!have && !exhausted) {
                const unsigned long long jj = base + __popc(need & ((1u << lane) - 1u));
                j = (unsigned)jj;
                if (jj < m) {
                    const float4 *q = reinterpret_cast<const float4 *>(wave_item(r, head, j));
                    const float4 P = __ldcs(q), D = __ldcs(q + 1), X = __ldcs(q + 3);
                    o = f3(P);
                    d = f3(D);
                    skip = __float_as_int(X.w);
                    const int room = (int)(__float_as_uint(X.z) >> 6);
                    const float dx = fabsf(d.x) < 1e-20f ? copysignf(1e-20f, d.x) : d.x;
                    const float dy = fabsf(d.y) < 1e-20f ? copysignf(1e-20f, d.y) : d.y;
                    const float dz = fabsf(d.z) < 1e-20f ? copysignf(1e-20f, d.z) : d.z;
                    ix = 1.0f / dx; iy = 1.0f / dy; iz = 1.0f / dz;
                    if constexpr (!QUANT) { ox = o.x * ix; oy = o.y * iy; oz = o.z * iz; }
                    node = r.n_rooms > 1 ? __ldg(&r.rooms[room].bvh_root) : 0;
                    teps = r.n_rooms > 1 ? __ldg(&r.rooms[room].t_eps) : S.t_eps;
                    if constexpr (SPEC) {
                        s_item[threadIdx.x] = j;
                        s_skip[threadIdx.x] = skip;
                        s_teps[threadIdx.x] = teps;
                    }
                    sp = 0; best = FLT_MAX; bi = -1;
                    have = true;
                } else {
                    exhausted = true;
                }
            }
        }
        if (!__any_sync(FULL, have)) break;
        if constexpr (SPEC) {
            // Speculative walk: a lane that has found a leaf keeps descending inner nodes while any
            // lane of the warp is still looking for its first leaf; then the warp tests its leaves
            // together.  node: >= 0 inner node, < 0 leaf, kEmptyChild nothing left; leaf: 0 none.
            if (have && node < 0 && node != kEmptyChild && leaf == 0) {
                leaf = node;
                node = stack_pop(stack, sp, best);
            }
            for (;;) {
                // stop when no lane is still looking for its first leaf, or when at most kSpecSlack are
                // and some lane holds a leaf to test (every pass of this loop advances the lanes still
                // looking, so it ends)
                const int looking = __popc(__ballot_sync(FULL, have && node >= 0 && leaf == 0));
                if (looking == 0 || (looking <= kSpecSlack && __any_sync(FULL, have && leaf != 0))) break;
                if (r.count_work) {
                    const unsigned stepping = __ballot_sync(FULL, have && node >= 0);
                    if (lane == 0) s_cnt[wid][0] += (unsigned)__popc(stepping);
                }
                if (have && node >= 0) {
                    int next;
                    if (QUANT ? bvh4q_step(S.bvhq, node, ix, iy, iz, o.x, o.y, o.z, best, stack, sp, next)
                              : bvh4_step(S.bvh, node, ix, iy, iz, ox, oy, oz, best, stack, sp, next))
                        node = next;
                    else node = stack_pop(stack, sp, best);
                    if (node < 0 && node != kEmptyChild && leaf == 0) {
                        leaf = node;
                        node = stack_pop(stack, sp, best);
                    }
                }
            }
            const bool testing = have && leaf != 0;
            if (r.count_work) {
                const unsigned ntri = __reduce_add_sync(FULL, testing ? (unsigned)(((~leaf) & 15) + 1) : 0u);
                if (lane == 0) s_cnt[wid][1] += ntri;
            }
            if (testing) {
                const int code = ~leaf;
                const int f0 = code >> 4, cnt = (code & 15) + 1;
                const int sk = s_skip[threadIdx.x];
                const float te = s_teps[threadIdx.x];
                for (int k = 0; k < cnt; ++k) test_tri(S, te, f0 + k, o, d, sk, best, bi, w);
                leaf = 0;
            }
            if (have && node == kEmptyChild) {
                write_hit(r, S, s_item[threadIdx.x], bi, best);
                have = false;
            }
        } else {
            if (!have) continue;
            while (node >= 0) {
                ++w.nodes;
                int next;
                node = (QUANT ? bvh4q_step(S.bvhq, node, ix, iy, iz, o.x, o.y, o.z, best, stack, sp, next)
                              : bvh4_step(S.bvh, node, ix, iy, iz, ox, oy, oz, best, stack, sp, next))
                           ? next
                           : stack_pop(stack, sp, best);
            }
            const bool fin = node == kEmptyChild;
            if (!fin) {
                const int code = ~node;
                const int f0 = code >> 4, cnt = (code & 15) + 1;
                w.tris += (unsigned)cnt;
                for (int k = 0; k < cnt; ++k) test_tri(S, teps, f0 + k, o, d, skip, best, bi, w);
                node = stack_pop(stack, sp, best);
            }
            if (node == kEmptyChild) {
                write_hit(r, S, j, bi, best);
                have = false;
            }
        }
    }
    // one atomic per warp for each counter
    unsigned long long a = w.retests, b = w.nodes, c2 = w.tris;
    if constexpr (SPEC) {
        __syncwarp();
        b = lane == 0 ? s_cnt[wid][0] : 0;
        c2 = lane == 0 ? s_cnt[wid][1] : 0;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(FULL, a, o);
        b += __shfl_down_sync(FULL, b, o);
        c2 += __shfl_down_sync(FULL, c2, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (a) atomicAdd(&r.cnt->retests, a);
        if (b) atomicAdd(&r.cnt->bvh_nodes, b);
        if (c2) atomicAdd(&r.cnt->tri_tests, c2);
    }
}

// FUSED: walk the ray here instead of reading k_trace's hit (small scenes, whose walk is a few
// cached nodes: the separate trace pass would only re-read the ray and round-trip its hit via HBM).
// the shading pass alone fits three 256-thread blocks per SM (80 registers; +1.6 % on a 500k-triangle
// arena, equal on a 20k-triangle hall); the fused walk, two (128 registers).  WIDE, for rooms of many
// receivers: the grouped detection and four blocks per SM (64 registers, more spilled: the long
// detection loop waits on its loads) -- on the 64-receiver arena -6 % shading time from the fourth
// block, -28 % more from the grouped detection; on the 16-receiver hall +17 % and +12 %, so it keeps
// three blocks and the plain loop.
constexpr int kShadeMinBlocks = 3;
template <bool FUSED, bool MAP, bool WIDE = false>
__global__ void __launch_bounds__(256, FUSED ? 2 : (WIDE ? 4 : kShadeMinBlocks)) k_shade(DevRun r) {
    extern __shared__ float4 s_rec_buf[];
    const int *s_rid;
    const float4 *s_rec = stage_receivers(r, s_rec_buf, s_rid);
    LocalCounters L;
    const DevScene &S = r.S;
    WaveCtl *c = r.ctl;
    const unsigned long long m = c->m, head = c->head;
    const unsigned long long m32 = (m + 31) & ~31ull;
    const int lane = threadIdx.x & 31;
    const unsigned long long warp0 = ((unsigned long long)blockIdx.x * blockDim.x + threadIdx.x) & ~31ull;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long base = warp0; base < m32; base += stride) {
        const unsigned long long j = base + lane;
        int nout = 0;
        Ray R, C;
        if (j < m) {
            R = to_ray(load_item(wave_item(r, head, j), 0));
            int4 h;  // (triangle, t bits, polygon, coplanar group)
            if constexpr (FUSED) {
                float tt;
                int tri;
                TraceWork tw;
                const int root = r.n_rooms > 1 ? __ldg(&r.rooms[R.room].bvh_root) : 0;
                const float teps = r.n_rooms > 1 ? __ldg(&r.rooms[R.room].t_eps) : S.t_eps;
                h = make_int4(-1, 0, -1, -1);
                if (trace_ray<int>(S, root, teps, R.p, R.d, R.plane, tt, tri, tw)) {
                    const float4 A = __ldg(S.tri + 3 * tri), B = __ldg(S.tri + 3 * tri + 1);
                    h = make_int4(tri, __float_as_int(tt), __float_as_int(B.w), __float_as_int(A.w));
                }
                L.v[C_RET] += tw.retests;
            } else {
                h = r.hits[j];
            }
            const bool hit = h.x >= 0;
            const float t = __int_as_float(h.y);
            ++L.v[R.phase == 0 ? C_SEGB : C_SEGC];
            const RoomParams &P = r.rooms[R.room];
            L.v[C_DET] += detect_octave<WIDE>(r, P, s_rec, s_rid, R.p, R.d, hit ? t : 1e6f, R.t_sum, R.I * R.scale, R.oct,
                                        R.mask, R.prim);
            if constexpr (MAP)
                L.v[C_DET] += map_detect_octave(r.map, P, R.p, R.d, hit ? t : 1e6f, R.t_sum, R.I * R.scale, R.oct);
            if (!hit) {
                // lost: no End_Trace after a miss in phase B (TaskAll:437-443), loop exit in phase C (500-505)
                L.lost += (double)(R.I * R.scale);
            } else {
                R.t_sum += (double)t * P.inv_c_d;
                R.p = R.p + R.d * t;
                R.plane = h.w;
                const int poly = h.z;
                const float3 n = f3(__ldg(S.pnormal + poly));
                const float cos_t = dot3(n, R.d);
                const float4 mt = __ldg(S.mat + poly * kBands + R.oct);  // (1-alpha, s_lo, s_mid, s_hi)
                R.I *= mt.x;
                const float4 U = draw(r.seed, R.prim, R.sid, 1u + R.nb);
                const uint32_t nb = R.nb++;
                const bool transmit = S.has_trans && !P.pure_specular && U.x < __ldg(S.trans + poly * kBands + R.oct);
                const float3 spec = R.d - n * (2.f * cos_t);
                const float3 nn = cos_t > 0.f ? n * -1.f : n;
                bool alive = true;
                bool split = false;
                if (R.phase == 0) {
                    // Scatter_Late
                    if (P.pure_specular || U.y > mt.w) {
                        R.d = transmit ? spec * -1.f : spec;
                        R.mask &= ~1;
                    } else {
                        if (U.y > mt.y) {
                            split = true;
                            C = R;
                            C.I = R.I * (1.f - mt.z);
                            R.I *= mt.z;
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
                    }
                    // phase-B loop test (TaskAll:473): failing it enters End_Trace, which always
                    // traces at least one more segment
                    if (!(R.t_sum < P.cotime && R.I > kTP2)) { R.phase = 1; ++L.v[C_END]; }
                } else {
                    // Scatter_VeryLate
                    if (!P.pure_specular && U.y < mt.z) {
                        R.d = lambert(nn, U.z, U.w);
                        R.mask |= 3;
                    } else {
                        R.d = spec;
                        R.mask &= ~1;
                    }
                    if (transmit) R.d = R.d * -1.f;
                    alive = R.t_sum < P.cotime && R.I > kTP3;  // TaskAll:534
                }
                if (alive && (long long)R.nb >= r.max_seg) { ++L.v[C_CAP]; alive = false; }
                if (!alive && split) { R = C; split = false; alive = true; }
                nout = (alive ? 1 : 0) + (split ? 1 : 0);
            }
        }
        const unsigned long long slot = warp_append(&c->tail, nout);
        if (nout >= 1) ring_store(r, slot, to_item(R));
        if (nout == 2) ring_store(r, slot + 1, to_item(C));
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
    TraceWork rt;
    for (int b = 0; b < maxb; ++b) {
        const size_t k = (size_t)i * maxb + b;
        poly[k] = -1; tout[k] = 0; pts[3 * k] = pts[3 * k + 1] = pts[3 * k + 2] = 0;
    }
    for (int b = 0; b < maxb; ++b) {
        float t;
        int tri;
        if (!trace_ray(S, 0, S.t_eps, p, d, plane, t, tri, rt)) break;
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
    const RoomParams &P = r.rooms[0];
    const int s = P.src_begin + (int)((prim + 1) % P.nsrc);
    const float3 d = emit_dir(r, P.nsrc, prim, (int)r.src[s].w);
    out[3 * i] = d.x; out[3 * i + 1] = d.y; out[3 * i + 2] = d.z;
}

// Direct-sound visibility (Direct_Sound.Check_Validity, Classes_Direct.cs:654-685): from each
// source towards each receiver, shoot; a hit before the receiver distance through a transmissive
// polygon multiplies the band transmission and the ray continues from the hit point, comparing its
// next hit with the full source-receiver distance again (as coded); any other hit decides.
__global__ void k_direct(DevScene S, const double *src, int nsrc, const double *rec, int nrec, int max_cross,
                         int *valid, double *transmod) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nsrc * nrec) return;
    const int k = p / nsrc, s = p % nsrc;
    const double dx = rec[3 * k] - src[3 * s], dy = rec[3 * k + 1] - src[3 * s + 1], dz = rec[3 * k + 2] - src[3 * s + 2];
    const double dist = sqrt(dx * dx + dy * dy + dz * dz);
    float3 o = make_float3((float)src[3 * s], (float)src[3 * s + 1], (float)src[3 * s + 2]);
    const float3 d = make_float3((float)(dx / dist), (float)(dy / dist), (float)(dz / dist));
    double tm[kBands];
#pragma unroll
    for (int b = 0; b < kBands; ++b) tm[b] = 1.0;
    int plane = -1, ok = 1;
    for (int c = 0; c < max_cross; ++c) {
        float t;
        int tri;
        TraceWork w;
        if (!trace_ray(S, 0, S.t_eps, o, d, plane, t, tri, w)) { ok = 1; break; }
        ok = (double)t >= dist ? 1 : 0;
        const float4 A = __ldg(S.tri + 3 * tri), B = __ldg(S.tri + 3 * tri + 1);
        const int poly = __float_as_int(B.w);
        bool transmissive = false;
        if (S.has_trans)
            for (int b = 0; b < kBands; ++b) transmissive = transmissive || __ldg(S.trans + poly * kBands + b) > 0.f;
        if (ok || !transmissive) break;
        for (int b = 0; b < kBands; ++b) tm[b] *= (double)__ldg(S.trans + poly * kBands + b);
        o = o + d * t;
        plane = __float_as_int(A.w);
    }
    valid[p] = ok;
#pragma unroll
    for (int b = 0; b < kBands; ++b) transmod[(size_t)p * kBands + b] = tm[b];
}

__global__ void k_prop_sample(DevRun r, long long p0, int n, float *dirs, float *weights) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float w;
    const float3 d = proposal_dir(r, (uint32_t)(p0 + i), w);
    dirs[3 * i] = d.x; dirs[3 * i + 1] = d.y; dirs[3 * i + 2] = d.z;
    weights[i] = w;
}

}  // namespace

// ------------------------------------------------------------------------------------------
// host wrappers
// ------------------------------------------------------------------------------------------
static size_t rec_smem(const DevRun &r) { return (size_t)receiver_smem_bytes(r.R); }

cudaError_t launch_feed(const DevRun &r, cudaStream_t s) {
    k_feed<<<1, 32, 0, s>>>(r);
    return cudaGetLastError();
}

cudaError_t launch_broadband(const DevRun &r, int blocks, int threads, cudaStream_t s, bool map, bool small) {
    if (map) {
        if (small) k_broadband<true, true><<<blocks, threads, rec_smem(r), s>>>(r);
        else k_broadband<true, false><<<blocks, threads, rec_smem(r), s>>>(r);
    } else {
        if (small) k_broadband<false, true><<<blocks, threads, rec_smem(r), s>>>(r);
        else k_broadband<false, false><<<blocks, threads, rec_smem(r), s>>>(r);
    }
    return cudaGetLastError();
}

cudaError_t launch_wave(const DevRun &r, cudaStream_t s) {
    k_wave<<<1, 32, 0, s>>>(r);
    return cudaGetLastError();
}

cudaError_t launch_cond(const DevRun &r, cudaGraphConditionalHandle h, cudaStream_t s) {
    k_cond<<<1, 32, 0, s>>>(r, h);
    return cudaGetLastError();
}

cudaError_t launch_sort(const DevRun &r, int blocks, cudaStream_t s) {
    k_sort_count<<<blocks, 256, 0, s>>>(r);
    k_sort_scan<<<1, 1024, 0, s>>>(r);
    k_sort_scatter<<<blocks, 256, 0, s>>>(r);
    return cudaGetLastError();
}

// variant = blocks per SM (3..6) + 16 x speculative + 32 x quantised nodes
#define PACH_TRACE_VARIANTS(X)                                                                         \
    X(3, false, false) X(4, false, false) X(5, false, false) X(6, false, false) X(4, true, false)    \
    X(6, true, false) X(4, false, true) X(6, false, true) X(4, true, true) X(6, true, true)

cudaError_t launch_trace(const DevRun &r, int variant, int blocks, int threads, cudaStream_t s) {
    switch (variant) {
#define PACH_LAUNCH(M, SP, Q) \
    case M + (SP ? 16 : 0) + (Q ? 32 : 0): k_trace<M, SP, Q><<<blocks, threads, 0, s>>>(r); break;
        PACH_TRACE_VARIANTS(PACH_LAUNCH)
#undef PACH_LAUNCH
        default: k_trace<4, false, false><<<blocks, threads, 0, s>>>(r); break;
    }
    return cudaGetLastError();
}

cudaError_t launch_shade(const DevRun &r, int blocks, int threads, cudaStream_t s, bool fused, bool map, bool wide) {
    if (map) {
        if (fused) k_shade<true, true><<<blocks, threads, rec_smem(r), s>>>(r);
        else k_shade<false, true><<<blocks, threads, rec_smem(r), s>>>(r);
    } else {
        if (fused) k_shade<true, false><<<blocks, threads, rec_smem(r), s>>>(r);
        else if (wide) k_shade<false, false, true><<<blocks, threads, rec_smem(r), s>>>(r);
        else k_shade<false, false><<<blocks, threads, rec_smem(r), s>>>(r);
    }
    return cudaGetLastError();
}

cudaError_t wave_kernel_occupancy(int variant, int threads, int smem_shade, int *bpsm_trace, int *bpsm_shade,
                                  bool fused, bool wide) {
    cudaError_t e;
    switch (variant) {
#define PACH_OCC(M, SP, Q)                                                                           \
    case M + (SP ? 16 : 0) + (Q ? 32 : 0):                                                           \
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(bpsm_trace, k_trace<M, SP, Q>, threads, 0); \
        break;
        PACH_TRACE_VARIANTS(PACH_OCC)
#undef PACH_OCC
        default: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(bpsm_trace, k_trace<4, false, false>, threads, 0); break;
    }
    if (e != cudaSuccess) return e;
    if (fused) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(bpsm_shade, k_shade<true, false>, threads, smem_shade);
    if (wide) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(bpsm_shade, k_shade<false, false, true>, threads, smem_shade);
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(bpsm_shade, k_shade<false, false>, threads, smem_shade);
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

cudaError_t launch_direct(const DevScene &S, const double *src, int nsrc, const double *rec, int nrec, int max_cross,
                          int *valid, double *transmod, cudaStream_t s) {
    const int n = nsrc * nrec;
    k_direct<<<(n + 127) / 128, 128, 0, s>>>(S, src, nsrc, rec, nrec, max_cross, valid, transmod);
    return cudaGetLastError();
}

cudaError_t launch_prop_sample(const DevRun &r, long long p0, int n, float *dirs, float *weights, cudaStream_t s) {
    k_prop_sample<<<(n + 127) / 128, 128, 0, s>>>(r, p0, n, dirs, weights);
    return cudaGetLastError();
}

}  // namespace pach
