// mlp.cu -- the learned emission proposal's network: BF16 tensor-core (tcgen05) training and inference.
//
// Network 12 -> 256 -> 256 -> 256 -> 160, exact GELU, output 32 von Mises-Fisher lobes
// (mean direction, log kappa, logit).  Loss: cross-entropy of a per-bin target distribution over
// emission-direction bins against the mixture density at the bin centres.
//
// Every matrix product runs in k_gemm: C[M][N] = A[M][K] . B[N][K]^T with both operands K-major BF16
// in the blocked layout below, one 128-row tile of C per CTA (up to 256 columns), FP32 accumulators in
// tensor memory.  One thread streams K in chunks of 64 through a three-stage ring of shared-memory
// buffers with bulk asynchronous copies (cp.async.bulk, completion on an mbarrier) and issues
// tcgen05.mma (kind::f16, M = 128, N <= 128 per instruction, K = 16); tcgen05.commit frees a stage
// when the MMAs reading it are done.  The four warps then read their 32 accumulator lanes with
// tcgen05.ld and run a fused epilogue (bias, GELU or GELU', BF16 stores in both the blocked and the
// transposed blocked layout, bias-gradient column sums).
//
// Blocked layout ("canonical K-major, no swizzle"): a [rows][K] matrix (rows padded to 128, K a
// multiple of 16) is a sequence of 128-row tiles; a tile is K/8 slabs of 8 columns, 2048 bytes each;
// a slab is 16 core matrices of 8 rows x 16 bytes.  So a 128 x 64 chunk of a tile is one contiguous
// 16 KB block (one bulk copy), and the MMA descriptors use leading (K-direction) byte offset 2048 and
// stride (row-direction) byte offset 128.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "engine.h"
#include "../../include/pach_proposal.h"

namespace pach {
namespace mlp {

constexpr int kIn = PACH_MLP_IN;
constexpr int kInPad = 16;
constexpr int kHid = PACH_MLP_HIDDEN;
constexpr int kOut = PACH_MLP_OUT;
constexpr int kLobes = PACH_MLP_LOBES;
constexpr int kBins = PACH_DIR_BINS;
constexpr int kTile = 128;
constexpr int kChunk = 64;
constexpr int kStages = 3;
constexpr int kOperandBytes = kTile * kChunk * 2;        // one 128 x 64 BF16 block
constexpr int kStageBytes = 3 * kOperandBytes;          // A + two B tiles
// Slack after the stages: every address an MMA descriptor can form stays inside the allocation even if
// the two descriptor strides were read the other way round.
constexpr int kSlack = 32 * 1024;
constexpr int kSmemBytes = kStages * kStageBytes + kSlack + 256 + 1024;
constexpr long long kSpin = 1ll << 24;                  // bounded mbarrier polls
constexpr float kInScale = 0.1f;                        // inputs are metres / 10
constexpr float kLogKapMin = -3.0f, kLogKapMax = 6.0f;  // kappa in [0.05, 403]
constexpr int kMaxRows = 1 << 16;

enum Epi { EPI_F32 = 0, EPI_GELU = 1, EPI_DGELU = 2 };

__host__ __device__ __forceinline__ size_t blk(int row, int k, int K) {
    return ((size_t)(row >> 7) * (size_t)(K >> 3) + (size_t)(k >> 3)) * 1024 + (size_t)((row & 127) >> 3) * 64 +
           (size_t)((row & 7) << 3) + (size_t)(k & 7);
}

// ------------------------------------------------------------------------------------------
// PTX wrappers
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    for (long long i = 0; i < kSpin; ++i)
        if (mbar_try(bar, parity)) return true;
    return false;
}
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}
__device__ __forceinline__ void tmem_alloc(uint32_t slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor: start, leading (K-direction) and stride (row-direction) byte
// offsets, fixed field 0b001 at bit 46, no swizzle.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
           (1ull << 46);
}
// Instruction descriptor, kind::f16: FP32 accumulator (bits 4-5 = 1), A and B BF16 (bits 7-9, 10-12 = 1),
// both K-major, N >> 3 at bits 17-22, M >> 4 at bits 24-28.
__device__ __forceinline__ uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
// 32 lanes x 32 consecutive FP32 columns: thread t of the warp gets lane (warp base + t).
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_d(float z) {
    return 0.5f * (1.f + erff(z * 0.70710678118654752f)) + z * 0.39894228040143268f * expf(-0.5f * z * z);
}

// ------------------------------------------------------------------------------------------
// the GEMM
// ------------------------------------------------------------------------------------------
struct Gemm {
    const __nv_bfloat16 *A;  // blocked [Mp][K]
    const __nv_bfloat16 *B;  // blocked [roundup(N, 128)][K]
    int Mp, N, K;            // Mp % 128 == 0, N % 16 == 0, K % 16 == 0
    int epi;
    int m_valid;             // rows >= m_valid: not stored (EPI_F32), zero (EPI_GELU, EPI_DGELU)
    const float *bias;       // [N] or null
    float *out;              // EPI_F32: row-major [M][ld_out]
    int ld_out;
    float *pre;              // EPI_GELU writes, EPI_DGELU reads: row-major [Mp][ld_pre]
    int ld_pre;
    __nv_bfloat16 *ob;       // blocked [Mp][N] (K = N)
    __nv_bfloat16 *obt;      // blocked [roundup(N,128)][Mp] (K = Mp), the transpose
    float *colsum;           // [N] column sums of the EPI_DGELU result, or null
    int *err;
};

__global__ void __launch_bounds__(128, 1) k_gemm(Gemm g) {
    extern __shared__ unsigned char smem_raw[];
    unsigned char *smem = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t *bars = (uint64_t *)(smem + kStages * kStageBytes + kSlack);
    uint32_t *tmem_slot = (uint32_t *)(bars + 2 * kStages + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.x * kTile, n0 = blockIdx.y * 256;
    const int ncols = min(256, g.N - n0);
    const int ntiles = (ncols + 127) / 128;
    const int nch = (g.K + kChunk - 1) / kChunk;
    const uint32_t sbase = smem_u32(smem);
    const uint32_t bar0 = smem_u32(bars);
    const uint32_t done = bar0 + 8 * (2 * kStages);

    if (tid == 0) {
        for (int s = 0; s < 2 * kStages + 1; ++s) mbar_init(bar0 + 8 * s, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        tmem_alloc(smem_u32(tmem_slot), 256);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (tid == 0) {
        bool ok = true;
        int loaded = 0, consumed = 0;
        auto load = [&](int c) {
            const int s = c % kStages, k0 = c * kChunk, kc = min(kChunk, g.K - k0);
            const uint32_t bytes = (uint32_t)kTile * kc * 2;
            const uint32_t st = sbase + s * kStageBytes;
            mbar_expect_tx(bar0 + 8 * s, bytes * (1 + ntiles));
            bulk_g2s(st, g.A + blk(m0, k0, g.K), bytes, bar0 + 8 * s);
            for (int t = 0; t < ntiles; ++t)
                bulk_g2s(st + (1 + t) * kOperandBytes, g.B + blk(n0 + 128 * t, k0, g.K), bytes, bar0 + 8 * s);
            ++loaded;
        };
        for (int c = 0; c < min(kStages, nch); ++c) load(c);
        for (int c = 0; c < nch; ++c) {
            const int s = c % kStages;
            const uint32_t par = (uint32_t)(c / kStages) & 1u;
            if (!mbar_wait(bar0 + 8 * s, par)) { ok = false; break; }
            ++consumed;
            tc_fence_after();
            const int kc = min(kChunk, g.K - c * kChunk);
            const uint32_t st = sbase + s * kStageBytes;
            for (int kk = 0; kk < kc / 16; ++kk) {
                const uint64_t ad = sdesc(st + kk * 4096, 2048, 128);
                for (int t = 0; t < ntiles; ++t) {
                    const int nt = min(128, ncols - 128 * t);
                    const uint64_t bd = sdesc(st + (1 + t) * kOperandBytes + kk * 4096, 2048, 128);
                    mma_bf16(tmem + 128 * t, ad, bd, idesc_bf16(128, nt), (c > 0 || kk > 0) ? 1u : 0u);
                }
            }
            mma_commit(bar0 + 8 * (kStages + s));
            if (c + kStages < nch) {
                if (!mbar_wait(bar0 + 8 * (kStages + s), par)) { ok = false; break; }
                load(c + kStages);
            }
        }
        if (!ok) {
            atomicExch(g.err, 1);
            // let the copies already in flight land before the block exits
            for (int c = consumed; c < loaded; ++c) mbar_wait(bar0 + 8 * (c % kStages), (uint32_t)(c / kStages) & 1u);
        }
        mma_commit(done);
    }
    __syncwarp();
    const bool ready = __all_sync(0xffffffffu, mbar_wait(done, 0));
    tc_fence_after();
    if (!ready) {
        atomicExch(g.err, 2);
    } else {
        const int row = m0 + 32 * warp + lane;
        const bool live = row < g.m_valid;
        for (int j = 0; j < (ncols + 31) / 32; ++j) {
            float v[32];
            tmem_ld32(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(32 * j), v);
            const int cb = n0 + 32 * j;
            const int cn = min(32, g.N - cb);
            if (g.epi == EPI_F32) {
                if (live) {
                    float *o = g.out + (size_t)row * g.ld_out + cb;
#pragma unroll
                    for (int i = 0; i < 32; ++i)
                        if (i < cn) o[i] = v[i] + (g.bias ? __ldg(g.bias + cb + i) : 0.f);
                }
                continue;
            }
            if (g.epi == EPI_GELU) {
                float *pr = g.pre + (size_t)row * g.ld_pre + cb;
#pragma unroll
                for (int i = 0; i < 32; ++i) {
                    if (i < cn) {
                        const float z = v[i] + __ldg(g.bias + cb + i);
                        if (live) pr[i] = z;
                        v[i] = live ? gelu(z) : 0.f;
                    }
                }
            } else {  // EPI_DGELU
                const float *pr = g.pre + (size_t)row * g.ld_pre + cb;
#pragma unroll
                for (int i = 0; i < 32; ++i)
                    if (i < cn) v[i] = live ? v[i] * gelu_d(pr[i]) : 0.f;
                if (g.colsum) {
                    // lane L ends with the sum over the warp's 32 rows of column cb + L
                    float w[32];
#pragma unroll
                    for (int i = 0; i < 32; ++i) w[i] = (i < cn) ? v[i] : 0.f;
#pragma unroll
                    for (int off = 16; off >= 1; off >>= 1) {
                        const bool upper = (lane & off) != 0;
#pragma unroll
                        for (int i = 0; i < off; ++i) {
                            const float send = upper ? w[i] : w[i + off];
                            const float keep = upper ? w[i + off] : w[i];
                            w[i] = keep + __shfl_xor_sync(0xffffffffu, send, off);
                        }
                    }
                    if (lane < cn) atomicAdd(g.colsum + cb + lane, w[0]);
                }
            }
            // BF16 stores: this row's columns (8 per 16-byte group) and the transpose
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                if (8 * q < cn) {
                    __align__(16) __nv_bfloat16 h[8];
#pragma unroll
                    for (int i = 0; i < 8; ++i) h[i] = __float2bfloat16_rn(v[8 * q + i]);
                    *reinterpret_cast<uint4 *>(g.ob + blk(row, cb + 8 * q, g.N)) = *reinterpret_cast<const uint4 *>(h);
                }
            }
#pragma unroll
            for (int i = 0; i < 32; ++i)
                if (i < cn) g.obt[blk(cb + i, row, g.Mp)] = __float2bfloat16_rn(v[i]);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, 256);
}

// ------------------------------------------------------------------------------------------
// loss: cross-entropy of the bin target against the vMF mixture, and its gradient
// ------------------------------------------------------------------------------------------
struct Loss {
    const float *out;     // [Mp][160]
    const float *target;  // [M][kBins]
    const float4 *bins;   // [kBins] centre direction, solid angle
    int M, Mp;
    float scale;          // 1 / M
    __nv_bfloat16 *dob;   // blocked [Mp][160]
    __nv_bfloat16 *dobt;  // blocked [256][Mp]
    float *db;            // [160] output-bias gradient
    float *loss;          // [Mp] per-row loss
};

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
    for (int o = 16; o; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Lobe parameters from the raw outputs (shared with the tracer's sampler through lobes_host):
// mu = u / |u|, kappa = exp(clamp(s)), log weight = log softmax(a) + log(kappa / (2 pi (1 - e^-2kappa))).
__global__ void __launch_bounds__(256) k_vmf_loss(Loss a) {
    __shared__ float s_mu[kLobes][3], s_kap[kLobes], s_lw[kLobes], s_pi[kLobes], s_inv[kLobes], s_free[kLobes];
    __shared__ float s_acc[8][5][kLobes];
    __shared__ float s_l[8], s_p[8];
    const int m = blockIdx.x, tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (m >= a.M) {
        for (int j = tid; j < kOut; j += 256) {
            a.dob[blk(m, j, kOut)] = __float2bfloat16_rn(0.f);
            a.dobt[blk(j, m, a.Mp)] = __float2bfloat16_rn(0.f);
        }
        if (tid == 0) a.loss[m] = 0.f;
        return;
    }
    const float *o = a.out + (size_t)m * kOut;
    if (warp == 0) {
        const int k = lane;
        const float ux = o[5 * k], uy = o[5 * k + 1], uz = o[5 * k + 2], sr = o[5 * k + 3], lg = o[5 * k + 4];
        const float n = fmaxf(sqrtf(ux * ux + uy * uy + uz * uz), 1e-6f);
        const float s = fminf(fmaxf(sr, kLogKapMin), kLogKapMax);
        const float kap = expf(s);
        const float lnorm = s - 1.8378770664093453f - logf(-expm1f(-2.f * kap));  // log(2 pi) = 1.8378...
        const float mx = warp_max(lg);
        const float e = expf(lg - mx);
        const float se = warp_sum(e);
        s_mu[k][0] = ux / n;
        s_mu[k][1] = uy / n;
        s_mu[k][2] = uz / n;
        s_kap[k] = kap;
        s_pi[k] = e / se;
        s_lw[k] = (lg - mx - logf(se)) + lnorm;
        s_inv[k] = 1.f / n;
        s_free[k] = (sr > kLogKapMin && sr < kLogKapMax) ? 1.f : 0.f;
    }
    __syncthreads();
    const float mux = s_mu[lane][0], muy = s_mu[lane][1], muz = s_mu[lane][2], kap = s_kap[lane], lw = s_lw[lane];
    float R = 0.f, S = 0.f, Gx = 0.f, Gy = 0.f, Gz = 0.f, L = 0.f, P = 0.f;
    const float *tg = a.target + (size_t)m * kBins;
    for (int b = warp; b < kBins; b += 8) {
        const float p = __ldg(tg + b);
        if (p == 0.f) continue;
        const float4 d = __ldg(a.bins + b);
        const float cm = mux * d.x + muy * d.y + muz * d.z - 1.f;
        const float x = lw + kap * cm;
        const float mx = warp_max(x);
        const float val = expf(x - mx);
        const float q = warp_sum(val);
        const float r = p * (val / q);
        R += r;
        S += r * cm;
        Gx += r * d.x;
        Gy += r * d.y;
        Gz += r * d.z;
        L -= p * (mx + logf(q));
        P += p;
    }
    s_acc[warp][0][lane] = R;
    s_acc[warp][1][lane] = S;
    s_acc[warp][2][lane] = Gx;
    s_acc[warp][3][lane] = Gy;
    s_acc[warp][4][lane] = Gz;
    if (lane == 0) {
        s_l[warp] = L;
        s_p[warp] = P;
    }
    __syncthreads();
    if (warp == 0) {
        const int k = lane;
        float t[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
        float Lt = 0.f, Pt = 0.f;
        for (int w = 0; w < 8; ++w) {
#pragma unroll
            for (int i = 0; i < 5; ++i) t[i] += s_acc[w][i][k];
            Lt += s_l[w];
            Pt += s_p[w];
        }
        const float kp = s_kap[k];
        const float dA = s_pi[k] * Pt - t[0];
        const float dK = -(t[0] * (1.f / kp - 2.f / expm1f(2.f * kp)) + t[1]);
        const float dS = dK * kp * s_free[k];
        const float gx = -kp * t[2], gy = -kp * t[3], gz = -kp * t[4];
        const float mx_ = s_mu[k][0], my_ = s_mu[k][1], mz_ = s_mu[k][2];
        const float gm = gx * mx_ + gy * my_ + gz * mz_;
        const float iv = s_inv[k];
        const float g[5] = {(gx - gm * mx_) * iv, (gy - gm * my_) * iv, (gz - gm * mz_) * iv, dS, dA};
#pragma unroll
        for (int i = 0; i < 5; ++i) {
            const float v = g[i] * a.scale;
            const int j = 5 * k + i;
            a.dob[blk(m, j, kOut)] = __float2bfloat16_rn(v);
            a.dobt[blk(j, m, a.Mp)] = __float2bfloat16_rn(v);
            atomicAdd(a.db + j, v);
        }
        if (k == 0) a.loss[m] = Lt;
    }
}

// ------------------------------------------------------------------------------------------
// inputs, weights, optimiser
// ------------------------------------------------------------------------------------------
// cond [rows][12] metres -> blocked [Mp][16] and its transpose [128][Mp]
__global__ void k_pack_input(const float *cond, int rows, int Mp, __nv_bfloat16 *xb, __nv_bfloat16 *xt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= Mp * kInPad) return;
    const int r = i / kInPad, c = i % kInPad;
    const float v = (r < rows && c < kIn) ? cond[(size_t)r * kIn + c] * kInScale : 0.f;
    const __nv_bfloat16 h = __float2bfloat16_rn(v);
    xb[blk(r, c, kInPad)] = h;
    xt[blk(c, r, Mp)] = h;
}

struct Layer {
    int n, k;          // out, in (in padded to 16 for the first layer)
    size_t w, b;       // offsets of W [n][k] and b [n] in the master arrays
    __nv_bfloat16 *wb; // blocked [roundup(n,128)][k]
    __nv_bfloat16 *wt; // blocked [roundup(k,128)][n] (null for the first layer)
};

struct Pack {
    const float *w;
    Layer L[4];
    size_t total;      // weight elements over the four layers
};

__global__ void k_pack_weights(Pack p) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.total) return;
    size_t j = i;
    int l = 0;
    while (l < 3 && j >= (size_t)p.L[l].n * p.L[l].k) { j -= (size_t)p.L[l].n * p.L[l].k; ++l; }
    const Layer &L = p.L[l];
    const int n = (int)(j / L.k), k = (int)(j % L.k);
    const __nv_bfloat16 h = __float2bfloat16_rn(p.w[L.w + j]);
    L.wb[blk(n, k, L.k)] = h;
    if (L.wt) L.wt[blk(k, n, L.n)] = h;
}

__global__ void k_adam(float *w, float *m1, float *m2, const float *g, const unsigned char *decay, size_t n,
                       int *step, float lr, float wd) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int t = *step + 1;
    if (i >= n) return;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float gi = g[i];
    const float a = b1 * m1[i] + (1.f - b1) * gi;
    const float b = b2 * m2[i] + (1.f - b2) * gi * gi;
    m1[i] = a;
    m2[i] = b;
    const float bc1 = 1.f - powf(b1, (float)t), bc2 = 1.f - powf(b2, (float)t);
    float wi = w[i];
    if (decay[i]) wi -= lr * wd * wi;
    w[i] = wi - lr * (a / bc1) / (sqrtf(b / bc2) + eps);
}

__global__ void k_step(int *step) { ++*step; }

__global__ void k_loss_sum(const float *loss, int M, float scale, float *out, int slot) {
    __shared__ float s[256];
    float v = 0.f;
    for (int i = threadIdx.x; i < M; i += 256) v += loss[i];
    s[threadIdx.x] = v;
    __syncthreads();
    for (int o = 128; o; o >>= 1) {
        if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[slot] = s[0] * scale;
}

// ------------------------------------------------------------------------------------------
// host side
// ------------------------------------------------------------------------------------------
int round_up(int x, int m) { return (x + m - 1) / m * m; }

cudaError_t launch_gemm(const Gemm &g, cudaStream_t s) {
    static std::once_flag once;
    static cudaError_t attr = cudaSuccess;
    std::call_once(once, [] {
        attr = cudaFuncSetAttribute(k_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
    });
    if (attr != cudaSuccess) return attr;
    dim3 grid(g.Mp / kTile, (g.N + 255) / 256);
    k_gemm<<<grid, 128, kSmemBytes, s>>>(g);
    return cudaGetLastError();
}

struct Buf {
    void *p = nullptr;
    cudaError_t alloc(size_t bytes) {
        cudaError_t e = cudaMalloc(&p, bytes);
        if (e == cudaSuccess) e = cudaMemset(p, 0, bytes);
        return e;
    }
    ~Buf() {
        if (p) cudaFree(p);
    }
    template <class T> T *as() const { return (T *)p; }
};

}  // namespace mlp

// Public parameter order (W[out][in] row-major, then b) and the padded device order differ only in
// the first layer's 12 -> 16 columns.
static const int kLayerN[4] = {mlp::kHid, mlp::kHid, mlp::kHid, mlp::kOut};
static const int kLayerK[4] = {mlp::kIn, mlp::kHid, mlp::kHid, mlp::kHid};
static const int kLayerKPad[4] = {mlp::kInPad, mlp::kHid, mlp::kHid, mlp::kHid};

}  // namespace pach

using namespace pach;
using namespace pach::mlp;

struct pach_mlp {
    int device = 0;
    int max_rows = 0, Mp_max = 0;
    int rows = 0;          // training rows set
    bool x_train = false;  // xb/xt hold the training conditions
    cudaStream_t stream = nullptr;
    size_t n_dev = 0;  // padded parameter count
    Buf w, m1, m2, g, decay, step, err;
    Buf wb[4], wt[4];
    Buf xb, xt, hb[3], ht[3], pre[3], out, dob, dobt, dzb[3], dzt[3], target, loss, losses, bins;
    Buf cond_in, cond_train;
    Layer L[4];
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    float graph_lr = -1.f, graph_wd = -1.f;
    std::mutex mu;
    ~pach_mlp() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace {

std::string cu_msg(cudaError_t e, const char *what) {
    return std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
}

pach_status mfail(pach_status s, const std::string &m) {
    set_last_error(m.c_str());
    return s;
}

#define MTRY(x)                                                              \
    do {                                                                     \
        cudaError_t e_ = (x);                                                \
        if (e_ != cudaSuccess) return mfail(PACH_ERR_CUDA, cu_msg(e_, #x)); \
    } while (0)

// splitmix64-based uniform in [-1, 1)
struct Rng {
    uint64_t s;
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double sym() { return (double)(next() >> 11) * (2.0 / 9007199254740992.0) - 1.0; }
};

void direction_bins_host(std::vector<float> &dirs, std::vector<float> &omega) {
    dirs.assign(3 * kBins, 0.f);
    omega.assign(kBins, 0.f);
    auto F = [](double u, double v) { return std::atan2(u * v, std::sqrt(1.0 + u * u + v * v)); };
    for (int f = 0; f < 6; ++f)
        for (int j = 0; j < 16; ++j)
            for (int i = 0; i < 16; ++i) {
                const double u0 = i / 8.0 - 1.0, u1 = (i + 1) / 8.0 - 1.0, v0 = j / 8.0 - 1.0, v1 = (j + 1) / 8.0 - 1.0;
                const double uc = 0.5 * (u0 + u1), vc = 0.5 * (v0 + v1);
                const double sg = (f & 1) ? -1.0 : 1.0;
                double d[3];
                if (f < 2) { d[0] = sg; d[1] = uc; d[2] = vc; }
                else if (f < 4) { d[0] = uc; d[1] = sg; d[2] = vc; }
                else { d[0] = uc; d[1] = vc; d[2] = sg; }
                const double n = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                const int b = f * 256 + j * 16 + i;
                for (int c = 0; c < 3; ++c) dirs[3 * b + c] = (float)(d[c] / n);
                omega[b] = (float)(F(u1, v1) - F(u0, v1) - F(u1, v0) + F(u0, v0));
            }
}

size_t padded_offset(int l, bool bias) {
    size_t off = 0;
    for (int i = 0; i < l; ++i) off += (size_t)kLayerN[i] * kLayerKPad[i] + kLayerN[i];
    return bias ? off + (size_t)kLayerN[l] * kLayerKPad[l] : off;
}

int64_t public_count() {
    int64_t n = 0;
    for (int l = 0; l < 4; ++l) n += (int64_t)kLayerN[l] * kLayerK[l] + kLayerN[l];
    return n;
}

// public <-> padded device order
void to_padded(const float *pub, std::vector<float> &dev, size_t n_dev) {
    dev.assign(n_dev, 0.f);
    size_t p = 0;
    for (int l = 0; l < 4; ++l) {
        const size_t w = padded_offset(l, false), b = padded_offset(l, true);
        for (int n = 0; n < kLayerN[l]; ++n)
            for (int k = 0; k < kLayerK[l]; ++k) dev[w + (size_t)n * kLayerKPad[l] + k] = pub[p++];
        for (int n = 0; n < kLayerN[l]; ++n) dev[b + n] = pub[p++];
    }
}
void from_padded(const std::vector<float> &dev, float *pub) {
    size_t p = 0;
    for (int l = 0; l < 4; ++l) {
        const size_t w = padded_offset(l, false), b = padded_offset(l, true);
        for (int n = 0; n < kLayerN[l]; ++n)
            for (int k = 0; k < kLayerK[l]; ++k) pub[p++] = dev[w + (size_t)n * kLayerKPad[l] + k];
        for (int n = 0; n < kLayerN[l]; ++n) pub[p++] = dev[b + n];
    }
}

cudaError_t pack_weights(pach_mlp *m) {
    Pack p;
    p.w = m->w.as<float>();
    p.total = 0;
    for (int l = 0; l < 4; ++l) {
        p.L[l] = m->L[l];
        p.total += (size_t)m->L[l].n * m->L[l].k;
    }
    k_pack_weights<<<(unsigned)((p.total + 255) / 256), 256, 0, m->stream>>>(p);
    return cudaGetLastError();
}

// forward over Mp rows of xb/xt (rows valid), writes out [Mp][160]
cudaError_t forward(pach_mlp *m, int rows, int Mp) {
    for (int l = 0; l < 4; ++l) {
        Gemm g{};
        g.A = l == 0 ? m->xb.as<__nv_bfloat16>() : m->hb[l - 1].as<__nv_bfloat16>();
        g.B = m->L[l].wb;
        g.Mp = Mp;
        g.N = m->L[l].n;
        g.K = m->L[l].k;
        g.m_valid = rows;
        g.bias = m->w.as<float>() + m->L[l].b;
        g.err = m->err.as<int>();
        if (l < 3) {
            g.epi = EPI_GELU;
            g.pre = m->pre[l].as<float>();
            g.ld_pre = kHid;
            g.ob = m->hb[l].as<__nv_bfloat16>();
            g.obt = m->ht[l].as<__nv_bfloat16>();
        } else {
            g.epi = EPI_F32;
            g.out = m->out.as<float>();
            g.ld_out = kOut;
        }
        cudaError_t e = launch_gemm(g, m->stream);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// loss + backward over the training rows; gradients into m->g (padded order)
cudaError_t backward(pach_mlp *m, int rows, int Mp) {
    float *g = m->g.as<float>();
    cudaError_t e = cudaMemsetAsync(g, 0, m->n_dev * sizeof(float), m->stream);
    if (e != cudaSuccess) return e;
    Loss a{};
    a.out = m->out.as<float>();
    a.target = m->target.as<float>();
    a.bins = m->bins.as<float4>();
    a.M = rows;
    a.Mp = Mp;
    a.scale = 1.f / (float)rows;
    a.dob = m->dob.as<__nv_bfloat16>();
    a.dobt = m->dobt.as<__nv_bfloat16>();
    a.db = g + m->L[3].b;
    a.loss = m->loss.as<float>();
    k_vmf_loss<<<Mp, 256, 0, m->stream>>>(a);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    // layer l = 3..0: dW_l = dz_l^T h_{l-1}; dz_{l-1} = (dz_l W_l) * gelu'(pre_{l-1})
    for (int l = 3; l >= 0; --l) {
        const __nv_bfloat16 *dzb = l == 3 ? m->dob.as<__nv_bfloat16>() : m->dzb[l].as<__nv_bfloat16>();
        const __nv_bfloat16 *dzt = l == 3 ? m->dobt.as<__nv_bfloat16>() : m->dzt[l].as<__nv_bfloat16>();
        Gemm w{};
        w.A = dzt;
        w.B = l == 0 ? m->xt.as<__nv_bfloat16>() : m->ht[l - 1].as<__nv_bfloat16>();
        w.Mp = round_up(m->L[l].n, kTile);
        w.N = m->L[l].k;
        w.K = Mp;
        w.epi = EPI_F32;
        w.m_valid = m->L[l].n;
        w.out = g + m->L[l].w;
        w.ld_out = m->L[l].k;
        w.err = m->err.as<int>();
        if ((e = launch_gemm(w, m->stream)) != cudaSuccess) return e;
        if (l == 0) break;
        Gemm d{};
        d.A = dzb;
        d.B = m->L[l].wt;
        d.Mp = Mp;
        d.N = m->L[l].k;
        d.K = m->L[l].n;
        d.epi = EPI_DGELU;
        d.m_valid = rows;
        d.pre = m->pre[l - 1].as<float>();
        d.ld_pre = kHid;
        d.ob = m->dzb[l - 1].as<__nv_bfloat16>();
        d.obt = m->dzt[l - 1].as<__nv_bfloat16>();
        d.colsum = g + m->L[l - 1].b;
        d.err = m->err.as<int>();
        if ((e = launch_gemm(d, m->stream)) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t load_train_inputs(pach_mlp *m) {
    if (m->x_train) return cudaSuccess;
    const int Mp = round_up(m->rows, kTile);
    k_pack_input<<<(Mp * kInPad + 255) / 256, 256, 0, m->stream>>>(m->cond_train.as<float>(), m->rows, Mp,
                                                                    m->xb.as<__nv_bfloat16>(), m->xt.as<__nv_bfloat16>());
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) m->x_train = true;
    return e;
}

pach_status check_err(pach_mlp *m) {
    int h = 0;
    MTRY(cudaMemcpy(&h, m->err.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (h) {
        cudaMemset(m->err.p, 0, sizeof(int));
        return mfail(PACH_ERR_GAVE_UP, "tensor-core GEMM: a bounded barrier wait ran out (code " + std::to_string(h) + ")");
    }
    return PACH_OK;
}

}  // namespace

namespace pach {
// Raw outputs [n][160] -> per lobe two float4: (mu xyz, kappa), (log pi + log vMF norm, cumulative pi, 0, 0).
void proposal_lobes(const float *raw, int n, std::vector<float> &out) {
    out.assign((size_t)n * kLobes * 8, 0.f);
    for (int j = 0; j < n; ++j) {
        const float *o = raw + (size_t)j * kOut;
        double mx = -1e300;
        for (int k = 0; k < kLobes; ++k) mx = std::max(mx, (double)o[5 * k + 4]);
        double se = 0.0;
        for (int k = 0; k < kLobes; ++k) se += std::exp((double)o[5 * k + 4] - mx);
        double cdf = 0.0;
        for (int k = 0; k < kLobes; ++k) {
            const double ux = o[5 * k], uy = o[5 * k + 1], uz = o[5 * k + 2];
            const double nn = std::max(std::sqrt(ux * ux + uy * uy + uz * uz), 1e-6);
            const double s = std::min(std::max((double)o[5 * k + 3], (double)kLogKapMin), (double)kLogKapMax);
            const double kap = std::exp(s);
            const double lpi = (double)o[5 * k + 4] - mx - std::log(se);
            const double lnorm = s - std::log(2.0 * M_PI) - std::log(-std::expm1(-2.0 * kap));
            cdf += std::exp(lpi);
            float *L = &out[((size_t)j * kLobes + k) * 8];
            L[0] = (float)(ux / nn);
            L[1] = (float)(uy / nn);
            L[2] = (float)(uz / nn);
            L[3] = (float)kap;
            L[4] = (float)(lpi + lnorm);
            L[5] = (float)(k == kLobes - 1 ? 1.0 : cdf);
        }
    }
}
}  // namespace pach

extern "C" {

int64_t pach_mlp_param_count(void) { return public_count(); }

pach_status pach_mlp_create(uint64_t seed, int32_t max_rows, pach_mlp **out) {
    return guarded([&]() -> pach_status {
        if (!out) return mfail(PACH_ERR_INVALID_ARGUMENT, "out is null");
        *out = nullptr;
        if (max_rows < 1 || max_rows > kMaxRows) return mfail(PACH_ERR_INVALID_ARGUMENT, "max_rows must be 1..65536");
        int nd = 0;
        if (cudaGetDeviceCount(&nd) != cudaSuccess || nd < 1) return mfail(PACH_ERR_NO_DEVICE, "no CUDA device");
        pach_mlp *m = new pach_mlp();
        std::unique_ptr<pach_mlp> guard(m);
        MTRY(cudaGetDevice(&m->device));
        m->max_rows = max_rows;
        m->Mp_max = round_up(max_rows, kTile);
        const int Mp = m->Mp_max;
        MTRY(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking));
        m->n_dev = padded_offset(3, true) + kOut;
        for (int l = 0; l < 4; ++l) {
            Layer &L = m->L[l];
            L.n = kLayerN[l];
            L.k = kLayerKPad[l];
            L.w = padded_offset(l, false);
            L.b = padded_offset(l, true);
            MTRY(m->wb[l].alloc((size_t)round_up(L.n, kTile) * L.k * 2));
            L.wb = m->wb[l].as<__nv_bfloat16>();
            if (l > 0) {
                MTRY(m->wt[l].alloc((size_t)round_up(L.k, kTile) * L.n * 2));
                L.wt = m->wt[l].as<__nv_bfloat16>();
            } else {
                L.wt = nullptr;
            }
        }
        const size_t F = sizeof(float);
        MTRY(m->w.alloc(m->n_dev * F));
        MTRY(m->m1.alloc(m->n_dev * F));
        MTRY(m->m2.alloc(m->n_dev * F));
        MTRY(m->g.alloc(m->n_dev * F));
        MTRY(m->decay.alloc(m->n_dev));
        MTRY(m->step.alloc(sizeof(int)));
        MTRY(m->err.alloc(sizeof(int)));
        MTRY(m->xb.alloc((size_t)Mp * kInPad * 2));
        MTRY(m->xt.alloc((size_t)kTile * Mp * 2));
        for (int i = 0; i < 3; ++i) {
            MTRY(m->hb[i].alloc((size_t)Mp * kHid * 2));
            MTRY(m->ht[i].alloc((size_t)kHid * Mp * 2));
            MTRY(m->pre[i].alloc((size_t)Mp * kHid * F));
            MTRY(m->dzb[i].alloc((size_t)Mp * kHid * 2));
            MTRY(m->dzt[i].alloc((size_t)kHid * Mp * 2));
        }
        MTRY(m->out.alloc((size_t)Mp * kOut * F));
        MTRY(m->dob.alloc((size_t)Mp * kOut * 2));
        MTRY(m->dobt.alloc((size_t)round_up(kOut, kTile) * Mp * 2));
        MTRY(m->target.alloc((size_t)max_rows * kBins * F));
        MTRY(m->loss.alloc((size_t)Mp * F));
        MTRY(m->losses.alloc((size_t)1024 * F));
        MTRY(m->cond_in.alloc((size_t)max_rows * kIn * F));
        MTRY(m->cond_train.alloc((size_t)max_rows * kIn * F));
        {
            std::vector<float> d, om;
            direction_bins_host(d, om);
            std::vector<float4> b(kBins);
            for (int i = 0; i < kBins; ++i) b[i] = make_float4(d[3 * i], d[3 * i + 1], d[3 * i + 2], om[i]);
            MTRY(m->bins.alloc(kBins * sizeof(float4)));
            MTRY(cudaMemcpy(m->bins.p, b.data(), kBins * sizeof(float4), cudaMemcpyHostToDevice));
        }
        // seeded initialisation (public order): uniform(+-sqrt(6 / fan_in)) hidden weights, small output
        // weights, zero biases except log kappa = 1 (kappa e), so the first mixture is broad
        std::vector<float> pub((size_t)public_count());
        Rng rng{seed ^ 0x6D6C7050726F70ull};
        size_t p = 0;
        for (int l = 0; l < 4; ++l) {
            const double a = (l < 3) ? std::sqrt(6.0 / kLayerK[l]) : 0.5 / std::sqrt((double)kLayerK[l]);
            for (int i = 0; i < kLayerN[l] * kLayerK[l]; ++i) pub[p++] = (float)(a * rng.sym());
            for (int n = 0; n < kLayerN[l]; ++n) pub[p++] = (l == 3 && n % 5 == 3) ? 1.f : 0.f;
        }
        std::vector<float> dev;
        to_padded(pub.data(), dev, m->n_dev);
        MTRY(cudaMemcpy(m->w.p, dev.data(), m->n_dev * F, cudaMemcpyHostToDevice));
        std::vector<unsigned char> dec(m->n_dev, 0);
        for (int l = 0; l < 4; ++l)
            for (size_t i = 0; i < (size_t)kLayerN[l] * kLayerKPad[l]; ++i) dec[padded_offset(l, false) + i] = 1;
        MTRY(cudaMemcpy(m->decay.p, dec.data(), m->n_dev, cudaMemcpyHostToDevice));
        MTRY(pack_weights(m));
        MTRY(cudaStreamSynchronize(m->stream));
        *out = guard.release();
        return PACH_OK;
    }, mfail);
}

void pach_mlp_destroy(pach_mlp *m) { delete m; }

pach_status pach_mlp_get_params(pach_mlp *m, float *params, int64_t n) {
    return guarded([&]() -> pach_status {
        if (!m || !params || n < public_count()) return mfail(PACH_ERR_INVALID_ARGUMENT, "bad arguments");
        std::lock_guard<std::mutex> lk(m->mu);
        std::vector<float> dev(m->n_dev);
        MTRY(cudaMemcpy(dev.data(), m->w.p, m->n_dev * sizeof(float), cudaMemcpyDeviceToHost));
        from_padded(dev, params);
        return PACH_OK;
    }, mfail);
}

pach_status pach_mlp_set_params(pach_mlp *m, const float *params, int64_t n) {
    return guarded([&]() -> pach_status {
        if (!m || !params || n != public_count()) return mfail(PACH_ERR_INVALID_ARGUMENT, "bad arguments");
        std::lock_guard<std::mutex> lk(m->mu);
        std::vector<float> dev;
        to_padded(params, dev, m->n_dev);
        MTRY(cudaMemcpy(m->w.p, dev.data(), m->n_dev * sizeof(float), cudaMemcpyHostToDevice));
        MTRY(cudaMemset(m->m1.p, 0, m->n_dev * sizeof(float)));
        MTRY(cudaMemset(m->m2.p, 0, m->n_dev * sizeof(float)));
        MTRY(cudaMemset(m->step.p, 0, sizeof(int)));
        MTRY(pack_weights(m));
        MTRY(cudaStreamSynchronize(m->stream));
        return PACH_OK;
    }, mfail);
}

pach_status pach_mlp_set_data(pach_mlp *m, const float *cond, const float *target, int32_t rows) {
    return guarded([&]() -> pach_status {
        if (!m || !cond || !target || rows < 1 || rows > m->max_rows) return mfail(PACH_ERR_INVALID_ARGUMENT, "bad arguments");
        std::lock_guard<std::mutex> lk(m->mu);
        for (int64_t i = 0; i < (int64_t)rows * kIn; ++i)
            if (!std::isfinite(cond[i])) return mfail(PACH_ERR_INVALID_ARGUMENT, "cond holds a non-finite value");
        for (int64_t i = 0; i < (int64_t)rows * kBins; ++i)
            if (!(target[i] >= 0.f) || !std::isfinite(target[i]))
                return mfail(PACH_ERR_INVALID_ARGUMENT, "target must be finite and non-negative");
        MTRY(cudaMemcpyAsync(m->cond_train.p, cond, (size_t)rows * kIn * sizeof(float), cudaMemcpyHostToDevice, m->stream));
        MTRY(cudaMemcpyAsync(m->target.p, target, (size_t)rows * kBins * sizeof(float), cudaMemcpyHostToDevice, m->stream));
        MTRY(cudaStreamSynchronize(m->stream));
        m->rows = rows;
        m->x_train = false;
        if (m->exec) {  // the captured step holds the old row count
            cudaGraphExecDestroy(m->exec);
            cudaGraphDestroy(m->graph);
            m->exec = nullptr;
            m->graph = nullptr;
        }
        return PACH_OK;
    }, mfail);
}

pach_status pach_mlp_loss_grad(pach_mlp *m, float *loss, float *grad) {
    return guarded([&]() -> pach_status {
        if (!m || !loss) return mfail(PACH_ERR_INVALID_ARGUMENT, "bad arguments");
        std::lock_guard<std::mutex> lk(m->mu);
        if (m->rows < 1) return mfail(PACH_ERR_NOT_READY, "no training data (pach_mlp_set_data)");
        const int Mp = round_up(m->rows, kTile);
        MTRY(load_train_inputs(m));
        MTRY(forward(m, m->rows, Mp));
        MTRY(backward(m, m->rows, Mp));
        k_loss_sum<<<1, 256, 0, m->stream>>>(m->loss.as<float>(), m->rows, 1.f / m->rows, m->losses.as<float>(), 0);
        MTRY(cudaGetLastError());
        MTRY(cudaStreamSynchronize(m->stream));
        pach_status st = check_err(m);
        if (st != PACH_OK) return st;
        MTRY(cudaMemcpy(loss, m->losses.p, sizeof(float), cudaMemcpyDeviceToHost));
        if (grad) {
            std::vector<float> dev(m->n_dev);
            MTRY(cudaMemcpy(dev.data(), m->g.p, m->n_dev * sizeof(float), cudaMemcpyDeviceToHost));
            from_padded(dev, grad);
        }
        return PACH_OK;
    }, mfail);
}

pach_status pach_mlp_train(pach_mlp *m, int32_t steps, float lr, float weight_decay, float *loss_curve) {
    return guarded([&]() -> pach_status {
        if (!m || steps < 0 || !(lr > 0.f) || !(weight_decay >= 0.f)) return mfail(PACH_ERR_INVALID_ARGUMENT, "bad arguments");
        std::lock_guard<std::mutex> lk(m->mu);
        if (m->rows < 1) return mfail(PACH_ERR_NOT_READY, "no training data (pach_mlp_set_data)");
        const int Mp = round_up(m->rows, kTile);
        MTRY(load_train_inputs(m));
        if (!m->exec || m->graph_lr != lr || m->graph_wd != weight_decay) {
            if (m->exec) {
                cudaGraphExecDestroy(m->exec);
                cudaGraphDestroy(m->graph);
                m->exec = nullptr;
                m->graph = nullptr;
            }
            // warm the GEMM attribute outside capture
            MTRY(forward(m, m->rows, Mp));
            MTRY(cudaStreamSynchronize(m->stream));
            MTRY(cudaStreamBeginCapture(m->stream, cudaStreamCaptureModeThreadLocal));
            cudaError_t e = forward(m, m->rows, Mp);
            if (e == cudaSuccess) e = backward(m, m->rows, Mp);
            if (e == cudaSuccess) {
                k_loss_sum<<<1, 256, 0, m->stream>>>(m->loss.as<float>(), m->rows, 1.f / m->rows, m->losses.as<float>(), 0);
                k_adam<<<(unsigned)((m->n_dev + 255) / 256), 256, 0, m->stream>>>(
                    m->w.as<float>(), m->m1.as<float>(), m->m2.as<float>(), m->g.as<float>(), m->decay.as<unsigned char>(),
                    m->n_dev, m->step.as<int>(), lr, weight_decay);
                k_step<<<1, 1, 0, m->stream>>>(m->step.as<int>());
                e = cudaGetLastError();
                if (e == cudaSuccess) e = pack_weights(m);
            }
            cudaGraph_t gr = nullptr;
            cudaError_t e2 = cudaStreamEndCapture(m->stream, &gr);
            if (e != cudaSuccess || e2 != cudaSuccess) {
                if (gr) cudaGraphDestroy(gr);
                return mfail(PACH_ERR_CUDA, cu_msg(e != cudaSuccess ? e : e2, "capturing the training step"));
            }
            m->graph = gr;
            MTRY(cudaGraphInstantiate(&m->exec, m->graph, 0));
            m->graph_lr = lr;
            m->graph_wd = weight_decay;
        }
        for (int s = 0; s < steps; ++s) {
            MTRY(cudaGraphLaunch(m->exec, m->stream));
            if (loss_curve) {
                MTRY(cudaMemcpyAsync(loss_curve + s, m->losses.p, sizeof(float), cudaMemcpyDeviceToHost, m->stream));
            }
        }
        MTRY(cudaStreamSynchronize(m->stream));
        return check_err(m);
    }, mfail);
}

pach_status pach_mlp_forward(pach_mlp *m, const float *cond, int32_t rows, float *out) {
    return guarded([&]() -> pach_status {
        if (!m || !cond || !out || rows < 1 || rows > m->max_rows) return mfail(PACH_ERR_INVALID_ARGUMENT, "bad arguments");
        std::lock_guard<std::mutex> lk(m->mu);
        const int Mp = round_up(rows, kTile);
        MTRY(cudaMemcpyAsync(m->cond_in.p, cond, (size_t)rows * kIn * sizeof(float), cudaMemcpyHostToDevice, m->stream));
        k_pack_input<<<(Mp * kInPad + 255) / 256, 256, 0, m->stream>>>(m->cond_in.as<float>(), rows, Mp,
                                                                        m->xb.as<__nv_bfloat16>(), m->xt.as<__nv_bfloat16>());
        MTRY(cudaGetLastError());
        MTRY(forward(m, rows, Mp));
        MTRY(cudaMemcpyAsync(out, m->out.p, (size_t)rows * kOut * sizeof(float), cudaMemcpyDeviceToHost, m->stream));
        MTRY(cudaStreamSynchronize(m->stream));
        m->x_train = false;
        return check_err(m);
    }, mfail);
}

pach_status pach_mlp_gemm(const float *A, const float *B, int32_t M, int32_t N, int32_t K, float *C) {
    return guarded([&]() -> pach_status {
        if (!A || !B || !C || M < 1 || N < 16 || K < 16 || M > 4096 || N > 4096 || K > 4096 || N % 16 || K % 16)
            return mfail(PACH_ERR_INVALID_ARGUMENT, "gemm: M, N, K must be 1..4096, N and K multiples of 16");
        int nd = 0;
        if (cudaGetDeviceCount(&nd) != cudaSuccess || nd < 1) return mfail(PACH_ERR_NO_DEVICE, "no CUDA device");
        const int Mp = round_up(M, kTile), Np = round_up(N, kTile);
        std::vector<__nv_bfloat16> a((size_t)Mp * K, __float2bfloat16_rn(0.f)), b((size_t)Np * K, __float2bfloat16_rn(0.f));
        for (int i = 0; i < M; ++i)
            for (int k = 0; k < K; ++k) a[blk(i, k, K)] = __float2bfloat16_rn(A[(size_t)i * K + k]);
        for (int i = 0; i < N; ++i)
            for (int k = 0; k < K; ++k) b[blk(i, k, K)] = __float2bfloat16_rn(B[(size_t)i * K + k]);
        Buf da, db, dc, de;
        MTRY(da.alloc(a.size() * 2));
        MTRY(db.alloc(b.size() * 2));
        MTRY(dc.alloc((size_t)M * N * sizeof(float)));
        MTRY(de.alloc(sizeof(int)));
        MTRY(cudaMemcpy(da.p, a.data(), a.size() * 2, cudaMemcpyHostToDevice));
        MTRY(cudaMemcpy(db.p, b.data(), b.size() * 2, cudaMemcpyHostToDevice));
        Gemm g{};
        g.A = da.as<__nv_bfloat16>();
        g.B = db.as<__nv_bfloat16>();
        g.Mp = Mp;
        g.N = N;
        g.K = K;
        g.epi = EPI_F32;
        g.m_valid = M;
        g.out = dc.as<float>();
        g.ld_out = N;
        g.err = de.as<int>();
        MTRY(launch_gemm(g, 0));
        MTRY(cudaDeviceSynchronize());
        int h = 0;
        MTRY(cudaMemcpy(&h, de.p, sizeof(int), cudaMemcpyDeviceToHost));
        if (h) return mfail(PACH_ERR_GAVE_UP, "tensor-core GEMM: a bounded barrier wait ran out");
        MTRY(cudaMemcpy(C, dc.p, (size_t)M * N * sizeof(float), cudaMemcpyDeviceToHost));
        return PACH_OK;
    }, mfail);
}

pach_status pach_direction_bins(float *dirs, float *solid_angle, int32_t cap) {
    return guarded([&]() -> pach_status {
        if (!dirs || !solid_angle || cap < kBins) return mfail(PACH_ERR_INVALID_ARGUMENT, "need room for 1536 bins");
        std::vector<float> d, om;
        direction_bins_host(d, om);
        std::memcpy(dirs, d.data(), d.size() * sizeof(float));
        std::memcpy(solid_angle, om.data(), om.size() * sizeof(float));
        return PACH_OK;
    }, mfail);
}

}  // extern "C"
