/*
 * pach_proposal.h -- learned emission proposal of the GB300 split ray tracer.
 *
 * No counterpart in the reference: there every primary ray leaves the source uniformly
 * (GeodesicSource / RandomSource, Pachyderm_Acoustic_Universal/Classes_Sources.cs:256-265, 390-403).
 *
 * A small MLP maps a condition -- source xyz, receiver xyz, room bounds min xyz and max xyz, 12
 * numbers in metres -- to a mixture of 32 von Mises-Fisher lobes over emission directions.  Layers
 * 12 -> 256 -> 256 -> 256 -> 160 with exact GELU between them; BF16 weights and activations, FP32
 * accumulation, FP32 master weights and Adam.  Training and inference run in the library's own
 * tensor-core kernels (tcgen05.mma with accumulators in tensor memory, operands staged by bulk
 * asynchronous copies).
 *
 * Training data come from the tracer itself.  With pach_trace_params.capture = 1 a run adds up, per
 * receiver, arrival-time window (edges in ms after the direct arrival) and emission-direction bin, the
 * energy its primaries deliver (pach_trace_get_capture).  The training target of a receiver is the
 * sum over windows of each window's energy share per bin: the proposal that spends rays where every
 * window's energy comes from.  The loss is the cross-entropy of that target against the mixture's
 * probability of each bin.
 *
 * A run given proposal lobes (pach_trace_params.proposal) emits from the defensive mixture
 *   q(d) = mix / (4 pi) + (1 - mix) / n * sum_j q_j(d)
 * over the n listed receivers' mixtures and weights every primary by (1 / (4 pi)) / q(d), so every
 * histogram stays an unbiased estimate of the uniform-emission result.
 */
#ifndef PACH_PROPOSAL_H
#define PACH_PROPOSAL_H

#include "pach_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

#define PACH_MLP_IN 12
#define PACH_MLP_HIDDEN 256
#define PACH_MLP_LOBES 32
#define PACH_MLP_OUT 160          /* per lobe: mean direction (3, normalised inside), log kappa, logit */
#define PACH_DIR_BINS 1536        /* emission-direction bins: cube map, 6 faces x 16 x 16 */
#define PACH_CAPTURE_WINDOWS 4

typedef struct pach_mlp pach_mlp;

/* Number of trainable parameters: W1[256][12] b1[256] W2[256][256] b2 W3[256][256] b3 W4[160][256] b4[160]
 * (W[out][in]), the order of every flat parameter or gradient array below. */
int64_t pach_mlp_param_count(void);

/* A network with seeded initial weights and room for up to max_rows conditions per call. */
pach_status pach_mlp_create(uint64_t seed, int32_t max_rows, pach_mlp **out);
void pach_mlp_destroy(pach_mlp *m);
pach_status pach_mlp_get_params(pach_mlp *m, float *params, int64_t n);
pach_status pach_mlp_set_params(pach_mlp *m, const float *params, int64_t n);   /* resets Adam */

/* Training set: cond [rows][12] (metres), target [rows][PACH_DIR_BINS] (each row sums to 1). */
pach_status pach_mlp_set_data(pach_mlp *m, const float *cond, const float *target, int32_t rows);

/* Mean loss over the training set and, when grad is not NULL, its gradient [param_count]. */
pach_status pach_mlp_loss_grad(pach_mlp *m, float *loss, float *grad);

/* steps full-batch Adam steps (replayed from a captured CUDA graph); loss_curve [steps] or NULL. */
pach_status pach_mlp_train(pach_mlp *m, int32_t steps, float lr, float weight_decay, float *loss_curve);

/* Inference: cond [rows][12] -> raw outputs [rows][160] (the values pach_trace_params.proposal takes). */
pach_status pach_mlp_forward(pach_mlp *m, const float *cond, int32_t rows, float *out);

/* Diagnostic: C[M][N] = bf16(A)[M][K] . bf16(B)[N][K]^T through the tensor-core GEMM kernel
 * (K a multiple of 16, N a multiple of 16, M, N, K <= 4096). */
pach_status pach_mlp_gemm(const float *A, const float *B, int32_t M, int32_t N, int32_t K, float *C);

/* The emission-direction bins: centre directions [cap][3] and solid angles [cap] (sr). */
pach_status pach_direction_bins(float *dirs, float *solid_angle, int32_t cap);

/* Bin of a direction (the same rule as the device). */
int32_t pach_direction_bin(double x, double y, double z);

/* Diagnostic: n emission directions [n][3] and weights [n] drawn by the device sampler for primaries
 * ray_begin .. ray_begin + n - 1 from the defensive mixture of n_prop raw MLP outputs. */
pach_status pach_proposal_sample(const float *proposal, int32_t n_prop, double mix, uint64_t seed,
                                 int64_t ray_begin, int32_t n, float *dirs, float *weights);

/* Capture of a finished run: capture = 1 gives [n_receivers][PACH_CAPTURE_WINDOWS][PACH_DIR_BINS],
 * capture = 2 gives [ray_count][n_receivers][PACH_CAPTURE_WINDOWS] (energy in W, unscaled); cap >= that
 * many floats. */
pach_status pach_trace_get_capture(pach_run *run, float *out, size_t cap);

#ifdef __cplusplus
}
#endif

#endif
