// filters.cu -- receiver filters on the GPU: Pach_SP.ETCToFilter (Pach_SP.cs:1584-1680) and the
// directional histogram's Create_Filter (Classes_Receivers.cs:1910-1937, 1968-1995).
//
// A filter is the sum over 9 bands of (band envelope) (*) (band carrier): the 8 octave pressure
// envelopes |P[b][t]| 10^((120 - SWL[b]) / 20) and a 16 kHz envelope (the 8 kHz one times an air
// attenuation ramp), each convolved with a 16384-sample band-limited sinc pulse
// (GenerateBandLimitedSincPulse, Pach_SP.cs:1682-1703).  The reference convolves band by band with
// zero-padded FFTW transforms (FFT_Convolution_double, Pach_SP.cs:1948-1975); here the sum is formed
// in the frequency domain, Y = sum_b FFT(env_b) FFT(carrier_b), and transformed back once.
//
// Transforms are FP64 (the reference's precision), length W = 2^m >= T + 16383, split as W = N1 x N2
// (four-step): column transforms of length N1 over the [n1][n2] view, a twiddle w_W^(n2 k1), then row
// transforms of length N2.  The forward result stays in [k1][k2] order (X[k1 + N1 k2] at row k1,
// column k2); the inverse reads that order, so no transpose is ever made.  Each short transform is a
// radix-2 Stockham pass sequence in shared memory.  Two real envelopes travel as one complex sequence
// (env_a + i env_b) and are separated after the row transform from X[k] and conj X[W - k], whose
// partner row N1 - k1 is handled by the same CTA.  Kernels:
//   k_fwd_cols  envelopes built from the histograms (P, P Dir / E), column transforms, twiddle
//   k_rows      row transforms, unpacking, sum of the band products, inverse row transform, twiddle
//   k_inv_cols  inverse column transforms, real part / W, cut to the filter length
// The carriers' spectra go through the same kernels once per call (k_rows in store mode).
// Bound: FP64 issue (GB300 has about 2 FP64 lanes per SM clock); the histograms and the per-filter
// spectra stay within L2-sized working sets.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "engine.h"

namespace pach {
namespace {

constexpr int kCarrierLen = 16384;
constexpr int kPacks = 5;        // (0,1) (2,3) (4,5) (6,7) (16 kHz, -)
constexpr int kMaxLogW = 20;
constexpr int kThreads = 256;
constexpr size_t kZBudget = size_t(512) << 20;  // bytes of per-filter spectra per chunk, at most

struct Geom {
    int W, logW, N1, N2, logN1, logN2, cb, logcb;
};

Geom make_geom(int T) {
    Geom g{};
    const long long need = (long long)T + kCarrierLen - 1;
    int m = 0;
    while ((1ll << m) < need) ++m;
    g.logW = m;
    g.W = 1 << m;
    g.logN1 = m / 2;
    g.logN2 = m - g.logN1;
    g.N1 = 1 << g.logN1;
    g.N2 = 1 << g.logN2;
    g.cb = std::min(16, 4096 / g.N1);  // columns per CTA: 2 x cb x N1 x 16 B of shared memory <= 128 KB
    g.logcb = 0;
    while ((1 << g.logcb) < g.cb) ++g.logcb;
    return g;
}

struct Job {
    const double *E, *P, *Dp, *Dn, *scale;
    const double *att;       // [T] 16 kHz ramp
    const double *car;       // [9][16384] carriers (carrier mode: the envelopes are these)
    double pmod[kBands];
    int T, kinds, job0;
};

struct Work {
    double2 *tw, *cs, *z;
    double *car, *att;
    int chunk;
};

size_t align_up(size_t x) { return (x + 255) & ~size_t(255); }

size_t fixed_bytes(const Geom &g, int T) {
    return align_up((size_t)g.W * sizeof(double2)) + align_up((size_t)9 * g.W * sizeof(double2)) +
           align_up((size_t)9 * kCarrierLen * sizeof(double)) + align_up((size_t)T * sizeof(double));
}

size_t per_job_bytes(const Geom &g) { return (size_t)kPacks * g.W * sizeof(double2); }

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// Radix-2 Stockham transforms of `cnt` sequences of length N = 2^logN in shared memory, natural order
// in and out (x: input, y: scratch; returns the buffer holding the result).  COLS: element i of
// sequence q at [i * cnt + q] (column view, consecutive threads on consecutive columns); else at
// [q * N + i].  tw[j] = w_N^j for j < N / 2.  Stages whose upper half is still all zero (the input
// is nonzero only in its first `sup` elements, and stage s spreads it to sup << s) reduce to copies;
// the twiddles of stages 0 and 1 (1 and -i) need no multiplication.  FP64 issue bounds these
// kernels, so every FP64 instruction saved counts.
template <bool COLS>
__device__ double2 *smem_fft(double2 *x, double2 *y, int logN, int cnt, int logcnt, const double2 *tw, bool inv,
                             int sup) {
    const int N = 1 << logN, half = N >> 1, nb = half * cnt;
    for (int s = 0; s < logN; ++s) {
        const int Ns = 1 << s;
        const bool copy = ((long long)sup << s) <= half;
        for (int b = threadIdx.x; b < nb; b += blockDim.x) {
            int j, q;
            if (COLS) {
                q = b & (cnt - 1);
                j = b >> logcnt;
            } else {
                j = b & (half - 1);
                q = b >> (logN - 1);
            }
            const int k = j & (Ns - 1);
            const int o = ((j - k) << 1) + k;
            const int ia = COLS ? j * cnt + q : q * N + j;
            const int io = COLS ? o * cnt + q : q * N + o;
            const int io2 = COLS ? (o + Ns) * cnt + q : q * N + o + Ns;
            const double2 a = x[ia];
            if (copy) {
                y[io] = a;
                y[io2] = a;
                continue;
            }
            const int ib = COLS ? (j + half) * cnt + q : q * N + j + half;
            double2 c = x[ib];
            if (s >= 2) {
                double2 w = tw[k << (logN - 1 - s)];
                if (inv) w.y = -w.y;
                c = cmul(c, w);
            } else if (k) {  // stage 1, k = 1: w = -i (forward) or +i (inverse); stage 0: w = 1
                c = inv ? make_double2(-c.y, c.x) : make_double2(c.y, -c.x);
            }
            y[io] = make_double2(a.x + c.x, a.y + c.y);
            y[io2] = make_double2(a.x - c.x, a.y - c.y);
        }
        __syncthreads();
        double2 *t = x;
        x = y;
        y = t;
    }
    return x;
}

__device__ __forceinline__ void load_tw(double2 *tw, const double2 *twW, int logW, int logN) {
    for (int j = threadIdx.x; j < (1 << (logN - 1)); j += blockDim.x) tw[j] = twW[(size_t)j << (logW - logN)];
}

__global__ void k_twiddles(double2 *tw, int W) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= W) return;
    double s, c;
    sincospi(-2.0 * (double)m / (double)W, &s, &c);
    tw[m] = make_double2(c, s);
}

// GenerateBandLimitedSincPulse for the 8 octave bands (fc = 62.5 x 2^b) and 16 kHz, one CTA each,
// with the expressions in the reference's order; then the 16 kHz ramp 10^(-add t / fs x 343 / 20).
__global__ void __launch_bounds__(1024) k_carriers(double *car, double *att, int fs, int T, double add) {
    __shared__ double red[32];
    const int b = blockIdx.x;
    if (b == 9) {
        for (int t = threadIdx.x; t < T; t += blockDim.x) {
            const double dist = (double)t * (1.0 / (double)fs) * 343.0;
            att[t] = pow(10.0, -add * dist / 20.0);
        }
        return;
    }
    const double rt2 = sqrt(2.0);
    const double fcb = b < 8 ? 62.5 * pow(2.0, (double)b) : 16000.0;
    const double fl = fcb / rt2, fu = fcb * rt2;
    const double fc = (fl + fu) / 2.0, bw = fu - fl, t0 = (kCarrierLen - 1) / 2.0;
    const double pi = 3.141592653589793;
    double part = 0.0;
    double *c = car + (size_t)b * kCarrierLen;
    for (int n = threadIdx.x; n < kCarrierLen; n += blockDim.x) {
        const double t = ((double)n - t0) / (double)fs;
        const double sinc = bw == 0.0 ? 1.0 : sin(pi * bw * t) / (pi * bw * t);
        const double v = sinc * cos(2.0 * pi * fc * t);
        c[n] = v;
        part += fabs(v);
    }
    for (int o = 16; o; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = part;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
        for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (threadIdx.x == 0) red[0] = v;
    }
    __syncthreads();
    const double norm = 2.0 / (red[0] * (double)kCarrierLen);
    if (norm > 0.0)
        for (int n = threadIdx.x; n < kCarrierLen; n += blockDim.x) c[n] *= norm;
}

// One band envelope sample of filter `job`: filter kind 0 takes |P|, kinds 2d+1 / 2d+2 take
// |P Dir_Rec_Neg[d] / E| / |P Dir_Rec_Pos[d] / E| (0 where E = 0); band 8 is band 7 on the 16 kHz ramp.
__device__ __forceinline__ double envelope(const Job &J, int job, int band, int t) {
    const int r = job / J.kinds, kind = job - r * J.kinds;
    const int b = band < kBands ? band : kBands - 1;
    const size_t i = ((size_t)r * kBands + b) * J.T + t;
    double p = J.P[i];
    if (kind > 0) {
        const int d = (kind - 1) >> 1;
        const double *D = (kind & 1) ? J.Dn : J.Dp;
        const double e = J.E[i];
        p = e == 0.0 ? 0.0 : p * D[(((size_t)r * 3 + d) * kBands + b) * J.T + t] / e;
    }
    double v = fabs(p);
    if (J.scale) v *= J.scale[r];
    v *= J.pmod[b];
    if (band == kBands) v *= J.att[t];
    return v;
}

// Column step of the forward transform for pack q of filter job0 + blockIdx.y / 5, columns
// [blockIdx.x cb, +cb): Z[k1][n2] = w_W^(n2 k1) sum_n1 z[n1 N2 + n2] w_N1^(n1 k1).
__global__ void __launch_bounds__(kThreads) k_fwd_cols(Job J, Geom g, double2 *Z, const double2 *twW, int carrier) {
    extern __shared__ double2 sm[];
    double2 *x = sm, *y = sm + g.cb * g.N1, *tw = sm + 2 * g.cb * g.N1;
    const int c0 = blockIdx.x * g.cb;
    const int job = blockIdx.y / kPacks, q = blockIdx.y - job * kPacks;
    load_tw(tw, twW, g.logW, g.logN1);
    const int T = carrier ? kCarrierLen : J.T;
    const int ba = 2 * q, bb = 2 * q + 1;  // bands of the real and imaginary parts (band 8 = 16 kHz)
    for (int idx = threadIdx.x; idx < g.cb * g.N1; idx += blockDim.x) {
        const int n1 = idx >> g.logcb, c = idx & (g.cb - 1);
        const long long n = (long long)n1 * g.N2 + c0 + c;
        double re = 0.0, im = 0.0;
        if (n < T) {
            if (carrier) {
                re = J.car[(size_t)ba * kCarrierLen + n];
                if (bb < 9) im = J.car[(size_t)bb * kCarrierLen + n];
            } else {
                re = envelope(J, J.job0 + job, ba, (int)n);
                if (bb < 9) im = envelope(J, J.job0 + job, bb, (int)n);
            }
        }
        x[idx] = make_double2(re, im);
    }
    __syncthreads();
    const long long rows = ((long long)T + g.N2 - 1) >> g.logN2;
    const int sup = rows < g.N1 ? (int)rows : g.N1;
    const double2 *res = smem_fft<true>(x, y, g.logN1, g.cb, g.logcb, tw, false, sup);
    double2 *dst = Z + ((size_t)job * kPacks + q) * g.W;
    for (int idx = threadIdx.x; idx < g.cb * g.N1; idx += blockDim.x) {
        const int k1 = idx >> g.logcb, c = idx & (g.cb - 1);
        const int n2 = c0 + c;
        dst[(size_t)k1 * g.N2 + n2] = cmul(res[idx], twW[(size_t)n2 * k1]);
    }
}

// Row step for the row pair (p, N1 - p) of filter blockIdx.y.  Per pack: forward row transforms; the
// two real spectra are E_a[k] = (Z[k] + conj Z[W-k]) / 2 and E_b[k] = (Z[k] - conj Z[W-k]) / 2i, so
// E_a C_a + E_b C_b = Z[k] G[k] + conj Z[W-k] H[k] with G = (C_a - i C_b) / 2, H = (C_a + i C_b) / 2.
// store = 1 (carriers): the packs are the carriers; G and H go to cs[2q], cs[2q + 1] (pack 4, the
// 16 kHz carrier alone: C / 2 to cs[8]).  store = 0: Y = sum over packs of Z G + conj(Z') H, then the
// inverse row transform and the twiddle conj w_W^(n2 k1) into pack 0.
__global__ void __launch_bounds__(kThreads) k_rows(Geom g, double2 *Z, double2 *cs, const double2 *twW, int store) {
    extern __shared__ double2 sm[];
    const int N2 = g.N2;
    double2 *x = sm, *y = sm + 2 * N2, *acc = sm + 4 * N2, *tw = sm + 6 * N2;
    const int p = blockIdx.x, job = blockIdx.y;
    const int r0 = p, r1 = (g.N1 - p) & (g.N1 - 1);
    const bool self = r0 == r1;
    const int nrow = self ? 1 : 2;
    load_tw(tw, twW, g.logW, g.logN2);
    if (!store)
        for (int i = threadIdx.x; i < nrow * N2; i += blockDim.x) acc[i] = make_double2(0.0, 0.0);
    for (int q = 0; q < kPacks; ++q) {
        const double2 *src = Z + ((size_t)job * kPacks + q) * g.W;
        for (int i = threadIdx.x; i < nrow * N2; i += blockDim.x) {
            const int slot = i >> g.logN2, c = i & (N2 - 1);
            x[i] = src[(size_t)(slot ? r1 : r0) * N2 + c];
        }
        __syncthreads();
        const double2 *res = smem_fft<false>(x, y, g.logN2, nrow, nrow - 1, tw, false, N2);
        const int ba = 2 * q, bb = 2 * q + 1;
        for (int i = threadIdx.x; i < nrow * N2; i += blockDim.x) {
            const int slot = i >> g.logN2, c = i & (N2 - 1);
            const int k1 = slot ? r1 : r0;
            const int ps = self ? 0 : 1 - slot;
            const int pc = k1 == 0 ? ((N2 - c) & (N2 - 1)) : (N2 - 1 - c);
            const double2 z = res[i], w = res[ps * N2 + pc];
            const size_t pos = (size_t)k1 * N2 + c;
            if (store) {
                const double2 ea = make_double2(0.5 * (z.x + w.x), 0.5 * (z.y - w.y));
                if (bb < 9) {
                    const double2 eb = make_double2(0.5 * (z.y + w.y), -0.5 * (z.x - w.x));
                    cs[(size_t)ba * g.W + pos] = make_double2(0.5 * (ea.x + eb.y), 0.5 * (ea.y - eb.x));
                    cs[(size_t)bb * g.W + pos] = make_double2(0.5 * (ea.x - eb.y), 0.5 * (ea.y + eb.x));
                } else {
                    cs[(size_t)ba * g.W + pos] = make_double2(0.5 * ea.x, 0.5 * ea.y);
                }
            } else {
                double2 a = acc[i];
                const double2 G = cs[(size_t)ba * g.W + pos];
                if (bb < 9) {
                    const double2 H = cs[(size_t)bb * g.W + pos];
                    a.x += z.x * G.x - z.y * G.y + w.x * H.x + w.y * H.y;
                    a.y += z.x * G.y + z.y * G.x + w.x * H.y - w.y * H.x;
                } else {
                    const double2 u = make_double2(z.x + w.x, z.y - w.y);
                    a.x += u.x * G.x - u.y * G.y;
                    a.y += u.x * G.y + u.y * G.x;
                }
                acc[i] = a;
            }
        }
        __syncthreads();
    }
    if (store) return;
    const double2 *res = smem_fft<false>(acc, x, g.logN2, nrow, nrow - 1, tw, true, N2);
    double2 *dst = Z + (size_t)job * kPacks * g.W;
    for (int i = threadIdx.x; i < nrow * N2; i += blockDim.x) {
        const int slot = i >> g.logN2, n2 = i & (N2 - 1);
        const int k1 = slot ? r1 : r0;
        double2 t = twW[(size_t)n2 * k1];
        t.y = -t.y;
        dst[(size_t)k1 * N2 + n2] = cmul(res[i], t);
    }
}

// Inverse column step: out[n1 N2 + n2] = Re(sum_k1 Y'[k1][n2] conj w_N1^(n1 k1)) / W for n < L.
__global__ void __launch_bounds__(kThreads) k_inv_cols(Geom g, const double2 *Z, const double2 *twW, double *out,
                                                      int L, int job0) {
    extern __shared__ double2 sm[];
    double2 *x = sm, *y = sm + g.cb * g.N1, *tw = sm + 2 * g.cb * g.N1;
    const int c0 = blockIdx.x * g.cb, job = blockIdx.y;
    load_tw(tw, twW, g.logW, g.logN1);
    const double2 *src = Z + (size_t)job * kPacks * g.W;
    for (int idx = threadIdx.x; idx < g.cb * g.N1; idx += blockDim.x) {
        const int k1 = idx >> g.logcb, c = idx & (g.cb - 1);
        x[idx] = src[(size_t)k1 * g.N2 + c0 + c];
    }
    __syncthreads();
    const double2 *res = smem_fft<true>(x, y, g.logN1, g.cb, g.logcb, tw, true, g.N1);
    const double invW = 1.0 / (double)g.W;
    double *o = out + (size_t)(job0 + job) * L;
    for (int idx = threadIdx.x; idx < g.cb * g.N1; idx += blockDim.x) {
        const int n1 = idx >> g.logcb, c = idx & (g.cb - 1);
        const long long n = (long long)n1 * g.N2 + c0 + c;
        if (n < L) o[n] = res[idx].x * invW;
    }
}

// ISO9613_1_attencoef, scalar form (Classes_Medium_Props.cs:193-202) as written: its exponents -1/2,
// -1/3, 1/2 and -5/2 are C# integer divisions (0, 0, 0 and -2).
double iso9613_scalar(double f, double tk, double pa, double hr) {
    const double h = hr * std::pow(10.0, -6.8346 * std::pow(273.16 / tk, 1.261) + 4.6151) / (pa / 101.325);
    const double frO = (pa / 101.325) * (24 + 4.04 * std::pow(10.0, 4) * h * ((0.02 + h) / (0.391 + h)));
    const double frN = (pa / 101.325) * std::pow(tk / 293.15, 0) *
                       (9 + 280 * h * std::exp(-4.170 * (std::pow(tk / 293.15, 0) - 1)));
    const double z = 0.1068 * std::exp(-3352 / tk) * std::pow(frN + f * f / frN, -1);
    const double y = std::pow(tk / 293.15, -2) * (0.01275 * std::exp(-2239.1 / tk) * std::pow(frO + f * f / frO, -1) + z);
    return 8.686 * f * f * ((1.84 * std::pow(10.0, -11) * std::pow(pa / 101.325, -1) * std::pow(tk / 293.15, 0)) + y);
}

// dB/m by which the 16 kHz band decays faster than the 8 kHz one (Pach_SP.cs:1628-1640: 20 C, the
// pressure passed as 101.325 x 1000, 50 %).
double hf_extra_attenuation() {
    const double tk = 20 + 273.15, pa = 101.325 * 1000, hr = 50.0;
    return iso9613_scalar(16000.0, tk, pa, hr) - iso9613_scalar(8000.0, tk, pa, hr);
}

pach_status ffail(pach_status s, const std::string &m) {
    set_last_error(m.c_str());
    return s;
}

pach_status cuda_fail(cudaError_t e, const char *what) {
    return ffail(PACH_ERR_CUDA, std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")");
}

pach_status check_shape(int R, int T, int kinds, int fs, int cut) {
    if (R < 1) return ffail(PACH_ERR_INVALID_ARGUMENT, "filter count < 1");
    if (T < 1) return ffail(PACH_ERR_INVALID_ARGUMENT, "histogram length T < 1");
    if ((long long)T + kCarrierLen - 1 > (1ll << kMaxLogW))
        return ffail(PACH_ERR_INVALID_ARGUMENT, "T + 16383 exceeds the 2^20-sample transform");
    if (kinds != 1 && kinds != 7) return ffail(PACH_ERR_INVALID_ARGUMENT, "kinds must be 1 or 7");
    if (fs < 1) return ffail(PACH_ERR_INVALID_ARGUMENT, "sample rate < 1");
    if (cut != 0 && cut != 4096) return ffail(PACH_ERR_INVALID_ARGUMENT, "cut must be 0 or 4096");
    if ((long long)R * kinds > (1 << 24)) return ffail(PACH_ERR_INVALID_ARGUMENT, "too many filters");
    return PACH_OK;
}

}  // namespace

size_t filters_workspace_bytes(int n_filters, int T) {
    if (n_filters < 1 || T < 1 || (long long)T + kCarrierLen - 1 > (1ll << kMaxLogW)) return 0;
    const Geom g = make_geom(T);
    const size_t pj = per_job_bytes(g);
    const size_t chunk = std::max<size_t>(1, std::min<size_t>((size_t)n_filters, kZBudget / pj));
    return fixed_bytes(g, T) + chunk * pj;
}

pach_status filters_device(const double *E, const double *P, const double *Dp, const double *Dn, const double *scale,
                           int R, int T, int kinds, int fs, const double *swl, int cut, double *out, void *ws,
                           size_t ws_bytes, cudaStream_t st) {
    if (pach_status s = check_shape(R, T, kinds, fs, cut)) return s;
    if (!P || !out || !ws) return ffail(PACH_ERR_INVALID_ARGUMENT, "pressure, output and workspace are required");
    if (kinds == 7 && (!E || !Dp || !Dn))
        return ffail(PACH_ERR_INVALID_ARGUMENT, "directional filters need energy, dir_pos and dir_neg");
    double pmod[kBands];
    for (int b = 0; b < kBands; ++b) {
        const double s = swl ? swl[b] : 120.0;
        if (!std::isfinite(s)) return ffail(PACH_ERR_INVALID_ARGUMENT, "swl must be finite");
        pmod[b] = std::pow(10.0, (120 - s) / 20.0);
    }
    const Geom g = make_geom(T);
    const size_t fixed = fixed_bytes(g, T), pj = per_job_bytes(g);
    if (ws_bytes < fixed + pj) return ffail(PACH_ERR_INVALID_ARGUMENT, "workspace smaller than one filter needs");
    const int n = R * kinds;
    Work w{};
    char *base = static_cast<char *>(ws);
    if (reinterpret_cast<uintptr_t>(base) & 255) return ffail(PACH_ERR_INVALID_ARGUMENT, "workspace not 256-byte aligned");
    w.tw = reinterpret_cast<double2 *>(base);
    base += align_up((size_t)g.W * sizeof(double2));
    w.cs = reinterpret_cast<double2 *>(base);
    base += align_up((size_t)9 * g.W * sizeof(double2));
    w.car = reinterpret_cast<double *>(base);
    base += align_up((size_t)9 * kCarrierLen * sizeof(double));
    w.att = reinterpret_cast<double *>(base);
    base += align_up((size_t)T * sizeof(double));
    w.z = reinterpret_cast<double2 *>(base);
    w.chunk = (int)std::min<size_t>((size_t)n, std::min<size_t>((ws_bytes - fixed) / pj, 65535 / kPacks));

    const size_t sm_cols = (size_t)(2 * g.cb * g.N1 + g.N1 / 2) * sizeof(double2);
    const size_t sm_rows = (size_t)(6 * g.N2 + g.N2 / 2) * sizeof(double2);
    cudaFuncSetAttribute(k_fwd_cols, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_cols);
    cudaFuncSetAttribute(k_inv_cols, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_cols);
    cudaFuncSetAttribute(k_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_rows);
    Job J{};
    J.E = E;
    J.P = P;
    J.Dp = Dp;
    J.Dn = Dn;
    J.scale = scale;
    J.att = w.att;
    J.car = w.car;
    std::memcpy(J.pmod, pmod, sizeof(pmod));
    J.T = T;
    J.kinds = kinds;
    const int L = T + kCarrierLen - 1 - cut;

    k_twiddles<<<(g.W + 255) / 256, 256, 0, st>>>(w.tw, g.W);
    k_carriers<<<10, 1024, 0, st>>>(w.car, w.att, fs, T, hf_extra_attenuation());
    // carriers' spectra: one "filter" of 5 packs, k_rows in store mode
    k_fwd_cols<<<dim3(g.N2 / g.cb, kPacks), kThreads, sm_cols, st>>>(J, g, w.z, w.tw, 1);
    k_rows<<<dim3(g.N1 / 2 + 1, 1), kThreads, sm_rows, st>>>(g, w.z, w.cs, w.tw, 1);
    for (int j0 = 0; j0 < n; j0 += w.chunk) {
        const int nj = std::min(w.chunk, n - j0);
        J.job0 = j0;
        k_fwd_cols<<<dim3(g.N2 / g.cb, nj * kPacks), kThreads, sm_cols, st>>>(J, g, w.z, w.tw, 0);
        k_rows<<<dim3(g.N1 / 2 + 1, nj), kThreads, sm_rows, st>>>(g, w.z, w.cs, w.tw, 0);
        k_inv_cols<<<dim3(g.N2 / g.cb, nj), kThreads, sm_cols, st>>>(g, w.z, w.tw, out, L, j0);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "filter kernels");
    return PACH_OK;
}

// Host-array form: copies in, computes on the calling thread's current device, copies out.
pach_status filters_host(const double *E, const double *P, const double *Dp, const double *Dn, int R, int T,
                         int kinds, int fs, const double *swl, int cut, double *out, size_t cap) {
    if (pach_status s = check_shape(R, T, kinds, fs, cut)) return s;
    const int L = T + kCarrierLen - 1 - cut;
    const size_t n_out = (size_t)R * kinds * L;
    if (!out || cap < n_out) return ffail(PACH_ERR_INVALID_ARGUMENT, "cap < filters x filter length");
    if (!P) return ffail(PACH_ERR_INVALID_ARGUMENT, "pressure is required");
    if (kinds == 7 && (!E || !Dp || !Dn))
        return ffail(PACH_ERR_INVALID_ARGUMENT, "directional filters need energy, dir_pos and dir_neg");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return ffail(PACH_ERR_NO_DEVICE, "no CUDA device");
    }
    const size_t nh = (size_t)R * kBands * T;
    const size_t wsb = filters_workspace_bytes(R * kinds, T);
    struct Buf {
        void *p = nullptr;
        ~Buf() { if (p) cudaFree(p); }
    } bP, bE, bDp, bDn, bOut, bWs;
    cudaStream_t st = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_fail(e, "stream");
    struct StreamGuard {
        cudaStream_t s;
        ~StreamGuard() { cudaStreamDestroy(s); }
    } sg{st};
    auto up = [&](Buf &b, const double *h, size_t n) -> cudaError_t {
        cudaError_t r = cudaMalloc(&b.p, n * sizeof(double));
        if (r != cudaSuccess) return r;
        return cudaMemcpyAsync(b.p, h, n * sizeof(double), cudaMemcpyHostToDevice, st);
    };
    if ((e = up(bP, P, nh)) != cudaSuccess) return cuda_fail(e, "filter input");
    if (kinds == 7) {
        if ((e = up(bE, E, nh)) != cudaSuccess || (e = up(bDp, Dp, 3 * nh)) != cudaSuccess ||
            (e = up(bDn, Dn, 3 * nh)) != cudaSuccess)
            return cuda_fail(e, "filter input");
    }
    if ((e = cudaMalloc(&bOut.p, n_out * sizeof(double))) != cudaSuccess) return cuda_fail(e, "filter output");
    if ((e = cudaMalloc(&bWs.p, wsb)) != cudaSuccess) return cuda_fail(e, "filter workspace");
    pach_status s = filters_device((const double *)bE.p, (const double *)bP.p, (const double *)bDp.p,
                                   (const double *)bDn.p, nullptr, R, T, kinds, fs, swl, cut, (double *)bOut.p,
                                   bWs.p, wsb, st);
    if (s != PACH_OK) {
        cudaStreamSynchronize(st);
        return s;
    }
    if ((e = cudaMemcpyAsync(out, bOut.p, n_out * sizeof(double), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return cuda_fail(e, "filter copy");
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cuda_fail(e, "filter kernels");
    return PACH_OK;
}

}  // namespace pach

using namespace pach;

extern "C" {

size_t pach_filters_workspace_bytes(int32_t n_filters, int32_t T) { return filters_workspace_bytes(n_filters, T); }

pach_status pach_filters_device(const double *d_energy, const double *d_pressure, const double *d_dir_pos,
                                const double *d_dir_neg, const double *d_scale, int32_t R, int32_t T, int32_t kinds,
                                int32_t sample_rate, const double *swl, int32_t cut, double *d_out,
                                void *d_workspace, size_t workspace_bytes, void *stream) {
    return guarded([&]() -> pach_status {
        return filters_device(d_energy, d_pressure, d_dir_pos, d_dir_neg, d_scale, R, T, kinds, sample_rate, swl, cut,
                              d_out, d_workspace, workspace_bytes, static_cast<cudaStream_t>(stream));
    }, ffail);
}

pach_status pach_etc_to_filter(const double *prms, int32_t n, int32_t T, const double *swl, int32_t sample_rate,
                               double *out, size_t cap) {
    return guarded([&]() -> pach_status {
        return filters_host(nullptr, prms, nullptr, nullptr, n, T, 1, sample_rate, swl, 0, out, cap);
    }, ffail);
}

pach_status pach_receiver_filters(const double *energy, const double *pressure, const double *dir_pos,
                                  const double *dir_neg, int32_t R, int32_t T, int32_t sample_rate, const double *swl,
                                  double *out, size_t cap) {
    return guarded([&]() -> pach_status {
        const int kinds = (dir_pos && dir_neg) ? 7 : 1;
        return filters_host(energy, pressure, dir_pos, dir_neg, R, T, kinds, sample_rate, swl, 4096, out, cap);
    }, ffail);
}

}  // extern "C"
