/*
 * pach_oracle.cpp -- CPU FP64 restatement of Pachyderm's stochastic split ray tracer.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GPU engine (see pach_oracle.h).  Parity is
 * unpinned against the reference itself (no runnable reference, no reference tests, Hare
 * unvendored); it is pinned to analytic known answers in tests/.
 *
 * Arithmetic is FP64 throughout, as in the reference.  Random numbers come from a Philox4x32-10
 * counter generator (Salmon et al., SC'11) keyed by ray identity instead of .NET System.Random,
 * so that the GPU engine can draw exactly the same numbers for the same ray regardless of
 * scheduling.  The reference seeds from the wall clock (TaskAll:212) and is not reproducible.
 */
#include "pach_oracle.h"

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

namespace {

const double kPi = 3.14159265358979323846;

/* ----------------------------------------------------------------------------------------
 * RNG: Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as
 * 1, 2, 3", SC 2011).  Multipliers and Weyl increments are the published constants.
 * -------------------------------------------------------------------------------------- */
inline void philox(uint32_t c[4], uint32_t k0, uint32_t k1) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
    for (int r = 0; r < 10; ++r) {
        if (r) { k0 += W0; k1 += W1; }
        uint64_t p0 = (uint64_t)M0 * c[0];
        uint64_t p1 = (uint64_t)M1 * c[2];
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
    }
}

/* 24-bit uniforms in [0,1): exactly representable in FP32 and FP64, so FP32 and FP64
 * comparisons against the same threshold agree. */
inline double u24(uint32_t x) { return (double)(x >> 8) * (1.0 / 16777216.0); }

struct Block { double u[4]; };

/* One draw block of stream `sid` of primary `ray`: counter (b, ray, sid lo, sid hi). */
inline Block draw_block(uint64_t seed, int64_t ray, uint64_t sid, uint32_t b) {
    uint32_t c[4] = {b, (uint32_t)ray, (uint32_t)sid, (uint32_t)(sid >> 32)};
    philox(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    Block B;
    for (int i = 0; i < 4; ++i) B.u[i] = u24(c[i]);
    return B;
}

/* SplitMix64 finaliser (Steele, Lea, Flood, OOPSLA'14). */
inline uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* Stream identifiers: who a ray is in the split tree of its primary. */
inline uint64_t sid_early(int k, int o, int q) {      /* Scatter_Early child, bounce k, band o, kind q */
    return (1ull << 62) | ((uint64_t)k << 5) | ((uint64_t)o << 2) | (uint64_t)q;
}
inline uint64_t sid_final(int o) { return (2ull << 62) | (uint64_t)o; } /* end-of-phase-A split */
inline uint64_t sid_late(uint64_t parent, uint32_t nb) {               /* Scatter_Late child */
    return (3ull << 62) | (mix64(parent + 0x9E3779B97F4A7C15ull * (uint64_t)(nb + 1)) & ((1ull << 62) - 1));
}

/* ----------------------------------------------------------------------------------------
 * Vector helpers (Hare_math.Dot / Cross semantics).
 * -------------------------------------------------------------------------------------- */
struct V3 { double x, y, z; };
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(V3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline V3 normalized(V3 a) { double l = std::sqrt(dot(a, a)); return l > 0 ? a * (1.0 / l) : a; }

/* ----------------------------------------------------------------------------------------
 * Air: Calculate_Attenuation (Classes_Medium_Props.cs:51-191), Calculate_Density (42-49),
 * Uniform_Medium ctor (286-299), SoundSpeed (Classes_Math.cs:272-275).  The C# integer
 * divisions in exponents are kept: -1/2 -> 0, -1/3 -> 0, -5/2 -> -2, 1/2 -> 0.
 * -------------------------------------------------------------------------------------- */
void attenuation(int air_choice, double Pa_kpa, double Tk, double hr, int edge, double out[8]) {
    const double F[8] = {62.5, 125, 250, 500, 1000, 2000, 4000, 8000};
    for (int i = 0; i < 8; ++i) out[i] = 0;
    if (air_choice == 0) {
        double h = hr * std::pow(10.0, -6.8346 * std::pow(273.16 / Tk, 1.261) + 4.6151) / (Pa_kpa / 101.325);
        for (int o = 0; o < 8; ++o) {
            double frO = (Pa_kpa / 101.325) * (24 + 4.04 * std::pow(10.0, 4) * h * ((0.02 + h) / (0.391 + h)));
            double frN = (Pa_kpa / 101.325) * std::pow(Tk / 293.15, (double)(-1 / 2)) *
                         (9 + 280 * h * std::exp(-4.170 * (std::pow(Tk / 293.15, (double)(-1 / 3)) - 1)));
            double z = 0.1068 * std::exp(-3352 / Tk) * std::pow(frN + F[o] * F[o] / frN, -1.0);
            double y = std::pow(Tk / 293.15, (double)(-5 / 2)) *
                       (0.01275 * std::exp(-2239.1 / Tk) * std::pow(frO + F[o] * F[o] / frO, -1.0) + z);
            out[o] = 8.686 * F[o] * F[o] *
                     ((1.84 * std::pow(10.0, -11) * std::pow(Pa_kpa / 101.325, -1.0) *
                       std::pow(Tk / 293.15, (double)(1 / 2))) + y);
        }
    } else if (air_choice == 1) {
        for (int q = 0; q <= 7; ++q) {
            out[q] = ((85 / hr) * (std::pow(F[q] / 1000, 2) * 0.0001)) / 8.7;
            out[q] -= 0.04 * (Tk - 273.15 - 20) * out[q];
            out[q] *= 0.50248756218905477;
        }
    }
    if (air_choice == 2) {
        static const double warm[3][8] = {
            {0.0001, 0.0001, 0.0003, 0.0006, 0.001, 0.0019, 0.0058, 0.0203},
            {0.0001, 0.0001, 0.0003, 0.0006, 0.001, 0.0017, 0.0041, 0.0135},
            {0.0001, 0.0001, 0.0003, 0.0006, 0.0011, 0.0017, 0.0035, 0.0106}};
        static const double cold[3][8] = {
            {0.0001, 0.0001, 0.0002, 0.0005, 0.0011, 0.0027, 0.0094, 0.029},
            {0.0001, 0.0001, 0.0002, 0.0005, 0.0008, 0.0018, 0.0059, 0.0211},
            {0.0001, 0.0001, 0.0002, 0.0005, 0.0007, 0.0014, 0.0044, 0.0158}};
        const double (*tab)[8] = (Tk - 273.15 > 15) ? warm : cold;
        int row = hr < 50 ? 0 : (hr < 70 ? 1 : (hr > 70 ? 2 : -1)); /* hr == 70 matches no branch */
        if (row >= 0) for (int o = 0; o < 8; ++o) out[o] = tab[row][o];
        if (edge) for (int o = 0; o < 8; ++o) out[o] /= std::sqrt(2.0);
    }
}

double density(double Tk, double Pa, double hr) {
    double Rd = 287.05, T = Tk - 273.15;
    double Pv = hr * 6.1078 * std::pow(10.0, (7.5 * T) / (237.3 + T));
    return (Pa / (Rd * Tk)) * (1 - 0.378 * Pv / Pa);
}

/* ----------------------------------------------------------------------------------------
 * Scene: fan triangles keeping the polygon id, flat polygon normals, polygon areas, and a
 * uniform voxel grid (Hare Voxel_Grid, domain cells per axis) for the nearest-hit search.
 * -------------------------------------------------------------------------------------- */
struct Tri { V3 v0, e1, e2; int poly; };

struct Scene {
    std::vector<Tri> tris;
    std::vector<V3> normal;          /* per polygon */
    std::vector<double> area;        /* per polygon */
    std::vector<double> alpha, scat, trans;   /* [P*8] */
    int P = 0;
    /* grid */
    int D = 7;
    V3 bmin{}, bmax{}, cell{};
    std::vector<std::vector<int>> cells;
    bool brute = false;
    double c = 343, rho = 1.2, rho_c = 411.6, atten[8] = {0};
};

bool tri_box_overlap(const Tri &t, V3 lo, V3 hi) {
    V3 a = t.v0, b = t.v0 + t.e1, c = t.v0 + t.e2;
    /* AABB test */
    if (std::max({a.x, b.x, c.x}) < lo.x || std::min({a.x, b.x, c.x}) > hi.x) return false;
    if (std::max({a.y, b.y, c.y}) < lo.y || std::min({a.y, b.y, c.y}) > hi.y) return false;
    if (std::max({a.z, b.z, c.z}) < lo.z || std::min({a.z, b.z, c.z}) > hi.z) return false;
    /* plane vs box (conservative: keeps every cell the triangle's plane passes through) */
    V3 n = cross(t.e1, t.e2);
    V3 ctr = (lo + hi) * 0.5, hh = (hi - lo) * 0.5;
    double r = hh.x * std::fabs(n.x) + hh.y * std::fabs(n.y) + hh.z * std::fabs(n.z);
    double s = dot(n, ctr - a);
    return std::fabs(s) <= r * (1 + 1e-9) + 1e-12;
}

void build_scene(const orc_scene_desc *d, int domain, bool brute, bool pure_specular, Scene &S) {
    S.P = d->n_polys;
    S.brute = brute;
    S.D = domain > 0 ? domain : 7;
    auto vtx = [&](int i) { return V3{d->vertices[3 * i], d->vertices[3 * i + 1], d->vertices[3 * i + 2]}; };
    S.normal.resize(S.P);
    S.area.resize(S.P);
    S.alpha.assign(d->absorption, d->absorption + 8 * (size_t)S.P);
    S.scat.assign(d->scattering, d->scattering + 8 * (size_t)S.P);
    if (d->transmission) S.trans.assign(d->transmission, d->transmission + 8 * (size_t)S.P);
    else S.trans.assign(8 * (size_t)S.P, 0.0);
    if (pure_specular) {
        std::fill(S.scat.begin(), S.scat.end(), 0.0);
        std::fill(S.trans.begin(), S.trans.end(), 0.0);
    }
    S.bmin = {1e300, 1e300, 1e300};
    S.bmax = {-1e300, -1e300, -1e300};
    for (int p = 0; p < S.P; ++p) {
        int b = d->poly_offsets[p], e = d->poly_offsets[p + 1];
        /* Newell normal: flat polygon normal (Classes_Scenes.cs:864-872 via Hare Topology). */
        V3 n{0, 0, 0};
        for (int k = b; k < e; ++k) {
            V3 p0 = vtx(d->poly_indices[k]), p1 = vtx(d->poly_indices[k + 1 < e ? k + 1 : b]);
            n.x += (p0.y - p1.y) * (p0.z + p1.z);
            n.y += (p0.z - p1.z) * (p0.x + p1.x);
            n.z += (p0.x - p1.x) * (p0.y + p1.y);
        }
        S.area[p] = 0.5 * std::sqrt(dot(n, n));
        S.normal[p] = normalized(n);
        V3 a = vtx(d->poly_indices[b]);
        for (int k = b + 1; k + 1 < e; ++k) {
            V3 pb = vtx(d->poly_indices[k]), pc = vtx(d->poly_indices[k + 1]);
            S.tris.push_back(Tri{a, pb - a, pc - a, p});
        }
        for (int k = b; k < e; ++k) {
            V3 q = vtx(d->poly_indices[k]);
            S.bmin = {std::min(S.bmin.x, q.x), std::min(S.bmin.y, q.y), std::min(S.bmin.z, q.z)};
            S.bmax = {std::max(S.bmax.x, q.x), std::max(S.bmax.y, q.y), std::max(S.bmax.z, q.z)};
        }
    }
    /* Inflate the box so that boundary walls lie strictly inside the grid. */
    V3 ext = S.bmax - S.bmin;
    double pad = 1e-6 * std::max({ext.x, ext.y, ext.z, 1e-3});
    S.bmin = S.bmin - V3{pad, pad, pad};
    S.bmax = S.bmax + V3{pad, pad, pad};
    ext = S.bmax - S.bmin;
    S.cell = {ext.x / S.D, ext.y / S.D, ext.z / S.D};
    S.cells.assign((size_t)S.D * S.D * S.D, {});
    for (int i = 0; i < (int)S.tris.size(); ++i) {
        const Tri &t = S.tris[i];
        V3 a = t.v0, b = t.v0 + t.e1, c = t.v0 + t.e2;
        V3 lo{std::min({a.x, b.x, c.x}), std::min({a.y, b.y, c.y}), std::min({a.z, b.z, c.z})};
        V3 hi{std::max({a.x, b.x, c.x}), std::max({a.y, b.y, c.y}), std::max({a.z, b.z, c.z})};
        auto cl = [&](double v, double mn, double cs) { int k = (int)std::floor((v - mn) / cs); return std::min(std::max(k, 0), S.D - 1); };
        int x0 = cl(lo.x, S.bmin.x, S.cell.x), x1 = cl(hi.x, S.bmin.x, S.cell.x);
        int y0 = cl(lo.y, S.bmin.y, S.cell.y), y1 = cl(hi.y, S.bmin.y, S.cell.y);
        int z0 = cl(lo.z, S.bmin.z, S.cell.z), z1 = cl(hi.z, S.bmin.z, S.cell.z);
        for (int x = x0; x <= x1; ++x)
            for (int y = y0; y <= y1; ++y)
                for (int z = z0; z <= z1; ++z) {
                    V3 clo{S.bmin.x + x * S.cell.x, S.bmin.y + y * S.cell.y, S.bmin.z + z * S.cell.z};
                    V3 chi = clo + S.cell;
                    V3 eps = S.cell * 1e-9;
                    if (tri_box_overlap(t, clo - eps, chi + eps)) S.cells[((size_t)x * S.D + y) * S.D + z].push_back(i);
                }
    }
    /* Air (Scene ctor -> Uniform_Medium(Air_Choice, Pa, Tk, hr, EC)). */
    double Tk = d->temp_c + 273.15;
    attenuation(d->air_choice, d->pressure_hpa / 10, Tk, d->rel_humidity, d->edge_correction, S.atten);
    S.rho = density(Tk, d->pressure_hpa * 100, d->rel_humidity);
    S.c = 331 + 0.6 * (Tk - 273.15);
    S.rho_c = S.rho * S.c;
}

/* Moller-Trumbore in FP64; inclusive edges. */
inline bool hit_tri(const Tri &t, V3 o, V3 d, double &tt) {
    V3 p = cross(d, t.e2);
    double det = dot(t.e1, p);
    if (det == 0) return false;
    double inv = 1.0 / det;
    V3 s = o - t.v0;
    double u = dot(s, p) * inv;
    if (u < 0 || u > 1) return false;
    V3 q = cross(s, t.e1);
    double v = dot(d, q) * inv;
    if (v < 0 || u + v > 1) return false;
    tt = dot(t.e2, q) * inv;
    return true;
}

struct Hit { int poly; double t; V3 x; };

/* Ray box entry for an origin outside the grid (Hare OBox.Intersect). */
bool box_entry(const Scene &S, V3 o, V3 d, double &t0) {
    double tn = -1e300, tf = 1e300;
    const double oo[3] = {o.x, o.y, o.z}, dd[3] = {d.x, d.y, d.z};
    const double lo[3] = {S.bmin.x, S.bmin.y, S.bmin.z}, hi[3] = {S.bmax.x, S.bmax.y, S.bmax.z};
    for (int a = 0; a < 3; ++a) {
        if (dd[a] == 0) { if (oo[a] < lo[a] || oo[a] > hi[a]) return false; continue; }
        double t1 = (lo[a] - oo[a]) / dd[a], t2 = (hi[a] - oo[a]) / dd[a];
        if (t1 > t2) std::swap(t1, t2);
        tn = std::max(tn, t1); tf = std::min(tf, t2);
    }
    if (tn > tf || tf < 0) return false;
    t0 = std::max(tn, 0.0);
    return true;
}

/* Nearest hit with t > 1e-10 (Hare Voxel_Grid.Shoot as seen through
 * Classes_VoxelGrid_PolyRefractive.cs:70-328: Amanatides-Woo stepping, per-ray mailbox, a hit is
 * accepted only once the walk has reached the cell that contains it). */
struct Tracer {
    const Scene &S;
    std::vector<uint32_t> mail;
    uint32_t stamp = 0;
    int64_t cells_visited = 0, tri_tests = 0;   /* algorithm-defined work of the reference traversal */
    explicit Tracer(const Scene &s) : S(s), mail(s.tris.size(), 0) {}

    bool shoot(V3 o, V3 d, Hit &h) {
        const double EPS = 0.0000000001;
        if (S.brute) {
            double best = 1e300; int bi = -1;
            tri_tests += (int64_t)S.tris.size();
            for (int i = 0; i < (int)S.tris.size(); ++i) {
                double t;
                if (hit_tri(S.tris[i], o, d, t) && t > EPS && t < best) { best = t; bi = i; }
            }
            if (bi < 0) return false;
            h.poly = S.tris[bi].poly; h.t = best; h.x = o + d * best;
            return true;
        }
        if (++stamp == 0) { std::fill(mail.begin(), mail.end(), 0); stamp = 1; }
        double t0 = 0;
        V3 rel = o - S.bmin;
        int X = (int)std::floor(rel.x / S.cell.x), Y = (int)std::floor(rel.y / S.cell.y), Z = (int)std::floor(rel.z / S.cell.z);
        if (X < 0 || X >= S.D || Y < 0 || Y >= S.D || Z < 0 || Z >= S.D) {
            if (!box_entry(S, o, d, t0)) return false;
            V3 p = o + d * t0 - S.bmin;
            X = std::min(std::max((int)std::floor(p.x / S.cell.x), 0), S.D - 1);
            Y = std::min(std::max((int)std::floor(p.y / S.cell.y), 0), S.D - 1);
            Z = std::min(std::max((int)std::floor(p.z / S.cell.z), 0), S.D - 1);
        }
        int stX = d.x < 0 ? -1 : 1, stY = d.y < 0 ? -1 : 1, stZ = d.z < 0 ? -1 : 1;
        auto tmax = [&](int idx, int st, double org, double dir, double mn, double cs) {
            if (dir == 0) return 1e300;
            double bound = mn + (idx + (st > 0 ? 1 : 0)) * cs;
            return (bound - org) / dir;
        };
        double tMX = tmax(X, stX, o.x, d.x, S.bmin.x, S.cell.x);
        double tMY = tmax(Y, stY, o.y, d.y, S.bmin.y, S.cell.y);
        double tMZ = tmax(Z, stZ, o.z, d.z, S.bmin.z, S.cell.z);
        double tDX = d.x != 0 ? std::fabs(S.cell.x / d.x) : 1e300;
        double tDY = d.y != 0 ? std::fabs(S.cell.y / d.y) : 1e300;
        double tDZ = d.z != 0 ? std::fabs(S.cell.z / d.z) : 1e300;
        double best = 1e300; int bi = -1;
        for (int guard = 0; guard < 3 * S.D + 3; ++guard) {
            ++cells_visited;
            for (int i : S.cells[((size_t)X * S.D + Y) * S.D + Z]) {
                if (mail[i] == stamp) continue;
                mail[i] = stamp;
                ++tri_tests;
                double t;
                if (hit_tri(S.tris[i], o, d, t) && t > EPS && t < best) { best = t; bi = i; }
            }
            double texit = std::min({tMX, tMY, tMZ});
            if (bi >= 0 && best <= texit * (1 + 1e-12) + 1e-12) break;
            if (tMX < tMY) {
                if (tMX < tMZ) { X += stX; if (X < 0 || X >= S.D) break; tMX += tDX; }
                else { Z += stZ; if (Z < 0 || Z >= S.D) break; tMZ += tDZ; }
            } else {
                if (tMY < tMZ) { Y += stY; if (Y < 0 || Y >= S.D) break; tMY += tDY; }
                else { Z += stZ; if (Z < 0 || Z >= S.D) break; tMZ += tDZ; }
            }
        }
        if (bi < 0) return false;
        h.poly = S.tris[bi].poly; h.t = best; h.x = o + d * best;
        return true;
    }
};

/* ----------------------------------------------------------------------------------------
 * Rays (Classes_Rays.cs): OctaveRay fields that matter to the physics plus the stream identity.
 * -------------------------------------------------------------------------------------- */
struct ORay {
    V3 p, d;
    double I;        /* Intensity */
    double t_sum;    /* seconds */
    double decim;    /* Decimation_threshold (TP3 of the band) */
    int oct;
    int mask;        /* Scatter_Mask: bit0 current-scattered, bit1 ever-scattered */
    uint64_t sid;
    uint32_t nb;     /* bounces drawn on this stream */
};

/* Lambert_Scattering thresholds (Classes_Materials.cs:4466-4485). */
inline void lambert_thresholds(double s, double out[3]) {
    out[1] = s;
    if (s < 0.25) { out[0] = 0.1; out[2] = 0.4; }
    else { double mod = std::fabs(1 - s) / 5; out[0] = s - mod; out[2] = s + mod; }
}

/* Uniform-hemisphere direction around n (Classes_Materials.cs:4521-4552, 4583-4612, 4666-4693):
 * frame z = n, x from (0,0,1) unless |n.z| in (0.99,1.01), then (1,0,0); azimuth 2*pi*U1,
 * zenith acos(U2). */
inline V3 lambert_dir(V3 n, double U1, double U2, bool very_late) {
    V3 dz = n, dx{0, 0, 1};
    double proj = std::fabs(dot(dz, dx));
    if (0.99 < proj && 1.01 > proj) dx = {1, 0, 0};
    V3 dy = cross(dz, dx);
    dx = cross(dy, dz);
    dx = normalized(dx); dy = normalized(dy); dz = normalized(dz);
    double u1 = 2.0 * kPi * U1;
    double u2 = std::acos(U2);
    double x = std::cos(u1) * std::sin(u2), y = std::sin(u1) * std::sin(u2);
    double z = very_late ? U2 : std::cos(u2);
    return normalized(dx * x + dy * y + dz * z);
}

/* ----------------------------------------------------------------------------------------
 * Receivers + histograms (Classes_Receivers.cs:803-877, 1813-1825).
 * -------------------------------------------------------------------------------------- */
struct Hist {
    int R = 0, T = 0;
    std::vector<double> E, Pr, Dp, Dn, An;
    void init(int r, int t) {
        R = r; T = t;
        E.assign((size_t)R * 8 * T, 0); Pr.assign((size_t)R * 8 * T, 0);
        Dp.assign((size_t)R * 24 * T, 0); Dn.assign((size_t)R * 24 * T, 0); An.assign((size_t)R * 24 * T, 0);
    }
    /* Directional_Histogram.Add(time, E, -dx, -dy, -dz, Rho_C, oct) */
    void add(int r, int oct, int sample, double e, V3 d, double rho_c) {
        size_t i = ((size_t)r * 8 + oct) * T + sample;
        E[i] += e;
        Pr[i] += std::sqrt(e * rho_c);
        const double c[3] = {-d.x, -d.y, -d.z};
        for (int a = 0; a < 3; ++a) {
            size_t j = (((size_t)r * 3 + a) * 8 + oct) * T + sample;
            double v = (double)(float)(c[a] * e);
            if (c[a] > 0) Dp[j] += v; else Dn[j] += v;
        }
    }
    void analysis(int r, int kind, int oct, int sample, double e) {
        An[(((size_t)r * 3 + kind) * 8 + oct) * T + sample] += e;
    }
};

struct Rec { V3 o; double r2; };

/* ----------------------------------------------------------------------------------------
 * Mapping receivers (PachMapReceiver, Pach_Map_Receiver.cs).
 * -------------------------------------------------------------------------------------- */
/* direction histograms of the last directional map traced on this thread (orc_map_directions) */
thread_local std::vector<double> g_map_dp, g_map_dn;

struct MapBank {
    int M = 0, T = 1, walk = 0;
    bool one_pt = false, directional = false;
    double rho_c = 0;
    double r = 0, r2 = 0, sizemod = 0, c = 343;
    double atten[8] = {0};
    std::vector<V3> org;
    std::vector<double> direct;
    double mn[3] = {0, 0, 0}, mx[3] = {0, 0, 0}, vd[3] = {1, 1, 1};
    int n[3] = {1, 1, 1};
    std::vector<std::vector<int>> inv;   /* Voxel_Inv, cell (x * ny + y) * nz + z */
    const std::vector<int> &cell(int x, int y, int z) const { return inv[((size_t)x * n[1] + y) * n[2] + z]; }
    double cmin(int a, int i) const { return (i * vd[a]) + mn[a]; }        /* Voxels[].Min_PT */
    double cmax(int a, int i) const { return ((i + 1) * vd[a]) + mn[a]; }  /* Voxels[].Max_PT */
};

/* Fill_in + Partition (Pach_Map_Receiver.cs:78-263) and the Map_Receiver ctor (1721-1768) for
 * receivers already placed. */
bool build_map(const orc_map_desc *d, V3 src, int nsrc, double c, const double atten[8], MapBank &B) {
    if (!d || d->n_receivers < 1 || !d->origins || !(d->increment > 0)) return false;
    B.M = d->n_receivers;
    B.one_pt = d->time_1pt != 0;
    B.walk = d->walk;
    B.directional = d->directional != 0;
    B.T = B.one_pt ? 1 : (int)(d->cutoff_ms / 1000.0 * 1000.0);  /* Histogram(1000, COTime_in) */
    if (B.T < 1) return false;
    B.r = d->increment * 0.5;                                       /* Radius = Diameter * 0.5 */
    B.r2 = B.r * B.r;
    B.sizemod = 1 / (kPi * B.r2);
    B.c = c;
    for (int o = 0; o < 8; ++o) B.atten[o] = atten[o];
    B.org.resize(B.M);
    B.direct.assign(B.M, 0.0);
    for (int k = 0; k < B.M; ++k) {
        B.org[k] = {d->origins[3 * k], d->origins[3 * k + 1], d->origins[3 * k + 2]};
        if (nsrc == 1) {  /* a SourceCluster leaves Direct_Time = min(0, ...) = 0 */
            double lx = src.x - B.org[k].x, ly = src.y - B.org[k].y, lz = src.z - B.org[k].z;
            B.direct[k] = std::sqrt(lx * lx + ly * ly + lz * lz) / c;
        }
    }
    for (int a = 0; a < 3; ++a) { B.mn[a] = INFINITY; B.mx[a] = -INFINITY; }
    for (int k = 0; k < B.M; ++k) {
        const double o[3] = {B.org[k].x, B.org[k].y, B.org[k].z};
        for (int a = 0; a < 3; ++a) {
            if (o[a] + d->increment * .5 > B.mx[a]) B.mx[a] = o[a] + d->increment * .5;
            if (o[a] - d->increment * .5 < B.mn[a]) B.mn[a] = o[a] - d->increment * .5;
        }
    }
    const double per[3] = {d->increment * 4, d->increment * 4, d->increment * 2.5};
    double inv_vd[3];
    for (int a = 0; a < 3; ++a) {
        B.n[a] = (int)std::ceil((B.mx[a] - B.mn[a]) / per[a]);
        B.vd[a] = (B.mx[a] - B.mn[a]) / B.n[a];
        inv_vd[a] = 1 / B.vd[a];
    }
    B.inv.assign((size_t)B.n[0] * B.n[1] * B.n[2], {});
    for (int k = 0; k < B.M; ++k) {
        const double o[3] = {B.org[k].x, B.org[k].y, B.org[k].z};
        int lo[3], hi[3];
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::max(0, (int)std::floor((o[a] - B.r - B.mn[a]) * inv_vd[a]));
            hi[a] = std::min(B.n[a] - 1, (int)std::floor((o[a] + B.r - B.mn[a]) * inv_vd[a]));
        }
        for (int x = lo[0]; x <= hi[0]; ++x)
            for (int y = lo[1]; y <= hi[1]; ++y)
                for (int z = lo[2]; z <= hi[2]; ++z) {
                    const int ix[3] = {x, y, z};
                    double q[3];
                    for (int a = 0; a < 3; ++a) q[a] = std::max(B.cmin(a, ix[a]) - o[a], std::max(0.0, o[a] - B.cmax(a, ix[a])));
                    if (q[0] * q[0] + q[1] * q[1] + q[2] * q[2] < B.r2) B.inv[((size_t)x * B.n[1] + y) * B.n[2] + z].push_back(k);
                }
    }
    return true;
}

/* OBox.IsPointInBox and OBox.Intersect of Hare's AABB (not in the reference tree), restated as
 * inclusive bounds and the slab test of the half-line; the entry point is o + t_near d. */
inline bool map_inside(const MapBank &B, V3 p) {
    return p.x >= B.mn[0] && p.x <= B.mx[0] && p.y >= B.mn[1] && p.y <= B.mx[1] && p.z >= B.mn[2] && p.z <= B.mx[2];
}
inline bool map_entry(const MapBank &B, V3 o, V3 d, V3 &pt) {
    const double oo[3] = {o.x, o.y, o.z}, dd[3] = {d.x, d.y, d.z};
    double tn = 0, tf = INFINITY;
    for (int a = 0; a < 3; ++a) {
        if (dd[a] == 0) {
            if (oo[a] < B.mn[a] || oo[a] > B.mx[a]) return false;
            continue;
        }
        double t1 = (B.mn[a] - oo[a]) / dd[a], t2 = (B.mx[a] - oo[a]) / dd[a];
        if (t1 > t2) std::swap(t1, t2);
        tn = std::max(tn, t1);
        tf = std::min(tf, t2);
    }
    if (tn > tf) return false;
    pt = o + d * tn;
    return true;
}
/* (int)Math.Floor(x) for the cell indices, kept inside int range */
inline int floor_int(double x) {
    double f = std::floor(x);
    if (!(f > -2147483648.0)) return INT32_MIN;
    if (f > 2147483647.0) return INT32_MAX;
    return (int)f;
}

struct Ctx {
    const Scene &S;
    MapBank map;
    const orc_params &p;
    std::vector<Rec> recs;
    std::vector<V3> src_org;
    std::vector<std::array<double, 8>> src_pow;
    std::vector<int> src_kind;
    int nsrc;
    double COTime;
    int h_oct;
    int T;
    int rate;
    Ctx(const Scene &s, const orc_params &pp) : S(s), p(pp), nsrc(1), COTime(0), h_oct(0), T(0), rate(1000) {}
};


/* Spherical_Receiver.CheckRay geometry (Classes_Receivers.cs:837-850): returns the chord
 * midpoint t and the half chord, or false. */
inline bool sphere_test(const Rec &rc, V3 o, V3 d, V3 end, double &t, double &half) {
    double mx = o.x - rc.o.x, my = o.y - rc.o.y, mz = o.z - rc.o.z;
    double b = mx * d.x + my * d.y + mz * d.z;
    double c = mx * mx + my * my + mz * mz - rc.r2;
    if (c > 0 && b > 0) return false;
    double discr = b * b - c;
    if (discr < 0) return false;
    double t1 = -b - std::sqrt(discr), t2 = -b + std::sqrt(discr);
    t = (t1 + t2) * .5;
    double ex = end.x - o.x, ey = end.y - o.y, ez = end.z - o.z;
    if (!(t > 0 && t * t < ex * ex + ey * ey + ez * ez)) return false;
    half = (t2 - t1) * 0.5;
    return true;
}

struct Worker {
    Ctx &C;
    Tracer tr;
    Hist H;
    orc_stats st{};
    std::vector<ORay> queue;
    std::vector<double> mE, mP;       /* map histograms [M][8][T] */
    std::vector<double> mDp, mDn;     /* directional maps: [M][3][8][T] */
    std::vector<uint32_t> stamp;      /* Map_Receiver.Ray_ID: the walk that last tested the receiver */
    uint32_t walk_id = 0;
    Worker(Ctx &c) : C(c), tr(c.S) {
        H.init((int)c.recs.size(), c.T);
        if (c.map.M) {
            mE.assign((size_t)c.map.M * 8 * c.map.T, 0);
            mP.assign((size_t)c.map.M * 8 * c.map.T, 0);
            if (c.map.directional) {
                mDp.assign((size_t)c.map.M * 24 * c.map.T, 0);
                mDn.assign((size_t)c.map.M * 24 * c.map.T, 0);
            }
            stamp.assign(c.map.M, 0);
        }
    }

    /* CheckBroadbandRay (broadband) / CheckRay (Pach_Map_Receiver.cs:1359-1631) with the
     * Ray_ID mailbox of CheckReceivers_* (349-408): test(k) once for every receiver listed in a
     * visited cell.  walk 0 is the reference's code: the broadband walk indexes from the ray's
     * origin (unclipped), steers by the sign of the POSITION (R.x where R.dx is meant) and stops
     * when any index reaches the end cell's; the octave walk starts at the entry point and stops on
     * reaching the end cell, unvisited.  walk 1 visits every crossed cell, the end cell included. */
    template <class F> void map_walk(V3 o, V3 d, V3 end, bool broadband, F test) {
        const MapBank &B = C.map;
        const bool quirk = broadband && B.walk == 0;
        V3 s = o;
        if (!map_inside(B, o)) {
            V3 pt = o;
            if (!map_entry(B, o, d, pt)) return;
            if (!quirk) s = pt;
        }
        const double sp[3] = {s.x, s.y, s.z}, ep[3] = {end.x, end.y, end.z};
        const double g[3] = {quirk ? o.x : d.x, quirk ? o.y : d.y, quirk ? o.z : d.z};
        int c[3], ce[3], step[3];
        double tmax[3], tdel[3];
        for (int a = 0; a < 3; ++a) {
            c[a] = floor_int((sp[a] - B.mn[a]) / B.vd[a]);
            ce[a] = floor_int((ep[a] - B.mn[a]) / B.vd[a]);
        }
        for (int a = 0; a < 3; ++a) c[a] = c[a] < 0 ? 0 : (c[a] >= B.n[a] ? B.n[a] - 1 : c[a]);
        for (int a = 0; a < 3; ++a)
            if ((g[a] < 0 && c[a] < ce[a]) || (g[a] >= 0 && c[a] > ce[a])) return;
        for (int a = 0; a < 3; ++a) {
            step[a] = g[a] < 0 ? -1 : 1;
            tmax[a] = ((g[a] < 0 ? B.cmin(a, c[a]) : B.cmax(a, c[a])) - sp[a]) / g[a];
            tdel[a] = B.vd[a] / g[a] * step[a];
        }
        if (++walk_id == 0) { std::fill(stamp.begin(), stamp.end(), 0u); walk_id = 1; }
        for (;;) {
            for (int k : B.cell(c[0], c[1], c[2])) {
                if (stamp[k] == walk_id) continue;
                stamp[k] = walk_id;
                test(k);
            }
            if (B.walk && c[0] == ce[0] && c[1] == ce[1] && c[2] == ce[2]) return;
            int a;
            if (tmax[0] < tmax[1]) a = tmax[0] < tmax[2] ? 0 : 2;
            else a = tmax[1] < tmax[2] ? 1 : 2;
            c[a] += step[a];
            if (c[a] < 0 || c[a] >= B.n[a]) return;  /* outside grid */
            tmax[a] = tmax[a] + tdel[a];
            if (quirk) { if (!(c[0] != ce[0] && c[1] != ce[1] && c[2] != ce[2])) return; }
            else if (B.walk == 0) { if (!(c[0] != ce[0] || c[1] != ce[1] || c[2] != ce[2])) return; }
        }
    }

    /* Histogram.Add / Histogram_1Pt.Add / Directional_Histogram.Add (Classes_Receivers.cs:1159-1166,
     * 1393-1396, 1813-1825), 1000 Hz; d = the ray direction (the arrival direction is -d) */
    void map_add(int k, int oct, double time, double e, V3 d) {
        const MapBank &B = C.map;
        size_t i = ((size_t)k * 8 + oct) * B.T;
        if (B.one_pt) { mE[i] += e; return; }
        const double x = time * 1000;
        if (!(x > -1) || x >= B.T) return;   /* (int) truncates: (-1, 0) is sample 0 */
        const int sample = (int)x;
        mE[i + sample] += e;
        if (!B.directional) { mP[i + sample] += std::sqrt(e); return; }
        mP[i + sample] += std::sqrt(e * B.rho_c);
        const double c[3] = {-d.x, -d.y, -d.z};
        for (int a = 0; a < 3; ++a) {
            const size_t j = (((size_t)k * 3 + a) * 8 + oct) * B.T + sample;
            const double v = (double)(float)(c[a] * e);
            if (c[a] > 0) mDp[j] += v; else mDn[j] += v;
        }
    }

    /* Map_Receiver.CheckRay / CheckBroadbandRay geometry (Pach_Map_Receiver.cs:1780-1826) */
    bool map_hit(int k, V3 o, V3 d, V3 end, double &t) const {
        const MapBank &B = C.map;
        double mx = o.x - B.org[k].x, my = o.y - B.org[k].y, mz = o.z - B.org[k].z;
        double b = mx * d.x + my * d.y + mz * d.z;
        double c = mx * mx + my * my + mz * mz - B.r2;
        if (c > 0 && b > 0) return false;
        double discr = b * b - c;
        if (discr < 0) return false;
        double t1 = -b - std::sqrt(discr), t2 = -b + std::sqrt(discr);
        t = (t1 + t2) / 2;
        double ex = end.x - o.x, ey = end.y - o.y, ez = end.z - o.z;
        return t > 0 && t * t < ex * ex + ey * ey + ez * ez;
    }
    void map_octave(const ORay &R, V3 end, double scale) {
        const MapBank &B = C.map;
        map_walk(R.p, R.d, end, false, [&](int k) {
            double t;
            if (!map_hit(k, R.p, R.d, end, t)) return;
            st.detections++;
            double raydist = t / B.c + R.t_sum - B.direct[k];
            map_add(k, R.oct, raydist, R.I * scale * std::pow(10, -.1 * B.atten[R.oct] * raydist) * B.sizemod, R.d);
        });
    }
    void map_broad(V3 o, V3 d, double t_sum, const double E[8], V3 end) {
        const MapBank &B = C.map;
        map_walk(o, d, end, true, [&](int k) {
            double t;
            if (!map_hit(k, o, d, end, t)) return;
            st.detections++;
            double raydist = t / B.c + t_sum - B.direct[k];
            for (int oct = 0; oct < 8; ++oct) map_add(k, oct, raydist, E[oct] * std::pow(10, -.1 * B.atten[oct] * raydist) * B.sizemod, d);
        });
    }

    /* Receiver_Bank.CheckRay -> Spherical_Receiver.CheckRay (Classes_Receivers.cs:197-200, 837-877). */
    void check_ray(const ORay &R, V3 end, double scale) {
        for (int r = 0; r < (int)C.recs.size(); ++r) {
            double t, half;
            if (!sphere_test(C.recs[r], R.p, R.d, end, t, half)) continue;
            double time = t / C.S.c + R.t_sum;
            double e = R.I * scale * std::pow(10, -.1 * C.S.atten[R.oct] * time * C.S.c) * (1 / kPi) * half;
            int sample = (int)(time * C.rate);
            st.detections++;
            if (sample < C.T) {
                H.add(r, R.oct, sample, e, R.d, C.S.rho_c);
                bool spec = (R.mask & 1) == 0, was = (R.mask & 2) == 2;
                H.analysis(r, spec ? (was ? 2 : 0) : 1, R.oct, sample, e);
            }
        }
    }

    /* Spherical_Receiver.CheckBroadbandRay (Classes_Receivers.cs:803-829). */
    void check_broad(V3 o, V3 d, double t_sum, const double E[8], V3 end) {
        for (int r = 0; r < (int)C.recs.size(); ++r) {
            double t, half;
            if (!sphere_test(C.recs[r], o, d, end, t, half)) continue;
            double time = t / C.S.c + t_sum;
            double dist = time * C.S.c;
            int sample = (int)(time * C.rate);
            st.detections++;
            for (int oct = C.p.oct_lo; oct <= C.p.oct_hi; ++oct) {
                double e = E[oct] * std::pow(10, -.1 * C.S.atten[oct] * dist) * (1 / kPi) * half;
                if (sample < C.T) {
                    H.add(r, oct, sample, e, d, C.S.rho_c);
                    H.analysis(r, 0, oct, sample, e);
                }
            }
        }
    }

    /* One primary ray: cast_ray_distributed (TaskAll:335-486) with End_Trace (TaskAll:489-536). */
    void primary(int64_t ray, const double *dir_override, double weight) {
        const Scene &S = C.S;
        int s = (int)((ray + 1) % C.nsrc);               /* SourceCluster round robin (Classes_Sources.cs:712-722) */
        double dir[3];
        if (dir_override) { dir[0] = dir_override[0]; dir[1] = dir_override[1]; dir[2] = dir_override[2]; }
        else orc_emit_direction(C.p.seed, ray, C.nsrc, C.src_kind[s], dir);
        double E[8];
        for (int o = 0; o < 8; ++o) E[o] = C.src_pow[s][o] * weight;
        for (int o = 0; o < 8; ++o) st.initial_energy += E[o];
        double TP1 = E[C.h_oct] * 1e-2, TP2[8], TP3[8];
        for (int o = 0; o < 8; ++o) { TP2[o] = E[o] * std::pow(10, -4.5); TP3[o] = E[o] * 1e-9; }
        V3 pos = C.src_org[s], d{dir[0], dir[1], dir[2]};
        double t_sum = 0;
        int order = 0;
        queue.clear();
        const int maxA = C.p.max_broadband_bounces;
        bool lost = false;
        /* ---- phase A: broadband ---- */
        do {
            Hit h;
            st.segments++; st.segments_broadband++;
            if (!tr.shoot(pos, d, h)) {
                if (order > C.p.is_order) {
                    check_broad(pos, d, t_sum, E, pos + d * 1000000);
                    if (C.map.M) map_broad(pos, d, t_sum, E, pos + d * 1000000);
                }
                for (int j = 0; j < 8; ++j) st.lost_energy += E[j];
                lost = true;
                break;
            }
            if (order > C.p.is_order) {
                check_broad(pos, d, t_sum, E, h.x);
                if (C.map.M) map_broad(pos, d, t_sum, E, h.x);
            }
            t_sum += h.t / S.c;
            pos = h.x;
            int k = order;  /* index of this broadband bounce */
            order++;
            V3 n = S.normal[h.poly];
            double cos_t = dot(d, n);                       /* Basic_Material.Absorb (Classes_Materials.cs:166-178) */
            for (int o = 0; o < 8; ++o) E[o] *= (1 - S.alpha[h.poly * 8 + o]);
            /* Scatter_Early (Classes_Materials.cs:4498-4570) */
            if (cos_t > 0) { n = n * -1; cos_t = -cos_t; }
            for (int o = 0; o < 8; ++o) {
                if (E[o] == 0) continue;
                double sc = S.scat[h.poly * 8 + o];
                ORay R{pos, d, E[o] * sc, t_sum, TP3[o], o, 0, sid_early(k, o, 0), 0};
                E[o] *= (1 - sc);
                Block B = draw_block(C.p.seed, ray, R.sid, 0);
                R.d = lambert_dir(n, B.u[0], B.u[1], false);
                R.mask |= 3;
                double tau = S.trans[h.poly * 8 + o];
                if (tau > 0) {
                    ORay trr{pos, d, E[o] * tau, t_sum, TP3[o], o, 0, sid_early(k, o, 1), 0};
                    E[o] *= (1 - tau);
                    trr.mask &= ~1;
                    queue.push_back(trr);
                    ORay td = R;
                    td.I = R.I * tau; R.I *= (1 - tau);
                    td.d = td.d * -1;
                    td.mask |= 3;
                    td.sid = sid_early(k, o, 2);
                    queue.push_back(td);
                }
                queue.push_back(R);
            }
            d = d - n * (cos_t * 2);
            if (maxA > 0 && order >= maxA && E[C.h_oct] > TP1) { st.capped++; break; }
        } while (E[C.h_oct] > TP1);
        if (!lost) {
            for (int o = C.p.oct_lo; o <= C.p.oct_hi; ++o) {
                ORay R{pos, d, E[o], t_sum, TP3[o], o, 0, sid_final(o), 0};
                E[o] = 0;
                queue.push_back(R);
            }
        }
        st.octave_rays += (int64_t)queue.size();
        /* ---- phases B and C: octave rays from the queue ---- */
        const double scale = 1.0;
        const int64_t cap = C.p.max_segments_per_ray > 0 ? C.p.max_segments_per_ray : (1ll << 22);
        while (!queue.empty()) {
            ORay R = queue.back();
            queue.pop_back();
            bool dead = false;
            int64_t nseg = 0;
            do {
                Hit h;
                st.segments++; st.segments_phase_b++; nseg++;
                if (!tr.shoot(R.p, R.d, h)) {
                    check_ray(R, R.p + R.d * 1000000, scale);
                    if (C.map.M) map_octave(R, R.p + R.d * 1000000, scale);
                    st.lost_energy += R.I;
                    dead = true;
                    break;
                }
                check_ray(R, h.x, scale);
                if (C.map.M) map_octave(R, h.x, scale);
                R.t_sum += h.t / S.c;
                R.p = h.x;
                V3 n = S.normal[h.poly];
                double cos_t = dot(n, R.d);
                R.I *= (1 - S.alpha[h.poly * 8 + R.oct]);
                Block B = draw_block(C.p.seed, ray, R.sid, 1 + R.nb);
                uint32_t nb = R.nb++;
                bool transmit = B.u[0] < S.trans[h.poly * 8 + R.oct];
                /* Scatter_Late (Classes_Materials.cs:4629-4701) */
                double th[3];
                lambert_thresholds(S.scat[h.poly * 8 + R.oct], th);
                double sel = B.u[1];
                if (C.p.pure_specular || sel > th[2]) {
                    R.d = R.d - n * (cos_t * 2);
                    if (transmit) R.d = R.d * -1;
                    R.mask &= ~1;
                } else {
                    if (sel > th[0]) {
                        ORay c = R;
                        c.I = R.I * (1 - th[1]);
                        R.I *= (1 - (1 - th[1]));
                        c.mask &= ~1;
                        c.d = R.d - n * (cos_t * 2);
                        if (transmit) c.d = c.d * -1;
                        c.sid = sid_late(R.sid, nb);
                        c.nb = 0;
                        queue.push_back(c);
                        st.octave_rays++;
                    }
                    V3 nn = cos_t > 0 ? n * -1 : n;
                    R.d = lambert_dir(nn, B.u[2], B.u[3], false);
                    R.mask |= 3;
                    if (transmit) R.d = R.d * -1;
                }
                if (nseg >= cap) { st.capped++; dead = true; break; }
            } while (R.t_sum < C.COTime && R.I > TP2[R.oct]);
            if (dead) continue;
            /* End_Trace (TaskAll:489-536) with Scatter_VeryLate (Classes_Materials.cs:4572-4627) */
            st.end_traces++;
            do {
                Hit h;
                st.segments++; st.segments_phase_c++; nseg++;
                if (!tr.shoot(R.p, R.d, h)) {
                    check_ray(R, R.p + R.d * 1000000, scale);
                    if (C.map.M) map_octave(R, R.p + R.d * 1000000, scale);
                    st.lost_energy += R.I;
                    break;
                }
                check_ray(R, h.x, scale);
                if (C.map.M) map_octave(R, h.x, scale);
                R.t_sum += h.t / S.c;
                R.p = h.x;
                V3 n = S.normal[h.poly];
                double cos_t = dot(n, R.d);
                R.I *= (1 - S.alpha[h.poly * 8 + R.oct]);
                Block B = draw_block(C.p.seed, ray, R.sid, 1 + R.nb);
                R.nb++;
                bool transmit = B.u[0] < S.trans[h.poly * 8 + R.oct];
                if (!C.p.pure_specular && B.u[1] < S.scat[h.poly * 8 + R.oct]) {
                    V3 nn = cos_t > 0 ? n * -1 : n;
                    R.d = lambert_dir(nn, B.u[2], B.u[3], true);
                    R.mask |= 3;
                } else {
                    R.d = R.d - n * (cos_t * 2);
                    R.mask &= ~1;
                }
                if (transmit) R.d = R.d * -1;
                if (nseg >= cap) { st.capped++; break; }
            } while (R.t_sum < C.COTime && R.I > R.decim);
        }
        st.primaries++;
    }
};

}  // namespace

/* ======================================================================================== */
extern "C" {

void orc_philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1, uint32_t out[4]) {
    uint32_t c[4] = {c0, c1, c2, c3};
    philox(c, k0, k1);
    for (int i = 0; i < 4; ++i) out[i] = c[i];
}

void orc_medium(double temp_c, double hr, double pa_hpa, int air_choice, int edge_correction,
                double atten_db_per_m[8], double *sound_speed, double *rho) {
    double Tk = temp_c + 273.15;
    attenuation(air_choice, pa_hpa / 10, Tk, hr, edge_correction, atten_db_per_m);
    if (sound_speed) *sound_speed = 331 + 0.6 * (Tk - 273.15);
    if (rho) *rho = density(Tk, pa_hpa * 100, hr);
}

/* GeodesicSource.GeoSphere(1) (Classes_Sources.cs:290-350): icosahedron, one subdivision. */
static void geosphere(std::vector<std::array<V3, 3>> &F) {
    double sqr5 = std::sqrt(5.0), phi = (1.0 + sqr5) * 0.5;
    double ratio = std::sqrt(10.0 + 2.0 * sqr5) / (4.0 * phi);
    double a = (.25 / ratio) * 0.5, b = (.25 / ratio) / (2.0 * phi);
    V3 P[12] = {{0, b, -a}, {b, a, 0}, {-b, a, 0}, {0, b, a}, {0, -b, a}, {-a, 0, b},
                {0, -b, -a}, {a, 0, -b}, {a, 0, b}, {-a, 0, -b}, {b, -a, 0}, {-b, -a, 0}};
    for (auto &p : P) p = normalized(p);
    const int T[20][3] = {{0, 1, 2}, {3, 2, 1}, {3, 4, 5}, {3, 8, 4}, {0, 6, 7}, {0, 9, 6}, {4, 10, 11},
                          {6, 11, 10}, {2, 5, 9}, {11, 9, 5}, {1, 7, 8}, {10, 8, 7}, {3, 5, 2}, {3, 1, 8},
                          {0, 2, 9}, {0, 7, 1}, {6, 9, 11}, {6, 10, 7}, {4, 11, 5}, {4, 8, 10}};
    F.clear();
    for (auto &t : T) {
        V3 p0 = P[t[0]], p1 = P[t[1]], p2 = P[t[2]];
        V3 p3 = normalized((p0 + p1) * 0.5), p4 = normalized((p1 + p2) * 0.5), p5 = normalized((p2 + p0) * 0.5);
        F.push_back({p0, p3, p5});
        F.push_back({p1, p4, p3});
        F.push_back({p2, p5, p4});
        F.push_back({p3, p4, p5});
    }
}

void orc_emit_direction(uint64_t seed, int64_t ray, int32_t n_src, int32_t kind, double dir[3]) {
    Block B = draw_block(seed, ray, 0, 0);
    V3 d;
    if (kind == 1) {
        /* RandomSource.Directions (Classes_Sources.cs:256-265): theta, phi ~ U[0, 2pi). */
        double th = B.u[0] * 2 * kPi, ph = B.u[1] * 2 * kPi;
        d = {std::sin(th) * std::cos(ph), std::sin(th) * std::sin(ph), std::cos(th)};
    } else if (kind == 2) {
        double z = 1 - 2 * B.u[0], ph = B.u[1] * 2 * kPi, r = std::sqrt(std::max(0.0, 1 - z * z));
        d = {r * std::cos(ph), r * std::sin(ph), z};
    } else {
        /* GeodesicSource.Directions (Classes_Sources.cs:390-403): face (per-source ray count) mod 80,
         * a random point on the face (Hare Polygon.GetRandomPoint, restated as the uniform
         * triangle map with reflection), normalised. */
        static std::vector<std::array<V3, 3>> F;
        static std::once_flag once;
        std::call_once(once, [] { geosphere(F); });
        int64_t j = ray / (n_src > 0 ? n_src : 1);
        const auto &f = F[(size_t)(j % 80)];
        double u = B.u[0], v = B.u[1];
        if (u + v > 1) { u = 1 - u; v = 1 - v; }
        d = normalized(f[0] + (f[1] - f[0]) * u + (f[2] - f[0]) * v);
    }
    dir[0] = d.x; dir[1] = d.y; dir[2] = d.z;
}

int orc_shoot(const orc_scene_desc *scene, int32_t grid_domain, int32_t brute_force,
              const double o[3], const double d[3], int32_t *poly, double *t, double hit[3]) {
    Scene S;
    build_scene(scene, grid_domain, brute_force != 0, false, S);
    Tracer tr(S);
    Hit h;
    V3 dd = normalized(V3{d[0], d[1], d[2]});
    if (!tr.shoot(V3{o[0], o[1], o[2]}, dd, h)) { *poly = -1; *t = 0; return 0; }
    *poly = h.poly; *t = h.t;
    hit[0] = h.x.x; hit[1] = h.x.y; hit[2] = h.x.z;
    return 1;
}

/* Direct_Sound.Check_Validity and the direct-path energy (Classes_Direct.cs:654-685, 772-823): shoot
 * from the source towards the receiver; a hit before the full source-receiver distance through a
 * polygon with any transmission multiplies the band transmissions and continues from the hit point
 * (its next hit again compared with the full distance, as coded); energy
 * P 10^(-0.1 m L) prod(tau) / (4 pi L^2). */
int orc_direct(const orc_scene_desc *scene, int32_t grid_domain, int32_t n_src, const orc_source *src,
               int32_t n_rec, const orc_receiver *rec, int32_t *valid, double *distance, double *energy) {
    Scene S;
    build_scene(scene, grid_domain, false, false, S);
    Tracer tr(S);
    for (int k = 0; k < n_rec; ++k)
        for (int s = 0; s < n_src; ++s) {
            const size_t p = (size_t)k * n_src + s;
            const V3 so{src[s].origin[0], src[s].origin[1], src[s].origin[2]};
            const V3 ro{rec[k].origin[0], rec[k].origin[1], rec[k].origin[2]};
            V3 d = V3{ro.x - so.x, ro.y - so.y, ro.z - so.z};
            const double L = std::sqrt(d.x * d.x + d.y * d.y + d.z * d.z);
            d = normalized(d);
            double tm[8] = {1, 1, 1, 1, 1, 1, 1, 1};
            V3 o = so;
            int ok = 1;
            for (int c = 0; c < 64; ++c) {
                Hit h;
                if (!tr.shoot(o, d, h)) { ok = 1; break; }
                ok = h.t >= L ? 1 : 0;
                bool transmissive = false;
                for (int b = 0; b < 8; ++b) transmissive = transmissive || S.trans[h.poly * 8 + b] > 0;
                if (ok || !transmissive) break;
                for (int b = 0; b < 8; ++b) tm[b] *= S.trans[h.poly * 8 + b];
                o = h.x;
            }
            valid[p] = ok;
            distance[p] = L;
            for (int b = 0; b < 8; ++b) {
                const double P = 1e-12 * std::pow(10.0, 0.1 * src[s].power_db[b]);
                energy[p * 8 + b] = P * std::pow(10.0, -0.1 * S.atten[b] * L) * tm[b] / (4 * M_PI * L * L);
            }
        }
    return 0;
}

int orc_specular_paths(const orc_scene_desc *scene, int32_t grid_domain, int32_t brute_force,
                       int32_t n, const double *origins, const double *dirs, int32_t max_bounces,
                       int32_t *poly_out, double *t_out, double *pts_out) {
    Scene S;
    build_scene(scene, grid_domain, brute_force != 0, true, S);
    Tracer tr(S);
    for (int i = 0; i < n; ++i) {
        V3 p{origins[3 * i], origins[3 * i + 1], origins[3 * i + 2]};
        V3 d = normalized(V3{dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]});
        for (int b = 0; b < max_bounces; ++b) {
            size_t k = (size_t)i * max_bounces + b;
            poly_out[k] = -1; t_out[k] = 0;
            pts_out[3 * k] = pts_out[3 * k + 1] = pts_out[3 * k + 2] = 0;
        }
        for (int b = 0; b < max_bounces; ++b) {
            size_t k = (size_t)i * max_bounces + b;
            Hit h;
            if (!tr.shoot(p, d, h)) break;
            poly_out[k] = h.poly; t_out[k] = h.t;
            pts_out[3 * k] = h.x.x; pts_out[3 * k + 1] = h.x.y; pts_out[3 * k + 2] = h.x.z;
            V3 nrm = S.normal[h.poly];
            d = d - nrm * (2 * dot(d, nrm));
            p = h.x;
        }
    }
    return 0;
}

int orc_trace_ex(const orc_scene_desc *scene, int32_t n_src, const orc_source *src,
                 int32_t n_rec, const orc_receiver *rec, const orc_params *pp,
                 int64_t ray_begin, int64_t ray_end, int32_t n_threads,
                 const double *prim_dirs, const double *prim_weights,
                 double *energy, double *pressure, double *dir_pos, double *dir_neg, double *analysis,
                 orc_stats *stats) {
    return orc_trace_map(scene, n_src, src, n_rec, rec, nullptr, pp, ray_begin, ray_end, n_threads, prim_dirs,
                         prim_weights, energy, pressure, dir_pos, dir_neg, analysis, nullptr, nullptr, nullptr, stats);
}

int orc_trace_map(const orc_scene_desc *scene, int32_t n_src, const orc_source *src,
                  int32_t n_rec, const orc_receiver *rec, const orc_map_desc *map, const orc_params *pp,
                  int64_t ray_begin, int64_t ray_end, int32_t n_threads,
                  const double *prim_dirs, const double *prim_weights,
                  double *energy, double *pressure, double *dir_pos, double *dir_neg, double *analysis,
                  double *map_energy, double *map_pressure, double *map_direct, orc_stats *stats) {
    if (!scene || !src || n_src < 1 || !pp || ray_end < ray_begin) return -1;
    if (pp->oct_lo < 0 || pp->oct_hi > 7 || pp->oct_lo > pp->oct_hi) return -1;
    Scene S;
    build_scene(scene, pp->grid_domain, pp->brute_force != 0, pp->pure_specular != 0, S);
    orc_params p = *pp;
    Ctx C(S, p);
    C.nsrc = n_src;
    for (int i = 0; i < n_rec; ++i) C.recs.push_back(Rec{{rec[i].origin[0], rec[i].origin[1], rec[i].origin[2]}, rec[i].radius * rec[i].radius});
    double cluster_pow[8] = {0};
    for (int s = 0; s < n_src; ++s) {
        C.src_org.push_back({src[s].origin[0], src[s].origin[1], src[s].origin[2]});
        std::array<double, 8> pw;
        for (int o = 0; o < 8; ++o) { pw[o] = 1e-12 * std::pow(10, .1 * src[s].power_db[o]); cluster_pow[o] = std::max(cluster_pow[o], pw[o]); }
        C.src_pow.push_back(pw);
        C.src_kind.push_back(src[s].kind);
    }
    /* TaskAll:83-109: COTime and h_oct. */
    C.COTime = p.cutoff_length_m / S.c;
    double totalAbs[8] = {0};
    for (int q = 0; q < S.P; ++q)
        for (int o = p.oct_lo; o <= p.oct_hi; ++o) totalAbs[o] += S.area[q] * S.alpha[q * 8 + o];
    double mn = 1e308 * 10, octpower = 0;
    C.h_oct = 0;
    for (int o = p.oct_lo; o <= p.oct_hi; ++o) if (cluster_pow[o] > octpower) octpower = cluster_pow[o];
    for (int o = p.oct_lo; o <= p.oct_hi; ++o) {
        if (cluster_pow[o] < octpower * 1E-6) continue;
        if (mn > totalAbs[o]) { mn = totalAbs[o]; C.h_oct = o; }
    }
    C.rate = p.sample_rate;
    C.T = (int)((double)p.sample_rate * (p.hist_cotime_ms / 1000.0));
    if (C.T < 1) return -1;
    if (map && !build_map(map, C.src_org[0], n_src, S.c, S.atten, C.map)) return -1;
    C.map.rho_c = S.rho_c;
    /* Derived phase-A bound: E[h] shrinks at least by fmax per bounce. */
    if (p.max_broadband_bounces <= 0) {
        double fmax = 0;
        for (int q = 0; q < S.P; ++q) fmax = std::max(fmax, (1 - S.alpha[q * 8 + C.h_oct]) * (1 - S.scat[q * 8 + C.h_oct]) * (1 - S.trans[q * 8 + C.h_oct]));
        if (fmax >= 1.0) p.max_broadband_bounces = 100000;
        else p.max_broadband_bounces = std::min(100000, (int)std::floor(std::log(1e-2) / std::log(fmax)) + 2);
    }
    int nt = n_threads > 0 ? n_threads : (int)std::max(1u, std::thread::hardware_concurrency());
    int64_t N = ray_end - ray_begin;
    if (nt > N) nt = (int)std::max<int64_t>(1, N);
    std::vector<Worker *> W;
    for (int t = 0; t < nt; ++t) W.push_back(new Worker(C));
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t) {
        int64_t a = ray_begin + (int64_t)((double)t * N / nt), b = (t == nt - 1) ? ray_end : ray_begin + (int64_t)((double)(t + 1) * N / nt);
        th.emplace_back([&, t, a, b] {
            for (int64_t r = a; r < b; ++r)
                W[t]->primary(r, prim_dirs ? prim_dirs + 3 * (r - ray_begin) : nullptr,
                              prim_weights ? prim_weights[r - ray_begin] : 1.0);
        });
    }
    for (auto &x : th) x.join();
    size_t nE = (size_t)n_rec * 8 * C.T, nD = (size_t)n_rec * 24 * C.T;
    orc_stats out{};
    for (int t = 0; t < nt; ++t) {
        Worker &w = *W[t];
        for (size_t i = 0; i < nE; ++i) {
            if (energy) energy[i] = (t ? energy[i] : 0) + w.H.E[i];
            if (pressure) pressure[i] = (t ? pressure[i] : 0) + w.H.Pr[i];
        }
        for (size_t i = 0; i < nD; ++i) {
            if (dir_pos) dir_pos[i] = (t ? dir_pos[i] : 0) + w.H.Dp[i];
            if (dir_neg) dir_neg[i] = (t ? dir_neg[i] : 0) + w.H.Dn[i];
            if (analysis) analysis[i] = (t ? analysis[i] : 0) + w.H.An[i];
        }
        out.primaries += w.st.primaries; out.segments += w.st.segments;
        out.segments_broadband += w.st.segments_broadband; out.segments_phase_b += w.st.segments_phase_b;
        out.segments_phase_c += w.st.segments_phase_c; out.octave_rays += w.st.octave_rays;
        out.end_traces += w.st.end_traces; out.detections += w.st.detections; out.capped += w.st.capped;
        out.cells_visited += w.tr.cells_visited; out.tri_tests += w.tr.tri_tests;
        out.lost_energy += w.st.lost_energy; out.initial_energy += w.st.initial_energy;
        const size_t nm = w.mE.size();
        for (size_t i = 0; i < nm; ++i) {
            if (map_energy) map_energy[i] = (t ? map_energy[i] : 0) + w.mE[i];
            if (map_pressure) map_pressure[i] = (t ? map_pressure[i] : 0) + w.mP[i];
        }
        if (t == 0) { g_map_dp.assign(w.mDp.size(), 0.0); g_map_dn.assign(w.mDn.size(), 0.0); }
        for (size_t i = 0; i < w.mDp.size(); ++i) { g_map_dp[i] += w.mDp[i]; g_map_dn[i] += w.mDn[i]; }
        delete W[t];
    }
    if (map_direct) for (int k = 0; k < C.map.M; ++k) map_direct[k] = C.map.direct[k];
    out.h_oct = C.h_oct; out.bins = C.T; out.cotime_s = C.COTime; out.sound_speed = S.c; out.rho_c = S.rho_c;
    for (int o = 0; o < 8; ++o) out.air_atten_db_per_m[o] = S.atten[o];
    if (stats) *stats = out;
    return 0;
}

int orc_map_directions(double *dir_pos, double *dir_neg, size_t cap) {
    if (g_map_dp.empty() || cap < g_map_dp.size()) return 0;
    if (dir_pos) std::copy(g_map_dp.begin(), g_map_dp.end(), dir_pos);
    if (dir_neg) std::copy(g_map_dn.begin(), g_map_dn.end(), dir_neg);
    return 1;
}

int orc_trace(const orc_scene_desc *scene, int32_t n_src, const orc_source *src,
              int32_t n_rec, const orc_receiver *rec, const orc_params *p,
              int64_t ray_begin, int64_t ray_end, int32_t n_threads,
              double *energy, double *pressure, double *dir_pos, double *dir_neg, double *analysis,
              orc_stats *stats) {
    return orc_trace_ex(scene, n_src, src, n_rec, rec, p, ray_begin, ray_end, n_threads, nullptr, nullptr,
                        energy, pressure, dir_pos, dir_neg, analysis, stats);
}

/* ---------------------------------------------------------------------------------------
 * Room-acoustic parameters (Classes_Math.cs).
 * ------------------------------------------------------------------------------------- */
void orc_schroeder(const double *etc, int32_t n, double *out) {       /* Schroeder_Integral 282-299 */
    double sum = 0;
    std::vector<double> b(n);
    for (int i = 0; i < n; ++i) b[i] = sum += etc[i];
    for (int i = 0; i < n; ++i) out[i] = sum == 0 ? 0 : 1 - b[i] / sum;
}

static std::vector<double> log10data(const double *x, int n, double lim) {  /* Log10Data 392-408 */
    std::vector<double> o(n, 0.0);
    double lv = std::pow(10, lim / 10);
    for (int i = 1; i <= n - 1; ++i) o[i] = x[i] >= lv ? 10 * std::log10(x[i]) : lim;
    return o;
}

static void limits(const std::vector<double> &l, double a, double b, int L[2]) {  /* Schroeder_Limits 417-438 */
    L[0] = L[1] = 0;
    int n = (int)l.size();
    for (int i = 1; i <= n - 1; ++i) if (l[i] < a) { L[0] = i; break; }
    for (int i = L[0]; i <= n - 1; ++i) if (l[i] < b) { L[1] = i; break; }
}

static double lsf_slope(const double *m, int len, double fs) {       /* Least_Square_Fit 446-473 */
    double ts = 0, ms = 0, tt = 0, tm = 0;
    for (int i = 0; i <= len - 1; ++i) { double q = i / fs; ts += q; ms += m[i]; tt += q * q; tm += q * m[i]; }
    return ((len * tm) - (ts * ms)) / ((len * tt) - (ts * ts));
}

double orc_t_x(const double *sch, int32_t n, int32_t depth, int32_t fs) {   /* T_X 511-526 */
    auto l = log10data(sch, n, -60);
    int L[2];
    limits(l, -5, -5 - std::abs(depth), L);
    int len = L[1] - L[0] + 1;
    if (len < 1) return std::nan("");
    return -60 / lsf_slope(l.data() + L[0], len, fs);
}

double orc_edt(const double *sch, int32_t n, int32_t fs) {             /* EarlyDecayTime 534-549 */
    auto l = log10data(sch, n, -60);
    int L[2];
    limits(l, -1, -10.0001, L);
    int len = L[1] - L[0] + 1;
    if (len < 1) return std::nan("");
    return -60 / lsf_slope(l.data() + L[0], len, fs);
}

double orc_clarity(const double *etc, int32_t n, double fs, double seconds, double start, int32_t pressure) { /* 559-586 */
    if (pressure) seconds += 8192.0 / fs;
    double bw = 1 / fs;
    int si = (int)std::floor(start * fs), ei = (int)std::floor((seconds + start) * fs);
    double early = 0, late = 0;
    for (int q = si; q < ei && q < n; ++q) early += etc[q];
    double split = (seconds + start - (ei * bw)) / bw;
    if (ei < n) early += split * etc[ei];
    for (int q = ei + 1; q < n; ++q) late += etc[q];
    if (ei < n) late += (1 - split) * etc[ei];
    return 10 * std::log10(early / late);
}

double orc_definition(const double *etc, int32_t n, double fs, double seconds, double start, int32_t pressure) { /* 934-962 */
    if (pressure) start += 8192.0 / fs;
    double bw = 1 / fs;
    int si = (int)std::floor(start * fs);
    int ei = (int)std::floor(seconds * fs) + si;
    double early = 0, all = 0;
    for (int q = 0; q < ei && q < n; ++q) early += etc[q];
    double split = (seconds + start - (ei * bw)) / bw;
    if (ei < n) early += split * etc[ei];
    for (int q = 0; q < n; ++q) all += etc[q];
    return early / all * 100;
}

double orc_center_time(const double *etc, int32_t n, int32_t fs, double direct, int32_t pressure) { /* 971-986 */
    if (pressure) direct += 8192.0 / fs;
    double spt = 0, st = 0, bw = 1 / (double)fs;
    int start = (int)std::floor(direct * fs);
    for (int i = std::max(start, 0); i < n; ++i) { spt += etc[i] * (i * bw - direct); st += etc[i]; }
    return spt / st;
}

double orc_strength(const double *etc, int32_t n, double swl, int32_t pressure) {  /* 993-1005 */
    (void)pressure;
    double all = 0;
    for (int q = 0; q < n; ++q) all += etc[q];
    double spl = 10 * std::log10(all / 1e-12);   /* SPL_Intensity (Classes_Math.cs:97-102) */
    if (spl < 0) spl = 0;
    return spl - swl + 31;
}

}  // extern "C"
