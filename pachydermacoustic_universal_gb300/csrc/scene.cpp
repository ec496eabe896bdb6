// scene.cpp -- host-side scene preparation for the device tracer.
//
// Restates Polygon_Scene.Construct / partition (Classes_Scenes.cs:447-630, 727-755) for a GPU:
// polygons are fan-triangulated (polygon id kept per triangle), flat polygon normals and areas are
// computed in FP64 (Classes_Scenes.cs:864-872, 894-897), coplanar triangles share a plane id (used
// to skip the surface a ray leaves), and a uniform grid (count -> scan -> fill) replaces Hare's
// Voxel_Grid.  Air properties follow Uniform_Medium (Classes_Medium_Props.cs:286-299).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <tuple>

#include "engine.h"

namespace pach {
namespace {

struct D3 { double x, y, z; };
inline D3 sub(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline D3 add(D3 a, D3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline D3 mul(D3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline double dot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline D3 cross(D3 a, D3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline D3 unit(D3 a) { double l = std::sqrt(dot(a, a)); return l > 0 ? mul(a, 1.0 / l) : a; }

// Separating-axis overlap of a triangle and an axis-aligned box (Akenine-Moller, JGT 2001),
// restated: 9 edge-cross axes, the 3 box normals and the triangle normal.
bool tri_box(D3 a, D3 b, D3 c, D3 ctr, D3 h) {
    D3 v0 = sub(a, ctr), v1 = sub(b, ctr), v2 = sub(c, ctr);
    D3 e[3] = {sub(v1, v0), sub(v2, v1), sub(v0, v2)};
    D3 V[3] = {v0, v1, v2};
    const double hh[3] = {h.x, h.y, h.z};
    for (int i = 0; i < 3; ++i) {
        for (int k = 0; k < 3; ++k) {
            D3 ax = k == 0 ? D3{0, -e[i].z, e[i].y} : (k == 1 ? D3{e[i].z, 0, -e[i].x} : D3{-e[i].y, e[i].x, 0});
            double p0 = dot(V[0], ax), p1 = dot(V[1], ax), p2 = dot(V[2], ax);
            double mn = std::min({p0, p1, p2}), mx = std::max({p0, p1, p2});
            double r = hh[0] * std::fabs(ax.x) + hh[1] * std::fabs(ax.y) + hh[2] * std::fabs(ax.z);
            double tol = 1e-9 * (r + std::fabs(mn) + std::fabs(mx)) + 1e-15;
            if (mn > r + tol || mx < -r - tol) return false;
        }
    }
    const double cs[3][3] = {{v0.x, v1.x, v2.x}, {v0.y, v1.y, v2.y}, {v0.z, v1.z, v2.z}};
    for (int a2 = 0; a2 < 3; ++a2) {
        double mn = std::min({cs[a2][0], cs[a2][1], cs[a2][2]}), mx = std::max({cs[a2][0], cs[a2][1], cs[a2][2]});
        double tol = 1e-9 * hh[a2] + 1e-15;
        if (mn > hh[a2] + tol || mx < -hh[a2] - tol) return false;
    }
    D3 n = cross(e[0], e[1]);
    double d = dot(n, v0);
    double r = hh[0] * std::fabs(n.x) + hh[1] * std::fabs(n.y) + hh[2] * std::fabs(n.z);
    return std::fabs(d) <= r * (1 + 1e-9) + 1e-15;
}

}  // namespace

// Calculate_Attenuation (Classes_Medium_Props.cs:51-191) as coded, including the C# integer
// divisions in the exponents (-1/2 -> 0, -1/3 -> 0, -5/2 -> -2, 1/2 -> 0); called by the
// Uniform_Medium ctor with Pa/10 (hPa -> kPa).  Density: Calculate_Density(Tk, Pa*100, hr).
void medium_properties(double temp_c, double hr, double pa_hpa, int air_choice, int edge, double atten[kBands],
                       double *c, double *rho) {
    static const double F[kBands] = {62.5, 125, 250, 500, 1000, 2000, 4000, 8000};
    const double Tk = temp_c + 273.15, Pa = pa_hpa / 10.0;
    for (int o = 0; o < kBands; ++o) atten[o] = 0.0;
    if (air_choice == 0) {
        const double h = hr * std::pow(10.0, -6.8346 * std::pow(273.16 / Tk, 1.261) + 4.6151) / (Pa / 101.325);
        const int e_half = -1 / 2, e_third = -1 / 3, e_fivehalf = -5 / 2, e_pos_half = 1 / 2;
        for (int o = 0; o < kBands; ++o) {
            double frO = (Pa / 101.325) * (24 + 4.04e4 * h * ((0.02 + h) / (0.391 + h)));
            double frN = (Pa / 101.325) * std::pow(Tk / 293.15, (double)e_half) *
                         (9 + 280 * h * std::exp(-4.170 * (std::pow(Tk / 293.15, (double)e_third) - 1)));
            double z = 0.1068 * std::exp(-3352 / Tk) / (frN + F[o] * F[o] / frN);
            double y = std::pow(Tk / 293.15, (double)e_fivehalf) *
                       (0.01275 * std::exp(-2239.1 / Tk) / (frO + F[o] * F[o] / frO) + z);
            atten[o] = 8.686 * F[o] * F[o] * ((1.84e-11 / (Pa / 101.325) * std::pow(Tk / 293.15, (double)e_pos_half)) + y);
        }
    } else if (air_choice == 1) {
        for (int o = 0; o < kBands; ++o) {
            double m = ((85 / hr) * ((F[o] / 1000) * (F[o] / 1000) * 0.0001)) / 8.7;
            m -= 0.04 * (Tk - 273.15 - 20) * m;
            atten[o] = m * 0.50248756218905477;
        }
    } else if (air_choice == 2) {
        static const double W[3][kBands] = {{0.0001, 0.0001, 0.0003, 0.0006, 0.001, 0.0019, 0.0058, 0.0203},
                                            {0.0001, 0.0001, 0.0003, 0.0006, 0.001, 0.0017, 0.0041, 0.0135},
                                            {0.0001, 0.0001, 0.0003, 0.0006, 0.0011, 0.0017, 0.0035, 0.0106}};
        static const double Cd[3][kBands] = {{0.0001, 0.0001, 0.0002, 0.0005, 0.0011, 0.0027, 0.0094, 0.029},
                                             {0.0001, 0.0001, 0.0002, 0.0005, 0.0008, 0.0018, 0.0059, 0.0211},
                                             {0.0001, 0.0001, 0.0002, 0.0005, 0.0007, 0.0014, 0.0044, 0.0158}};
        const double(*tab)[kBands] = (Tk - 273.15 > 15) ? W : Cd;
        int row = hr < 50 ? 0 : hr < 70 ? 1 : hr > 70 ? 2 : -1;  // hr == 70 falls through every branch
        if (row >= 0)
            for (int o = 0; o < kBands; ++o) atten[o] = tab[row][o];
        if (edge)
            for (int o = 0; o < kBands; ++o) atten[o] /= std::sqrt(2.0);
    }
    if (c) *c = 331 + 0.6 * (Tk - 273.15);                      // AcousticalMath.SoundSpeed
    if (rho) {
        const double P = pa_hpa * 100, Rd = 287.05, T = Tk - 273.15;
        const double Pv = hr * 6.1078 * std::pow(10.0, (7.5 * T) / (237.3 + T));
        *rho = (P / (Rd * Tk)) * (1 - 0.378 * Pv / P);
    }
}

// GeodesicSource.GeoSphere(1) (Classes_Sources.cs:290-350): the 20 icosahedron faces, each split
// once into 4 (corner, corner, corner, centre order), 80 faces of 3 unit vertices.
void geodesic_faces(std::vector<double> &out) {
    const double s5 = std::sqrt(5.0), phi = (1.0 + s5) * 0.5;
    const double ratio = std::sqrt(10.0 + 2.0 * s5) / (4.0 * phi);
    const double a = (.25 / ratio) * 0.5, b = (.25 / ratio) / (2.0 * phi);
    D3 P[12] = {{0, b, -a}, {b, a, 0}, {-b, a, 0}, {0, b, a}, {0, -b, a}, {-a, 0, b},
                {0, -b, -a}, {a, 0, -b}, {a, 0, b}, {-a, 0, -b}, {b, -a, 0}, {-b, -a, 0}};
    for (auto &p : P) p = unit(p);
    static const int T[20][3] = {{0, 1, 2}, {3, 2, 1}, {3, 4, 5}, {3, 8, 4}, {0, 6, 7}, {0, 9, 6}, {4, 10, 11},
                                 {6, 11, 10}, {2, 5, 9}, {11, 9, 5}, {1, 7, 8}, {10, 8, 7}, {3, 5, 2}, {3, 1, 8},
                                 {0, 2, 9}, {0, 7, 1}, {6, 9, 11}, {6, 10, 7}, {4, 11, 5}, {4, 8, 10}};
    out.clear();
    auto put = [&](D3 x, D3 y, D3 z) {
        for (D3 v : {x, y, z}) { out.push_back(v.x); out.push_back(v.y); out.push_back(v.z); }
    };
    for (auto &t : T) {
        D3 p0 = P[t[0]], p1 = P[t[1]], p2 = P[t[2]];
        D3 p3 = unit(mul(add(p0, p1), 0.5)), p4 = unit(mul(add(p1, p2), 0.5)), p5 = unit(mul(add(p2, p0), 0.5));
        put(p0, p3, p5);
        put(p1, p4, p3);
        put(p2, p5, p4);
        put(p3, p4, p5);
    }
}

// Phase A ends when E[h_oct] <= 1e-2 E0 (TaskAll:351, 417); each broadband bounce multiplies
// E[h_oct] by at most max over surfaces of (1-alpha)(1-s)(1-tau), which bounds the bounce count.
unsigned long long derived_broadband_bound(const HostScene &hs, int h, bool pure) {
    double fmax = 0;
    for (int p = 0; p < hs.npoly; ++p) {
        double f = (1 - hs.alpha[p * 8 + h]) * (pure ? 1.0 : (1 - hs.scat[p * 8 + h]) * (1 - hs.trans[p * 8 + h]));
        fmax = std::max(fmax, f);
    }
    if (fmax >= 1.0) return 0;  // lossless: the reference loop would not terminate
    if (fmax <= 0.0) return 1;
    double k = std::floor(std::log(1e-2) / std::log(fmax)) + 2;
    return (unsigned long long)std::min(k, 1e6);
}

bool build_host_scene(const pach_scene_desc *d, HostScene &hs, std::string &err) {
    if (!d || d->n_vertices <= 0 || !d->vertices || d->n_polys <= 0 || !d->poly_offsets || !d->poly_indices ||
        !d->absorption || !d->scattering) {
        err = "scene: missing vertices, polygons or coefficients";
        return false;
    }
    hs = HostScene();
    hs.npoly = d->n_polys;
    const int nv = d->n_vertices;
    for (int i = 0; i < 3 * nv; ++i)
        if (!std::isfinite(d->vertices[i])) { err = "scene: non-finite vertex coordinate"; return false; }
    auto V = [&](int i) { return D3{d->vertices[3 * i], d->vertices[3 * i + 1], d->vertices[3 * i + 2]}; };
    hs.alpha.assign(d->absorption, d->absorption + 8 * (size_t)hs.npoly);
    hs.scat.assign(d->scattering, d->scattering + 8 * (size_t)hs.npoly);
    if (d->transmission) hs.trans.assign(d->transmission, d->transmission + 8 * (size_t)hs.npoly);
    else hs.trans.assign(8 * (size_t)hs.npoly, 0.0);
    for (size_t i = 0; i < hs.alpha.size(); ++i) {
        if (!(hs.alpha[i] >= 0 && hs.alpha[i] <= 1) || !(hs.scat[i] >= 0 && hs.scat[i] <= 1) ||
            !(hs.trans[i] >= 0 && hs.trans[i] <= 1)) {
            err = "scene: absorption, scattering and transmission must lie in [0, 1]";
            return false;
        }
        if (hs.trans[i] > 0) hs.has_trans = true;
    }
    hs.normal.resize(3 * (size_t)hs.npoly);
    hs.area.resize(hs.npoly);
    for (int k = 0; k < 3; ++k) { hs.bmin[k] = 1e300; hs.bmax[k] = -1e300; }
    for (int p = 0; p < hs.npoly; ++p) {
        int b = d->poly_offsets[p], e = d->poly_offsets[p + 1];
        if (e - b < 3 || b < 0) { err = "scene: polygon " + std::to_string(p) + " has fewer than 3 vertices"; return false; }
        for (int k = b; k < e; ++k)
            if (d->poly_indices[k] < 0 || d->poly_indices[k] >= nv) { err = "scene: vertex index out of range"; return false; }
        D3 n{0, 0, 0};
        for (int k = b; k < e; ++k) {  // Newell
            D3 p0 = V(d->poly_indices[k]), p1 = V(d->poly_indices[k + 1 < e ? k + 1 : b]);
            n.x += (p0.y - p1.y) * (p0.z + p1.z);
            n.y += (p0.z - p1.z) * (p0.x + p1.x);
            n.z += (p0.x - p1.x) * (p0.y + p1.y);
        }
        hs.area[p] = 0.5 * std::sqrt(dot(n, n));
        if (!(hs.area[p] > 0)) { err = "scene: degenerate polygon " + std::to_string(p); return false; }
        D3 u = unit(n);
        hs.normal[3 * p] = u.x; hs.normal[3 * p + 1] = u.y; hs.normal[3 * p + 2] = u.z;
        D3 a = V(d->poly_indices[b]);
        for (int k = b + 1; k + 1 < e; ++k) {
            D3 pb = V(d->poly_indices[k]), pc = V(d->poly_indices[k + 1]);
            D3 e1 = sub(pb, a), e2 = sub(pc, a);
            if (dot(cross(e1, e2), cross(e1, e2)) == 0) continue;  // zero-area fan piece
            const double t9[9] = {a.x, a.y, a.z, e1.x, e1.y, e1.z, e2.x, e2.y, e2.z};
            hs.tri64.insert(hs.tri64.end(), t9, t9 + 9);
            hs.tri_poly.push_back(p);
        }
        for (int k = b; k < e; ++k) {
            D3 q = V(d->poly_indices[k]);
            hs.bmin[0] = std::min(hs.bmin[0], q.x); hs.bmin[1] = std::min(hs.bmin[1], q.y); hs.bmin[2] = std::min(hs.bmin[2], q.z);
            hs.bmax[0] = std::max(hs.bmax[0], q.x); hs.bmax[1] = std::max(hs.bmax[1], q.y); hs.bmax[2] = std::max(hs.bmax[2], q.z);
        }
    }
    hs.ntri = (int)hs.tri_poly.size();
    if (hs.ntri == 0) { err = "scene: no triangles"; return false; }
    double ext[3];
    for (int k = 0; k < 3; ++k) ext[k] = hs.bmax[k] - hs.bmin[k];
    hs.scale = std::max({ext[0], ext[1], ext[2], 1e-3});
    const double pad = 1e-5 * hs.scale;
    for (int k = 0; k < 3; ++k) { hs.bmin[k] -= pad; hs.bmax[k] += pad; ext[k] = hs.bmax[k] - hs.bmin[k]; }

    // Coplanar groups: quantised (canonical normal, offset) of each triangle's own plane.
    std::map<std::tuple<long long, long long, long long, long long>, int> planes;
    hs.tri_plane.resize(hs.ntri);
    for (int i = 0; i < hs.ntri; ++i) {
        const double *t = &hs.tri64[9 * (size_t)i];
        D3 n = unit(cross(D3{t[3], t[4], t[5]}, D3{t[6], t[7], t[8]}));
        if (n.x < 0 || (n.x == 0 && (n.y < 0 || (n.y == 0 && n.z < 0)))) n = mul(n, -1);
        double off = dot(n, D3{t[0], t[1], t[2]}) / hs.scale;
        auto key = std::make_tuple(std::llround(n.x * 1e6), std::llround(n.y * 1e6), std::llround(n.z * 1e6),
                                   std::llround(off * 1e6));
        auto it = planes.find(key);
        if (it == planes.end()) it = planes.emplace(key, (int)planes.size()).first;
        hs.tri_plane[i] = it->second;
    }

    // Uniform grid: about `lambda` cells per triangle, cubic cells.
    double lambda = d->grid_cells_per_tri > 0 ? d->grid_cells_per_tri : 4.0;
    double vol = ext[0] * ext[1] * ext[2];
    double h = std::cbrt(vol / (lambda * hs.ntri));
    long long total = 1;
    for (int k = 0; k < 3; ++k) {
        hs.dims[k] = (int)std::max(1.0, std::min(1024.0, std::round(ext[k] / h)));
        total *= hs.dims[k];
    }
    while (total > (1ll << 24)) {
        total = 1;
        for (int k = 0; k < 3; ++k) { hs.dims[k] = std::max(1, hs.dims[k] / 2); total *= hs.dims[k]; }
    }
    const D3 bmin{hs.bmin[0], hs.bmin[1], hs.bmin[2]};
    const D3 cell{ext[0] / hs.dims[0], ext[1] / hs.dims[1], ext[2] / hs.dims[2]};
    std::vector<uint32_t> counts((size_t)total + 1, 0);
    std::vector<std::pair<uint32_t, uint32_t>> pairs;  // (cell, tri)
    pairs.reserve((size_t)hs.ntri * 4);
    for (int i = 0; i < hs.ntri; ++i) {
        const double *t = &hs.tri64[9 * (size_t)i];
        D3 a{t[0], t[1], t[2]}, b = add(a, D3{t[3], t[4], t[5]}), c = add(a, D3{t[6], t[7], t[8]});
        D3 lo{std::min({a.x, b.x, c.x}), std::min({a.y, b.y, c.y}), std::min({a.z, b.z, c.z})};
        D3 hi{std::max({a.x, b.x, c.x}), std::max({a.y, b.y, c.y}), std::max({a.z, b.z, c.z})};
        auto cl = [&](double v, double mn, double cs, int n) {
            int k = (int)std::floor((v - mn) / cs);
            return std::min(std::max(k, 0), n - 1);
        };
        int x0 = cl(lo.x, bmin.x, cell.x, hs.dims[0]), x1 = cl(hi.x, bmin.x, cell.x, hs.dims[0]);
        int y0 = cl(lo.y, bmin.y, cell.y, hs.dims[1]), y1 = cl(hi.y, bmin.y, cell.y, hs.dims[1]);
        int z0 = cl(lo.z, bmin.z, cell.z, hs.dims[2]), z1 = cl(hi.z, bmin.z, cell.z, hs.dims[2]);
        D3 hh = mul(cell, 0.5 * (1 + 1e-6));
        for (int x = x0; x <= x1; ++x)
            for (int y = y0; y <= y1; ++y)
                for (int z = z0; z <= z1; ++z) {
                    D3 ctr{bmin.x + (x + 0.5) * cell.x, bmin.y + (y + 0.5) * cell.y, bmin.z + (z + 0.5) * cell.z};
                    if (!tri_box(a, b, c, ctr, hh)) continue;
                    uint32_t ci = (uint32_t)(((size_t)z * hs.dims[1] + y) * hs.dims[0] + x);
                    pairs.emplace_back(ci, (uint32_t)i);
                    counts[ci]++;
                }
    }
    hs.cell_start.assign((size_t)total + 1, 0);
    for (long long ci = 0; ci < total; ++ci) hs.cell_start[ci + 1] = hs.cell_start[ci] + counts[ci];
    hs.cell_tris.assign(pairs.size(), 0);
    std::vector<uint32_t> fill(hs.cell_start.begin(), hs.cell_start.end() - 1);
    for (auto &pr : pairs) hs.cell_tris[fill[pr.first]++] = pr.second;

    medium_properties(d->temp_c, d->rel_humidity, d->pressure_hpa, d->air_choice, d->edge_correction, hs.atten,
                      &hs.c, &hs.rho);
    hs.rho_c = hs.rho * hs.c;
    if (!(hs.c > 0)) { err = "scene: non-positive sound speed"; return false; }
    return true;
}

}  // namespace pach
