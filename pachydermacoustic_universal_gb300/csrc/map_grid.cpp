// map_grid.cpp -- host set-up of mapping receivers (PachMapReceiver.Partition and the
// Map_Receiver ctor, Pach_Map_Receiver.cs:98-263, 1721-1768): the receivers' uniform grid with its
// per-cell receiver lists, the direct arrival times and the histogram length.
#include <algorithm>
#include <cmath>

#include "engine.h"

namespace pach {

bool build_map_grid(const pach_map_desc &d, const double src[3], int nsrc, double c, MapGrid &g, std::string &err) {
    if (d.n_receivers < 1 || !d.origins) { err = "map: no receivers"; return false; }
    if (!(d.increment > 0) || !std::isfinite(d.increment)) { err = "map: increment must be positive"; return false; }
    if (!d.time_1pt && !(d.cutoff_ms >= 1.0)) { err = "map: cutoff_ms must be at least 1"; return false; }
    if (d.walk != 0 && d.walk != 1) { err = "map: walk must be 0 or 1"; return false; }
    const int M = d.n_receivers;
    for (size_t i = 0; i < 3 * (size_t)M; ++i)
        if (!std::isfinite(d.origins[i])) { err = "map: receiver origins must be finite"; return false; }
    g.M = M;
    g.one_pt = d.time_1pt != 0;
    g.walk = d.walk;
    g.directional = d.directional != 0;
    if (g.directional && g.one_pt) { err = "map: a one-point histogram has no directions"; return false; }
    // Histogram(SampleRate 1000, COTime_in ms): CO_Time = COTime_in / 1000, SampleCT = (int)(CO_Time * 1000)
    g.T = g.one_pt ? 1 : (int)(d.cutoff_ms / 1000.0 * 1000.0);
    if (g.T < 1) { err = "map: no histogram bins"; return false; }
    g.r = d.increment * 0.5;
    g.r2 = g.r * g.r;
    // bounding box of the spheres (Partition, 161-170)
    for (int a = 0; a < 3; ++a) { g.mn[a] = HUGE_VAL; g.mx[a] = -HUGE_VAL; }
    for (int k = 0; k < M; ++k)
        for (int a = 0; a < 3; ++a) {
            const double o = d.origins[3 * k + a];
            g.mx[a] = std::max(g.mx[a], o + d.increment * .5);
            g.mn[a] = std::min(g.mn[a], o - d.increment * .5);
        }
    // cells of 4 x 4 x 2.5 increments (174-181)
    const double per[3] = {d.increment * 4, d.increment * 4, d.increment * 2.5};
    double cells = 1;
    for (int a = 0; a < 3; ++a) {
        g.n[a] = (int)std::ceil((g.mx[a] - g.mn[a]) / per[a]);
        if (g.n[a] < 1) g.n[a] = 1;
        g.vd[a] = (g.mx[a] - g.mn[a]) / g.n[a];
        cells *= g.n[a];
    }
    if (cells > (double)(1 << 26)) { err = "map: the receiver grid would need more than 2^26 cells"; return false; }
    const int nc = (int)cells;
    auto cell_of = [&](int x, int y, int z) { return (x * g.n[1] + y) * g.n[2] + z; };
    // receivers per cell: the sphere-box test of the registration loop (210-245)
    std::vector<std::vector<int>> lists((size_t)nc);
    std::vector<std::vector<int>> rec_cells((size_t)M);
    const double inv[3] = {1 / g.vd[0], 1 / g.vd[1], 1 / g.vd[2]};
    for (int k = 0; k < M; ++k) {
        const double *o = d.origins + 3 * k;
        int lo[3], hi[3];
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::max(0, (int)std::floor((o[a] - g.r - g.mn[a]) * inv[a]));
            hi[a] = std::min(g.n[a] - 1, (int)std::floor((o[a] + g.r - g.mn[a]) * inv[a]));
        }
        for (int x = lo[0]; x <= hi[0]; ++x)
            for (int y = lo[1]; y <= hi[1]; ++y)
                for (int z = lo[2]; z <= hi[2]; ++z) {
                    const int ix[3] = {x, y, z};
                    double dd = 0;
                    for (int a = 0; a < 3; ++a) {
                        const double bmin = (ix[a] * g.vd[a]) + g.mn[a], bmax = ((ix[a] + 1) * g.vd[a]) + g.mn[a];
                        const double q = std::max(bmin - o[a], std::max(0.0, o[a] - bmax));
                        dd += q * q;
                    }
                    if (dd < g.r2) {
                        lists[(size_t)cell_of(x, y, z)].push_back(k);
                        rec_cells[(size_t)k].push_back(cell_of(x, y, z));
                    }
                }
    }
    // entries with the neighbour masks (a sphere spans at most two cells per axis: the cells are at
    // least 1.25 increments wide when an axis has more than one, and the diameter is one increment)
    auto coords = [&](int ci, int &x, int &y, int &z) {
        z = ci % g.n[2];
        y = (ci / g.n[2]) % g.n[1];
        x = ci / (g.n[2] * g.n[1]);
    };
    g.cell_off.assign((size_t)nc + 1, 0);
    g.entry.clear();
    for (int ci = 0; ci < nc; ++ci) {
        g.cell_off[(size_t)ci] = (int)g.entry.size();
        int cx, cy, cz;
        coords(ci, cx, cy, cz);
        for (int k : lists[(size_t)ci]) {
            uint32_t mask = 0;
            for (int cj : rec_cells[(size_t)k]) {
                if (cj == ci) continue;
                int x, y, z;
                coords(cj, x, y, z);
                const int dx = x - cx, dy = y - cy, dz = z - cz;
                if (dx < -1 || dx > 1 || dy < -1 || dy > 1 || dz < -1 || dz > 1) {
                    err = "map: a receiver spans more than two cells on an axis";
                    return false;
                }
                mask |= 1u << ((dx + 1) * 9 + (dy + 1) * 3 + (dz + 1));
            }
            g.entry.push_back({(uint32_t)k, mask});
        }
    }
    g.cell_off[(size_t)nc] = (int)g.entry.size();
    // direct arrival (Map_Receiver ctor, 1737-1751): |source - receiver| / c for one source; a
    // SourceCluster leaves it at min(0, ...) = 0
    g.direct.assign((size_t)M, 0.0);
    if (nsrc == 1)
        for (int k = 0; k < M; ++k) {
            const double lx = src[0] - d.origins[3 * k], ly = src[1] - d.origins[3 * k + 1],
                         lz = src[2] - d.origins[3 * k + 2];
            g.direct[(size_t)k] = std::sqrt(lx * lx + ly * ly + lz * lz) / c;
        }
    return true;
}

}  // namespace pach
