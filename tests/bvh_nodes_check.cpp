// Host check of the quantised BVH nodes the scene builder writes (csrc/scene.cpp quantize_bvh):
// every 48-byte node decodes, as the walk decodes it (csrc/device_common.cuh bvh4q_step), to the
// float node's children -- the same inner node ids and leaf codes -- every triangle sits in exactly
// one leaf, and every decoded child box contains the float child box with s / 256 to spare on each
// side (the margin the walk's folded decode needs).  Random triangle soups of several sizes and leaf
// limits; exit status 0 when all hold.  Built and run by tests/test_bvh_nodes.py (CPU only).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "../pachydermacoustic_universal_gb300/csrc/engine.h"

using namespace pach;

static int check(int ntri, int leaf_max, unsigned seed) {
    std::mt19937 rng(seed);
    std::uniform_real_distribution<double> pos(0, 50), jit(-1, 1);
    std::vector<double> v, ab((size_t)ntri * 8, 0.1), sc((size_t)ntri * 8, 0.2);
    std::vector<int> off{0}, idx;
    for (int t = 0; t < ntri; ++t) {
        const double c[3] = {pos(rng), pos(rng), 0.4 * pos(rng)};
        for (int k = 0; k < 3; ++k) {
            for (int a = 0; a < 3; ++a) v.push_back(c[a] + jit(rng));
            idx.push_back(3 * t + k);
        }
        off.push_back(3 * (t + 1));
    }
    pach_scene_desc d{};
    d.n_vertices = (int)v.size() / 3;
    d.vertices = v.data();
    d.n_polys = ntri;
    d.poly_offsets = off.data();
    d.poly_indices = idx.data();
    d.absorption = ab.data();
    d.scattering = sc.data();
    d.temp_c = 20;
    d.rel_humidity = 50;
    d.pressure_hpa = 1013.25;
    d.bvh_leaf_max = leaf_max;
    HostScene hs;
    std::string err;
    if (!build_host_scene(&d, hs, err)) {
        std::printf("build failed: %s\n", err.c_str());
        return 1;
    }
    const size_t nodes = hs.bvh.size() / kBvhNodeFloats;
    if (hs.bvhq.size() != nodes * kBvhQNodeFloats) {
        std::printf("no quantised copy\n");
        return 1;
    }
    long bad = 0, children = 0;
    std::vector<int> seen((size_t)hs.ntri, 0);
    for (size_t q = 0; q < nodes; ++q) {
        const float *f = &hs.bvh[q * kBvhNodeFloats];
        const float *g = &hs.bvhq[q * kBvhQNodeFloats];
        uint32_t e, w[8];
        std::memcpy(&e, &g[3], 4);
        std::memcpy(w, &g[4], sizeof(w));
        const uint32_t slots = (e >> 24) | ((w[7] >> 24) << 8);
        int inner = (int)w[6], tri = (int)(w[7] & 0xFFFFFFu);
        for (int k = 0; k < 4; ++k) {
            const int vv = (int)((slots >> (4 * k)) & 15u);
            const int id = vv == 0 ? inner : (vv <= 8 ? ~(tri * 16 + vv - 1) : (int)0x80000000);
            inner += vv == 0;
            tri += vv <= 8 ? vv : 0;
            int code;
            std::memcpy(&code, &f[24 + k], 4);
            bool valid = code != (int)0x80000000;
            for (int a = 0; a < 3; ++a) valid = valid && std::isfinite(f[8 * a + k]) && std::isfinite(f[8 * a + 4 + k]);
            if (!valid) {
                bad += vv != 15;
                continue;
            }
            ++children;
            bad += id != code;
            if (id >= 0) {
                bad += (size_t)id >= nodes;
            } else {
                const int c = ~id, first = c >> 4, cnt = (c & 15) + 1;
                if (first < 0 || first + cnt > hs.ntri) ++bad;
                else for (int t = 0; t < cnt; ++t) seen[(size_t)first + t]++;
            }
            for (int a = 0; a < 3; ++a) {
                const double s = std::ldexp(1.0, (int)((e >> (8 * a)) & 255u) - 127 + 8);
                const uint32_t wl = w[2 * a], wh = w[2 * a + 1];
                const double lo = (double)g[a] + (double)((wl >> (8 * k)) & 255u) * s;
                const double hi = (double)g[a] + (double)((wh >> (8 * k)) & 255u) * s;
                bad += !(lo <= (double)f[8 * a + k] - s / 256.0 && hi >= (double)f[8 * a + 4 + k] + s / 256.0);
            }
        }
    }
    long not_once = 0;
    for (int x : seen) not_once += x != 1;
    std::printf("triangles %d leaf max %d: nodes %zu, children %ld, mismatches %ld, triangles not in exactly one leaf %ld\n",
                hs.ntri, leaf_max, nodes, children, bad, not_once);
    return bad || not_once;
}

int main() {
    int fails = 0;
    const int sizes[] = {1, 2, 5, 37, 1000, 20000, 150000};
    for (int n : sizes) fails += check(n, 0, 11u + (unsigned)n);
    for (int leaf = 1; leaf <= kLeafMax; ++leaf) fails += check(5000, leaf, 97u + (unsigned)leaf);
    return fails ? 1 : 0;
}
