// scene.cpp -- host-side scene preparation for the device tracer.
//
// Restates Polygon_Scene.Construct / partition (Classes_Scenes.cs:447-630, 727-755) for a GPU:
// polygons are fan-triangulated (polygon id kept per triangle), flat polygon normals and areas are
// computed in FP64 (Classes_Scenes.cs:864-872, 894-897), coplanar triangles share a plane id (used
// to skip the surface a ray leaves), and a binned-SAH bounding volume hierarchy replaces Hare's
// Voxel_Grid as the nearest-hit structure (any structure that returns the nearest hit with t > eps
// gives the same answer).  Air properties follow Uniform_Medium (Classes_Medium_Props.cs:286-299).
#include <algorithm>
#include <atomic>
#include <array>
#include <cmath>
#include <cstring>
#include <future>
#include <map>
#include <thread>
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

// ---- BVH: binned SAH (16-64 bins, 3 axes), leaves of at most kLeafMax triangles ----
// The builder partitions an array of triangle references (box, centroid, triangle id) in place, so
// every pass over a node's range streams through contiguous memory.
struct BRef { float lo[3], hi[3], c[3]; int id; };
struct BNode { double lo[3], hi[3]; int left = -1, right = -1, first = 0, count = 0; };

// Subtrees of at least this many triangles, in the top levels, are built on their own threads (each
// into a builder of its own, appended in left-right order: the result equals the sequential build).
constexpr int kParallelBuildMin = 4096;
constexpr int kParallelBuildDepth = 5;
// Ranges of at least this many triangles are boxed and binned in parallel chunks.
constexpr int kParallelBinMin = 131072;
// SAH bins per axis: 16 for ranges below 256 triangles, up to 64 for large ones (n / 16).  The finer
// top-level splits cost the walk 2-3 % fewer node visits (measured on the 20k-triangle hall and the
// 500k-triangle arena); small ranges keep 16, where the sweep over the bins would dominate.
constexpr int kBinsMin = 16, kBinsMax = 64;
inline int bins_for(int n) { return std::min(kBinsMax, std::max(kBinsMin, n / 16)); }
// SAH cost of a split relative to testing one triangle: 1.6 x the parent's (measured best of 1.0,
// 1.6 and 2.2: the shallower tree saves more node visits than its extra triangle tests cost).
constexpr double kTraversalCost = 1.6;
constexpr bool kDepthFirstLayout = false;

// Node box and centroid box of a range (float min/max: exact in any order).
struct RangeBoxes {
    float lo[3], hi[3], clo[3], chi[3];
    void clear() {
        for (int k = 0; k < 3; ++k) { lo[k] = clo[k] = INFINITY; hi[k] = chi[k] = -INFINITY; }
    }
    void add(const RangeBoxes &o) {
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::min(lo[k], o.lo[k]); hi[k] = std::max(hi[k], o.hi[k]);
            clo[k] = std::min(clo[k], o.clo[k]); chi[k] = std::max(chi[k], o.chi[k]);
        }
    }
    void add(const BRef &x) {
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::min(lo[k], x.lo[k]); hi[k] = std::max(hi[k], x.hi[k]);
            clo[k] = std::min(clo[k], x.c[k]); chi[k] = std::max(chi[k], x.c[k]);
        }
    }
};

// Two-ended partition (each element tested once: from the front while it passes, from the back while
// it fails, then one swap), accumulating the boxes of both sides so that the children need no pass
// of their own for them.
template <class P>
BRef *partition_boxes(BRef *first, BRef *last, P pred, RangeBoxes &L, RangeBoxes &R) {
    L.clear();
    R.clear();
    for (;;) {
        for (;;) {
            if (first == last) return first;
            if (!pred(*first)) break;
            L.add(*first);
            ++first;
        }
        R.add(*first);  // fails: ends on the right (returned position or swapped to the back)
        --last;
        for (;;) {
            if (first == last) return first;
            if (pred(*last)) break;
            R.add(*last);
            --last;
        }
        L.add(*last);
        std::swap(*first, *last);
        ++first;
    }
}

// Per axis and bin: triangle count and the union of the triangles' boxes.
struct Bins {
    int nb = kBinsMin;
    int cnt[3][kBinsMax];
    float lo[3][kBinsMax][3], hi[3][kBinsMax][3];
    void clear(int bins) {
        nb = bins;
        for (int a = 0; a < 3; ++a)
            for (int q = 0; q < nb; ++q) {
                cnt[a][q] = 0;
                for (int k = 0; k < 3; ++k) { lo[a][q][k] = INFINITY; hi[a][q][k] = -INFINITY; }
            }
    }
    void add(const Bins &o) {
        for (int a = 0; a < 3; ++a)
            for (int q = 0; q < nb; ++q) {
                cnt[a][q] += o.cnt[a][q];
                for (int k = 0; k < 3; ++k) {
                    lo[a][q][k] = std::min(lo[a][q][k], o.lo[a][q][k]);
                    hi[a][q][k] = std::max(hi[a][q][k], o.hi[a][q][k]);
                }
            }
    }
};

inline int bin_of(float c, double clo, double ext, int nb) {
    return std::min(nb - 1, (int)(((double)c - clo) / ext * nb));
}

void range_boxes(const BRef *r, int b, int e, RangeBoxes &out) {
    out.clear();
    for (int i = b; i < e; ++i)
        for (int k = 0; k < 3; ++k) {
            out.lo[k] = std::min(out.lo[k], r[i].lo[k]); out.hi[k] = std::max(out.hi[k], r[i].hi[k]);
            out.clo[k] = std::min(out.clo[k], r[i].c[k]); out.chi[k] = std::max(out.chi[k], r[i].c[k]);
        }
}

// Bins [b, e) along every axis with a positive centroid extent, in one sweep.
void range_bins(const BRef *r, int b, int e, const double clo[3], const double ext[3], int nb, Bins &out) {
    out.clear(nb);
    bool live[3];
    for (int a = 0; a < 3; ++a) live[a] = ext[a] > 0;
    for (int i = b; i < e; ++i) {
        const BRef &x = r[i];
        for (int a = 0; a < 3; ++a) {
            if (!live[a]) continue;
            const int q = bin_of(x.c[a], clo[a], ext[a], nb);
            ++out.cnt[a][q];
            for (int k = 0; k < 3; ++k) {
                out.lo[a][q][k] = std::min(out.lo[a][q][k], x.lo[k]);
                out.hi[a][q][k] = std::max(out.hi[a][q][k], x.hi[k]);
            }
        }
    }
}

// f over [b, e) split into chunks run in parallel, merged with T::add (exact: min/max and counts).
template <class T, class F>
void reduce_range(int b, int e, T &out, F &&f) {
    const int n = e - b;
    if (n < kParallelBinMin) {
        f(b, e, out);
        return;
    }
    const int nt = (int)std::min<unsigned>(16u, std::max(1u, std::thread::hardware_concurrency()));
    const int step = (n + nt - 1) / nt;
    std::vector<T> part((size_t)nt);
    std::vector<std::future<void>> fut;
    for (int t = 1; t < nt; ++t) {
        const int c0 = b + t * step, c1 = std::min(e, c0 + step);
        fut.push_back(std::async(std::launch::async, [&, t, c0, c1] { f(c0, std::max(c0, c1), part[(size_t)t]); }));
    }
    f(b, std::min(e, b + step), part[0]);
    for (auto &x : fut) x.get();
    out = part[0];
    for (int t = 1; t < nt; ++t) out.add(part[(size_t)t]);
}

struct BvhBuilder {
    BRef *r = nullptr;              // shared by every builder of one tree (disjoint ranges)
    std::vector<BNode> nodes;
    std::vector<int> order;
    int max_depth = 0, leaves = 0;
    int leaf_max = kLeafMax;

    static double area(const double lo[3], const double hi[3]) {
        double e0 = std::max(0.0, hi[0] - lo[0]), e1 = std::max(0.0, hi[1] - lo[1]), e2 = std::max(0.0, hi[2] - lo[2]);
        return 2 * (e0 * e1 + e1 * e2 + e2 * e0);
    }

    int make_leaf(int b, int e, const RangeBoxes &bx) {
        BNode n;
        for (int k = 0; k < 3; ++k) { n.lo[k] = bx.lo[k]; n.hi[k] = bx.hi[k]; }
        n.first = (int)order.size();
        n.count = e - b;
        for (int i = b; i < e; ++i) order.push_back(r[i].id);
        nodes.push_back(n);
        ++leaves;
        return (int)nodes.size() - 1;
    }

    // appends a subtree builder's nodes and leaf order; returns its root's index here
    int append(const BvhBuilder &s, int root) {
        const int noff = (int)nodes.size(), ooff = (int)order.size();
        for (BNode n : s.nodes) {
            if (n.left >= 0) { n.left += noff; n.right += noff; }
            else n.first += ooff;
            nodes.push_back(n);
        }
        order.insert(order.end(), s.order.begin(), s.order.end());
        leaves += s.leaves;
        max_depth = std::max(max_depth, s.max_depth);
        return root + noff;
    }

    // known: the boxes of [b, e) when the parent's partition accumulated them
    int build(int b, int e, int depth, const RangeBoxes *known = nullptr) {
        max_depth = std::max(max_depth, depth);
        const int n = e - b;
        RangeBoxes bx;
        if (known) bx = *known;
        else reduce_range(b, e, bx, [this](int c0, int c1, RangeBoxes &o) { range_boxes(r, c0, c1, o); });
        if (n <= 2 || depth >= 56) {
            if (n <= leaf_max) return make_leaf(b, e, bx);
        }
        double clo[3], ext[3], nlo[3], nhi[3];
        for (int k = 0; k < 3; ++k) {
            clo[k] = bx.clo[k];
            ext[k] = (double)bx.chi[k] - clo[k];
            nlo[k] = bx.lo[k];
            nhi[k] = bx.hi[k];
        }
        const double parea = area(nlo, nhi);
        Bins bins;
        const int nb = bins_for(n);
        reduce_range(b, e, bins, [this, &clo, &ext, nb](int c0, int c1, Bins &o) { range_bins(r, c0, c1, clo, ext, nb, o); });
        double best = 1e300;
        int best_axis = -1, best_split = -1;
        for (int ax = 0; ax < 3; ++ax) {
            if (!(ext[ax] > 0)) continue;
            double rarea[kBinsMax];
            int rcnt[kBinsMax];
            double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
            int c = 0;
            for (int q = nb - 1; q > 0; --q) {
                c += bins.cnt[ax][q];
                for (int k = 0; k < 3; ++k) {
                    lo[k] = std::min(lo[k], (double)bins.lo[ax][q][k]);
                    hi[k] = std::max(hi[k], (double)bins.hi[ax][q][k]);
                }
                rarea[q] = area(lo, hi);
                rcnt[q] = c;
            }
            for (int k = 0; k < 3; ++k) { lo[k] = 1e300; hi[k] = -1e300; }
            c = 0;
            for (int q = 0; q < nb - 1; ++q) {
                c += bins.cnt[ax][q];
                for (int k = 0; k < 3; ++k) {
                    lo[k] = std::min(lo[k], (double)bins.lo[ax][q][k]);
                    hi[k] = std::max(hi[k], (double)bins.hi[ax][q][k]);
                }
                if (c == 0 || rcnt[q + 1] == 0) continue;
                const double cost = kTraversalCost + (area(lo, hi) * c + rarea[q + 1] * rcnt[q + 1]) / parea;
                if (cost < best) { best = cost; best_axis = ax; best_split = q; }
            }
        }
        if (n <= leaf_max && (best_axis < 0 || best >= (double)n)) return make_leaf(b, e, bx);
        int mid;
        RangeBoxes lbx, rbx;
        bool split_boxes = false;
        if (best_axis < 0) {
            mid = b + n / 2;  // coincident centroids: split the list
        } else {
            const double c0 = clo[best_axis], ex = ext[best_axis];
            BRef *it = partition_boxes(r + b, r + e, [&](const BRef &x) { return bin_of(x.c[best_axis], c0, ex, nb) <= best_split; },
                                       lbx, rbx);
            mid = (int)(it - r);
            split_boxes = true;
            if (mid == b || mid == e) {
                mid = b + n / 2;
                split_boxes = false;
            }
        }
        const RangeBoxes *lk = split_boxes ? &lbx : nullptr, *rk = split_boxes ? &rbx : nullptr;
        BNode node;
        for (int k = 0; k < 3; ++k) { node.lo[k] = nlo[k]; node.hi[k] = nhi[k]; }
        nodes.push_back(node);
        const int me = (int)nodes.size() - 1;
        if (n >= kParallelBuildMin && depth < kParallelBuildDepth) {
            // both halves on their own builders (disjoint ranges of the shared reference array)
            BvhBuilder L, R;
            L.r = R.r = r;
            L.leaf_max = R.leaf_max = leaf_max;
            auto fl = std::async(std::launch::async, [&] { return L.build(b, mid, depth + 1, lk); });
            const int rr = R.build(mid, e, depth + 1, rk);
            const int lr = fl.get();
            const int l = append(L, lr);
            const int rt = append(R, rr);
            nodes[me].left = l;
            nodes[me].right = rt;
            return me;
        }
        const int l = build(b, mid, depth + 1, lk);
        const int rt = build(mid, e, depth + 1, rk);
        nodes[me].left = l;
        nodes[me].right = rt;
        return me;
    }
};

// Builds hs.bvh and reorders the triangle arrays into leaf order.
void build_bvh(HostScene &hs, int leaf_max) {
    BvhBuilder B;
    B.leaf_max = (leaf_max >= 1 && leaf_max <= kLeafMax) ? leaf_max : kLeafDefault;
    std::vector<BRef> refs((size_t)hs.ntri);
    parallel_chunks((size_t)hs.ntri, 65536, [&](size_t i0, size_t i1) {
        for (size_t i = i0; i < i1; ++i) {
            const double *q = &hs.tri64[9 * i];
            BRef &x = refs[i];
            for (int k = 0; k < 3; ++k) {
                const double a = q[k], b = q[k] + q[3 + k], c = q[k] + q[6 + k];
                x.lo[k] = (float)std::min({a, b, c});
                x.hi[k] = (float)std::max({a, b, c});
                x.c[k] = (float)((a + b + c) / 3.0);
            }
            x.id = (int)i;
        }
    });
    B.r = refs.data();
    int root = B.build(0, hs.ntri, 0);
    // The device walk starts at an inner node: wrap a leaf root.
    if (B.nodes[root].left < 0) {
        BNode top;
        for (int k = 0; k < 3; ++k) { top.lo[k] = B.nodes[root].lo[k]; top.hi[k] = B.nodes[root].hi[k]; }
        BNode empty;
        for (int k = 0; k < 3; ++k) { empty.lo[k] = 1e300; empty.hi[k] = -1e300; }
        empty.first = 0;
        empty.count = 1;
        B.nodes.push_back(empty);
        top.left = root;
        top.right = (int)B.nodes.size() - 1;
        B.nodes.push_back(top);
        root = (int)B.nodes.size() - 1;
    }
    // Collapse to a 4-wide tree: an inner node's children are its binary descendants, opened
    // largest-surface-area first until four (or only leaves) remain.  Nodes are laid out
    // breadth-first so that the levels every ray walks share cache lines.
    auto area_of = [&](int n) { return BvhBuilder::area(B.nodes[n].lo, B.nodes[n].hi); };
    auto open = [&](int n, std::vector<int> &kids) {
        kids.assign({B.nodes[n].left, B.nodes[n].right});
        while (kids.size() < 4) {
            int best = -1;
            double ba = -1;
            for (int k = 0; k < (int)kids.size(); ++k)
                if (B.nodes[kids[k]].left >= 0 && area_of(kids[k]) > ba) { ba = area_of(kids[k]); best = k; }
            if (best < 0) break;
            const int x = kids[best];
            kids[best] = B.nodes[x].left;
            kids.push_back(B.nodes[x].right);
        }
    };
    // the 4-wide children of every inner binary node, in parallel chunks (the breadth-first pass below
    // reads those of the nodes it keeps)
    std::vector<std::array<int, 4>> open4(B.nodes.size());
    std::vector<signed char> nopen4(B.nodes.size(), 0);
    parallel_chunks(B.nodes.size(), 16384, [&](size_t n0, size_t n1) {
        std::vector<int> kk;
        for (size_t n = n0; n < n1; ++n) {
            if (B.nodes[n].left < 0) continue;
            open((int)n, kk);
            for (size_t k = 0; k < kk.size(); ++k) open4[n][k] = kk[k];
            nopen4[n] = (signed char)kk.size();
        }
    });
    // Node ids: the inner children of a node get consecutive ids when the node is expanded; nodes are
    // expanded breadth-first (kDepthFirstLayout false: the top levels every ray walks share lines) or
    // depth-first (a subtree's nodes sit together; measured 0.3-0.5 % slower on the hall and arena).
    std::vector<int> order4{root};            // binary id of each 4-wide inner node
    std::vector<int> depth4{0};               // their depths
    std::vector<std::array<int, 4>> kids4(1); // their children (binary ids), nkids4 of them
    std::vector<int> nkids4(1, 0);
    std::vector<int> id4(B.nodes.size(), -1);
    id4[root] = 0;
    std::vector<int> todo{0};
    size_t todo_head = 0;
    while (todo_head < todo.size()) {
        int q;
        if (kDepthFirstLayout) { q = todo.back(); todo.pop_back(); }
        else q = todo[todo_head++];
        const int bn = order4[q], nk = nopen4[bn];
        std::array<int, 4> a{-1, -1, -1, -1};
        const int first_new = (int)order4.size();
        for (int k = 0; k < nk; ++k) {
            const int kid = open4[bn][k];
            a[k] = kid;
            if (B.nodes[kid].left >= 0) {
                id4[kid] = (int)order4.size();
                order4.push_back(kid);
                depth4.push_back(depth4[q] + 1);
                kids4.emplace_back();
                nkids4.push_back(0);
            }
        }
        kids4[q] = a;
        nkids4[q] = nk;
        if (kDepthFirstLayout)
            for (int n = (int)order4.size() - 1; n >= first_new; --n) todo.push_back(n);  // first child next
        else
            for (int n = first_new; n < (int)order4.size(); ++n) todo.push_back(n);
    }
    // Leaf triangles in node order: the leaves that are children of one 4-wide node sit together, in
    // slot order, so a quantised node names them by one base index and per-slot counts.  (The empty
    // leaf of a wrapped leaf root holds no triangle.)
    std::vector<int> leaf_first(B.nodes.size(), 0);
    {
        std::vector<int> norder;
        norder.reserve((size_t)hs.ntri);
        for (size_t q = 0; q < order4.size(); ++q)
            for (int k = 0; k < nkids4[q]; ++k) {
                const int kid = kids4[q][k];
                const BNode &x = B.nodes[kid];
                if (x.left >= 0) continue;
                leaf_first[kid] = (int)norder.size();
                if (x.lo[0] > x.hi[0]) continue;
                for (int t = 0; t < x.count; ++t) norder.push_back(B.order[x.first + t]);
            }
        if (norder.size() == B.order.size()) {
            B.order.swap(norder);
        } else {  // not every triangle reached once: keep the builder's order (no quantised copy then)
            for (size_t n = 0; n < B.nodes.size(); ++n) leaf_first[n] = B.nodes[n].first;
        }
    }
    const int max_depth4 = *std::max_element(depth4.begin(), depth4.end());
    const double pad = 2e-6 * hs.scale;
    auto lo_f = [&](double v) { return v > 1e299 ? INFINITY : (float)(v - pad); };
    auto hi_f = [&](double v) { return v < -1e299 ? -INFINITY : (float)(v + pad); };
    hs.bvh.resize(order4.size() * kBvhNodeFloats);
    parallel_chunks(order4.size(), 16384, [&](size_t q0, size_t q1) {
        for (size_t q = q0; q < q1; ++q) {
            float *f = &hs.bvh[kBvhNodeFloats * q];
            const std::array<int, 4> &kq = kids4[q];
            for (int k = 0; k < 4; ++k) {
                int code;
                if (k < nkids4[q]) {
                    const BNode &x = B.nodes[kq[k]];
                    f[0 + k] = lo_f(x.lo[0]); f[4 + k] = hi_f(x.hi[0]);
                    f[8 + k] = lo_f(x.lo[1]); f[12 + k] = hi_f(x.hi[1]);
                    f[16 + k] = lo_f(x.lo[2]); f[20 + k] = hi_f(x.hi[2]);
                    code = x.left >= 0 ? id4[kq[k]] : ~(leaf_first[kq[k]] * 16 + (x.count - 1));
                } else {  // empty slot: flagged by its code (a slab test cannot reject an inverted box)
                    f[0 + k] = f[4 + k] = f[8 + k] = f[12 + k] = f[16 + k] = f[20 + k] = 0.f;
                    code = (int)0x80000000;
                }
                std::memcpy(&f[24 + k], &code, 4);
                f[28 + k] = 0.f;
            }
        }
    });
    B.max_depth = max_depth4 + 1;
    hs.bvh_nodes = (int)order4.size();
    hs.bvh_leaves = B.leaves;
    hs.bvh_depth = B.max_depth;
    // reorder triangles into leaf order
    hvec<double> t64(hs.tri64.size());
    hvec<int32_t> tp(hs.ntri), tl(hs.ntri);
    parallel_chunks((size_t)hs.ntri, 65536, [&](size_t i0, size_t i1) {
        for (size_t i = i0; i < i1; ++i) {
            const int s = B.order[i];
            std::copy(&hs.tri64[9 * (size_t)s], &hs.tri64[9 * (size_t)s] + 9, &t64[9 * i]);
            tp[i] = hs.tri_poly[s];
            tl[i] = hs.tri_plane[s];
        }
    });
    hs.tri64.swap(t64);
    hs.tri_poly.swap(tp);
    hs.tri_plane.swap(tl);
}

// 48-byte copy of the 4-wide BVH: per node a frame (origin of the children's union box and a
// power-of-two step s = 2^e per axis, 255 steps spanning it), each child's box as 8-bit steps, the
// lower bound rounded down and the upper rounded up, at least s / 256 outside the float box (the walk
// folds the byte decode's bias into the slab offset, one rounding of at most 2^-9 s, so a decoded box
// still contains the float box), and the children as one base index each for inner nodes and leaf
// triangles plus a 4-bit code per slot.  The stored exponent is that of 2^(e - 8) = s / 256, the scale
// of a byte decoded as 2^23 + 256 q.
//   float4 (origin x, y, z, bits: ex | ey << 8 | ez << 16 | slot codes 0-1 << 24)
//   uint4  (lo.x of children 0-3 as bytes, hi.x, lo.y, hi.y)
//   uint4  (lo.z, hi.z, first inner child's node id, first leaf triangle | slot codes 2-3 << 24)
// Slot code: 0 inner child (the node ids of a node's inner children are consecutive), 1-8 a leaf of
// that many triangles (a node's leaves' triangles are consecutive), 15 empty.  A scene whose triangle
// ids need more than 24 bits keeps no quantised copy.
static bool quantize_nodes(HostScene &hs, size_t q0, size_t q1);

void quantize_bvh(HostScene &hs) {
    const size_t nodes = hs.bvh.size() / kBvhNodeFloats;
    hs.bvhq.resize(nodes * kBvhQNodeFloats);  // every float of every node is written
    std::atomic<bool> ok{hs.ntri < (1 << 24)};
    // nodes are independent: large trees are quantised in chunks on several threads
    parallel_chunks(nodes, 8192, [&hs, &ok](size_t q0, size_t q1) {
        if (!quantize_nodes(hs, q0, q1)) ok = false;
    });
    if (!ok) hs.bvhq.clear();
}

// Quantised copy of nodes [q0, q1) (see quantize_bvh); false if a node's children do not fit the
// base-and-count form.
static bool quantize_nodes(HostScene &hs, size_t q0, size_t q1) {
    bool fits = true;
    for (size_t q = q0; q < q1; ++q) {
        const float *f = &hs.bvh[q * kBvhNodeFloats];
        int code[4];
        for (int k = 0; k < 4; ++k) std::memcpy(&code[k], &f[24 + k], 4);
        double lo[3] = {HUGE_VAL, HUGE_VAL, HUGE_VAL}, hi[3] = {-HUGE_VAL, -HUGE_VAL, -HUGE_VAL};
        bool valid[4];
        for (int k = 0; k < 4; ++k) {
            valid[k] = code[k] != (int)0x80000000;
            for (int a = 0; a < 3; ++a) valid[k] = valid[k] && std::isfinite(f[8 * a + k]) && std::isfinite(f[8 * a + 4 + k]);
            if (!valid[k]) continue;
            for (int a = 0; a < 3; ++a) {
                lo[a] = std::min(lo[a], (double)f[8 * a + k]);
                hi[a] = std::max(hi[a], (double)f[8 * a + 4 + k]);
            }
        }
        // children: base ids and slot codes
        uint32_t slots = 0;
        int nbase = -1, tbase = -1, ninner = 0, ntris = 0;
        for (int k = 0; k < 4; ++k) {
            uint32_t v = 15;
            if (valid[k] && code[k] >= 0) {
                if (nbase < 0) nbase = code[k];
                fits = fits && code[k] == nbase + ninner;
                ++ninner;
                v = 0;
            } else if (valid[k]) {
                const int c = ~code[k], first = c >> 4, cnt = (c & 15) + 1;
                if (tbase < 0) tbase = first;
                fits = fits && first == tbase + ntris && cnt <= 8;
                ntris += cnt;
                v = (uint32_t)cnt;
            }
            slots |= v << (4 * k);
        }
        if (nbase < 0) nbase = 0;
        if (tbase < 0) tbase = 0;
        fits = fits && tbase + ntris <= (1 << 24);
        float origin[3] = {0.f, 0.f, 0.f};
        int ebias[3] = {127, 127, 127};
        uint32_t qlo[3] = {0, 0, 0}, qhi[3] = {0, 0, 0};  // 4 children x 8 bits each
        for (int a = 0; a < 3; ++a) {
            if (lo[a] > hi[a]) continue;  // no valid child: the node is never entered
            const double ext = hi[a] - lo[a];
            int e = ext > 0 ? (int)std::ceil(std::log2(ext / 254.0)) : -100;
            e = std::max(-100, std::min(127, e));  // e - 8 stays a normal exponent
            float org = 0.f;
            for (;;) {  // the decoded boxes must contain every child box with s / 256 to spare
                const float s = std::ldexp(1.0f, e);
                org = (float)(lo[a] - s / 256.0);
                if ((double)org > lo[a] - s / 256.0) org = std::nextafter(org, -INFINITY);
                bool ok = std::isfinite(org);
                uint32_t L = 0, H = 0;
                for (int k = 0; k < 4 && ok; ++k) {
                    int ql = 255, qh = 0;  // invalid children: an inverted box (never tested: code check)
                    if (valid[k]) {
                        // decoded bounds org + q s are exact in double
                        const double wl = (double)f[8 * a + k] - s / 256.0, wh = (double)f[8 * a + 4 + k] + s / 256.0;
                        ql = (int)std::floor((wl - org) / s);
                        qh = (int)std::ceil((wh - org) / s);
                        ql = std::max(0, ql);
                        while (ql > 0 && (double)org + (double)ql * s > wl) --ql;
                        while (qh <= 255 && (double)org + (double)qh * s < wh) ++qh;
                        if (qh > 255 || (double)org + (double)ql * s > wl) ok = false;
                    }
                    L |= (uint32_t)ql << (8 * k);
                    H |= (uint32_t)std::min(qh, 255) << (8 * k);
                }
                if (ok || e >= 127) {
                    origin[a] = org;
                    qlo[a] = L;
                    qhi[a] = H;
                    ebias[a] = e - 8 + 127;
                    break;
                }
                ++e;
            }
        }
        float *g = &hs.bvhq[q * kBvhQNodeFloats];
        g[0] = origin[0];
        g[1] = origin[1];
        g[2] = origin[2];
        const uint32_t ex = (uint32_t)ebias[0] | ((uint32_t)ebias[1] << 8) | ((uint32_t)ebias[2] << 16) |
                            ((slots & 255u) << 24);
        std::memcpy(&g[3], &ex, 4);
        const uint32_t words[8] = {qlo[0], qhi[0], qlo[1], qhi[1], qlo[2], qhi[2], (uint32_t)nbase,
                                   ((uint32_t)tbase & 0xFFFFFFu) | ((slots >> 8) << 24)};
        std::memcpy(&g[4], words, sizeof(words));
    }
    return fits;
}

}  // namespace

// Calculate_Attenuation (Classes_Medium_Props.cs:51-191) as coded, over a frequency table: the eight
// octave centres, or the reference's third-octave table (23 entries: it skips 2500 Hz).  Includes the
// C# integer divisions in the exponents (-1/2 -> 0, -1/3 -> 0, -5/2 -> -2, 1/2 -> 0); the Evans-Bazley
// and table branches fill the first eight entries only, whatever the table.  Called by the
// Uniform_Medium ctor with Pa/10 (hPa -> kPa).
static void attenuation_table(const double *F, int nf, double temp_c, double hr, double pa_hpa, int air_choice,
                              int edge, double *atten) {
    const double Tk = temp_c + 273.15, Pa = pa_hpa / 10.0;
    for (int o = 0; o < nf; ++o) atten[o] = 0.0;
    if (air_choice == 0) {
        const double h = hr * std::pow(10.0, -6.8346 * std::pow(273.16 / Tk, 1.261) + 4.6151) / (Pa / 101.325);
        const int e_half = -1 / 2, e_third = -1 / 3, e_fivehalf = -5 / 2, e_pos_half = 1 / 2;
        for (int o = 0; o < nf; ++o) {
            double frO = (Pa / 101.325) * (24 + 4.04e4 * h * ((0.02 + h) / (0.391 + h)));
            double frN = (Pa / 101.325) * std::pow(Tk / 293.15, (double)e_half) *
                         (9 + 280 * h * std::exp(-4.170 * (std::pow(Tk / 293.15, (double)e_third) - 1)));
            double z = 0.1068 * std::exp(-3352 / Tk) / (frN + F[o] * F[o] / frN);
            double y = std::pow(Tk / 293.15, (double)e_fivehalf) *
                       (0.01275 * std::exp(-2239.1 / Tk) / (frO + F[o] * F[o] / frO) + z);
            atten[o] = 8.686 * F[o] * F[o] * ((1.84e-11 / (Pa / 101.325) * std::pow(Tk / 293.15, (double)e_pos_half)) + y);
        }
    } else if (air_choice == 1) {
        for (int o = 0; o < kBands && o < nf; ++o) {
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
            for (int o = 0; o < kBands && o < nf; ++o) atten[o] = tab[row][o];
        if (edge)
            for (int o = 0; o < kBands && o < nf; ++o) atten[o] /= std::sqrt(2.0);
    }
}

const double kThirdOctaveCentres[kThirdOctaveBands] = {50,   62.5, 80,   100,  125,  160,  200,  250,
                                                      315,  400,  500,  630,  800,  1000, 1250, 1600,
                                                      2000, 3150, 4000, 5000, 6300, 8000, 10000};

void medium_attenuation_third_octave(double temp_c, double hr, double pa_hpa, int air_choice, int edge,
                                     double atten[kThirdOctaveBands]) {
    attenuation_table(kThirdOctaveCentres, kThirdOctaveBands, temp_c, hr, pa_hpa, air_choice, edge, atten);
}

// The octave bands, with sound speed and density (Calculate_Density(Tk, Pa*100, hr)).
void medium_properties(double temp_c, double hr, double pa_hpa, int air_choice, int edge, double atten[kBands],
                       double *c, double *rho) {
    static const double F[kBands] = {62.5, 125, 250, 500, 1000, 2000, 4000, 8000};
    attenuation_table(F, kBands, temp_c, hr, pa_hpa, air_choice, edge, atten);
    const double Tk = temp_c + 273.15;
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

// The same 80 faces into a caller-owned array (no heap use).
void geodesic_faces_fixed(double out[kGeoFaces * 9]) {
    const double s5 = std::sqrt(5.0), phi = (1.0 + s5) * 0.5;
    const double ratio = std::sqrt(10.0 + 2.0 * s5) / (4.0 * phi);
    const double a = (.25 / ratio) * 0.5, b = (.25 / ratio) / (2.0 * phi);
    D3 P[12] = {{0, b, -a}, {b, a, 0}, {-b, a, 0}, {0, b, a}, {0, -b, a}, {-a, 0, b},
                {0, -b, -a}, {a, 0, -b}, {a, 0, b}, {-a, 0, -b}, {b, -a, 0}, {-b, -a, 0}};
    for (auto &p : P) p = unit(p);
    static const int T[20][3] = {{0, 1, 2}, {3, 2, 1}, {3, 4, 5}, {3, 8, 4}, {0, 6, 7}, {0, 9, 6}, {4, 10, 11},
                                 {6, 11, 10}, {2, 5, 9}, {11, 9, 5}, {1, 7, 8}, {10, 8, 7}, {3, 5, 2}, {3, 1, 8},
                                 {0, 2, 9}, {0, 7, 1}, {6, 9, 11}, {6, 10, 7}, {4, 11, 5}, {4, 8, 10}};
    int n = 0;
    auto put = [&](D3 x, D3 y, D3 z) {
        for (D3 v : {x, y, z}) { out[n++] = v.x; out[n++] = v.y; out[n++] = v.z; }
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

bool bvh_shoot_host(const HostScene &hs, const double o[3], const double d[3], double t_min, int &tri, double &t) {
    auto safe = [](double x) { return std::fabs(x) < 1e-20 ? std::copysign(1e-20, x) : x; };
    const float ix = (float)(1.0 / safe(d[0])), iy = (float)(1.0 / safe(d[1])), iz = (float)(1.0 / safe(d[2]));
    const float ox = (float)o[0] * ix, oy = (float)o[1] * iy, oz = (float)o[2] * iz;
    std::vector<int> stack;
    int node = 0;
    double best = 1e300;
    float bestf = 3.4e38f;
    int bi = -1;
    for (;;) {
        bool done = false;
        while (node >= 0) {
            // one 4-wide node, as the device walks it (bvh4_step)
            const float *f = &hs.bvh[kBvhNodeFloats * (size_t)node];
            float tk[4];
            int id[4];
            for (int k = 0; k < 4; ++k) {
                std::memcpy(&id[k], &f[24 + k], 4);
                auto slab = [&](float a, float b, float inv, float oi, float &lo, float &hi) {
                    const float t0 = std::fma(a, inv, -oi), t1 = std::fma(b, inv, -oi);
                    lo = std::min(t0, t1);
                    hi = std::max(t0, t1);
                };
                float x0, x1, y0, y1, z0, z1;
                slab(f[0 + k], f[4 + k], ix, ox, x0, x1);
                slab(f[8 + k], f[12 + k], iy, oy, y0, y1);
                slab(f[16 + k], f[20 + k], iz, oz, z0, z1);
                const float tn = std::max(std::max(x0, y0), std::max(z0, 0.f));
                const float tf = std::min(std::min(x1, y1), std::min(z1, bestf));
                tk[k] = (tn <= tf && id[k] != (int)0x80000000) ? tn : 3.4028235e38f;
            }
            auto cs = [&](int a, int b) {
                if (tk[b] < tk[a]) { std::swap(tk[a], tk[b]); std::swap(id[a], id[b]); }
            };
            cs(0, 1); cs(2, 3); cs(0, 2); cs(1, 3); cs(1, 2);
            if (tk[0] == 3.4028235e38f) {
                if (stack.empty()) { done = true; break; }
                node = stack.back();
                stack.pop_back();
                continue;
            }
            for (int k = 3; k >= 1; --k)
                if (tk[k] != 3.4028235e38f) stack.push_back(id[k]);
            node = id[0];
        }
        if (done) break;
        const int code = ~node, f0 = code >> 4, cnt = (code & 15) + 1;
        for (int k = 0; k < cnt; ++k) {
            const double *q = &hs.tri64[9 * (size_t)(f0 + k)];
            const D3 e1{q[3], q[4], q[5]}, e2{q[6], q[7], q[8]}, dd{d[0], d[1], d[2]};
            const D3 p = cross(dd, e2);
            const double det = dot(e1, p);
            if (det == 0) continue;
            const double inv = 1.0 / det;
            const D3 s{o[0] - q[0], o[1] - q[1], o[2] - q[2]};
            const double u = dot(s, p) * inv;
            if (u < 0 || u > 1) continue;
            const D3 qq = cross(s, e1);
            const double v = dot(dd, qq) * inv;
            if (v < 0 || u + v > 1) continue;
            const double tt = dot(e2, qq) * inv;
            if (tt > t_min && tt < best) { best = tt; bestf = (float)tt * 1.0000002f; bi = f0 + k; }
        }
        if (stack.empty()) break;
        node = stack.back();
        stack.pop_back();
    }
    if (bi < 0) return false;
    tri = bi;
    t = best;
    return true;
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
    hs.alpha.resize(8 * (size_t)hs.npoly);
    hs.scat.resize(8 * (size_t)hs.npoly);
    hs.trans.resize(8 * (size_t)hs.npoly);
    hs.normal.resize(3 * (size_t)hs.npoly);
    hs.area.resize(hs.npoly);

    // Polygons in parallel chunks: coefficient ranges, vertex indices, Newell normal and area, and the
    // count of non-degenerate fan pieces.  A coefficient out of range is reported first, else the first
    // failing polygon in polygon order names the error.
    constexpr size_t kPolyGrain = 16384;
    const size_t nchunk = ((size_t)hs.npoly + kPolyGrain - 1) / kPolyGrain;
    struct PolyChunk {
        bool bad_coef = false;
        int bad = -1;
        std::string msg;
        bool trans = false;
        double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    };
    std::vector<PolyChunk> pc(nchunk);
    std::vector<int> fan(hs.npoly + 1, 0);
    parallel_chunks((size_t)hs.npoly, kPolyGrain, [&](size_t p0, size_t p1) {
        PolyChunk &c = pc[p0 / kPolyGrain];
        std::copy(d->absorption + 8 * p0, d->absorption + 8 * p1, hs.alpha.begin() + 8 * p0);
        std::copy(d->scattering + 8 * p0, d->scattering + 8 * p1, hs.scat.begin() + 8 * p0);
        if (d->transmission) std::copy(d->transmission + 8 * p0, d->transmission + 8 * p1, hs.trans.begin() + 8 * p0);
        else std::fill(hs.trans.begin() + 8 * p0, hs.trans.begin() + 8 * p1, 0.0);
        for (size_t i = 8 * p0; i < 8 * p1; ++i) {
            if (!(hs.alpha[i] >= 0 && hs.alpha[i] <= 1) || !(hs.scat[i] >= 0 && hs.scat[i] <= 1) ||
                !(hs.trans[i] >= 0 && hs.trans[i] <= 1)) {
                c.bad_coef = true;
                break;
            }
            if (hs.trans[i] > 0) c.trans = true;
        }
        for (int p = (int)p0; p < (int)p1; ++p) {
            int b = d->poly_offsets[p], e = d->poly_offsets[p + 1];
            if (e - b < 3 || b < 0) {
                c.bad = p;
                c.msg = "scene: polygon " + std::to_string(p) + " has fewer than 3 vertices";
                return;
            }
            for (int k = b; k < e; ++k)
                if (d->poly_indices[k] < 0 || d->poly_indices[k] >= nv) {
                    c.bad = p;
                    c.msg = "scene: vertex index out of range";
                    return;
                }
            D3 n{0, 0, 0};
            for (int k = b; k < e; ++k) {  // Newell
                D3 p0v = V(d->poly_indices[k]), p1v = V(d->poly_indices[k + 1 < e ? k + 1 : b]);
                n.x += (p0v.y - p1v.y) * (p0v.z + p1v.z);
                n.y += (p0v.z - p1v.z) * (p0v.x + p1v.x);
                n.z += (p0v.x - p1v.x) * (p0v.y + p1v.y);
            }
            hs.area[p] = 0.5 * std::sqrt(dot(n, n));
            if (!(hs.area[p] > 0)) {
                c.bad = p;
                c.msg = "scene: degenerate polygon " + std::to_string(p);
                return;
            }
            D3 u = unit(n);
            hs.normal[3 * p] = u.x; hs.normal[3 * p + 1] = u.y; hs.normal[3 * p + 2] = u.z;
            D3 a = V(d->poly_indices[b]);
            int cnt = 0;
            for (int k = b + 1; k + 1 < e; ++k) {
                D3 e1 = sub(V(d->poly_indices[k]), a), e2 = sub(V(d->poly_indices[k + 1]), a);
                if (dot(cross(e1, e2), cross(e1, e2)) != 0) ++cnt;  // zero-area fan pieces are dropped
            }
            fan[p + 1] = cnt;
            for (int k = b; k < e; ++k) {
                D3 q = V(d->poly_indices[k]);
                c.lo[0] = std::min(c.lo[0], q.x); c.lo[1] = std::min(c.lo[1], q.y); c.lo[2] = std::min(c.lo[2], q.z);
                c.hi[0] = std::max(c.hi[0], q.x); c.hi[1] = std::max(c.hi[1], q.y); c.hi[2] = std::max(c.hi[2], q.z);
            }
        }
    });
    for (const PolyChunk &c : pc)
        if (c.bad_coef) {
            err = "scene: absorption, scattering and transmission must lie in [0, 1]";
            return false;
        }
    for (int k = 0; k < 3; ++k) { hs.bmin[k] = 1e300; hs.bmax[k] = -1e300; }
    for (const PolyChunk &c : pc) {
        if (c.bad >= 0) { err = c.msg; return false; }
        hs.has_trans = hs.has_trans || c.trans;
        for (int k = 0; k < 3; ++k) { hs.bmin[k] = std::min(hs.bmin[k], c.lo[k]); hs.bmax[k] = std::max(hs.bmax[k], c.hi[k]); }
    }
    for (int p = 0; p < hs.npoly; ++p) fan[p + 1] += fan[p];
    hs.ntri = fan[hs.npoly];
    if (hs.ntri == 0) { err = "scene: no triangles"; return false; }
    hs.tri64.resize(9 * (size_t)hs.ntri);
    hs.tri_poly.resize(hs.ntri);
    parallel_chunks((size_t)hs.npoly, kPolyGrain, [&](size_t p0, size_t p1) {
        for (int p = (int)p0; p < (int)p1; ++p) {
            const int b = d->poly_offsets[p], e = d->poly_offsets[p + 1];
            int t = fan[p];
            D3 a = V(d->poly_indices[b]);
            for (int k = b + 1; k + 1 < e; ++k) {
                D3 e1 = sub(V(d->poly_indices[k]), a), e2 = sub(V(d->poly_indices[k + 1]), a);
                if (dot(cross(e1, e2), cross(e1, e2)) == 0) continue;
                double *t9 = &hs.tri64[9 * (size_t)t];
                t9[0] = a.x; t9[1] = a.y; t9[2] = a.z;
                t9[3] = e1.x; t9[4] = e1.y; t9[5] = e1.z;
                t9[6] = e2.x; t9[7] = e2.y; t9[8] = e2.z;
                hs.tri_poly[t++] = p;
            }
        }
    });
    double ext[3];
    for (int k = 0; k < 3; ++k) ext[k] = hs.bmax[k] - hs.bmin[k];
    hs.scale = std::max({ext[0], ext[1], ext[2], 1e-3});
    const double pad = 1e-5 * hs.scale;
    for (int k = 0; k < 3; ++k) { hs.bmin[k] -= pad; hs.bmax[k] += pad; ext[k] = hs.bmax[k] - hs.bmin[k]; }

    // Coplanar groups: quantised (canonical normal, offset) of each triangle's own plane; ids in order
    // of first appearance.  Keys are computed in parallel; large scenes are grouped in shards (by the
    // top bits of the key's hash, one open-addressing table per shard), each triangle pointing at the
    // first triangle of its group, and the ids are then numbered in triangle order.
    struct PlaneKey {
        long long v[4];
        bool operator==(const PlaneKey &o) const { return v[0] == o.v[0] && v[1] == o.v[1] && v[2] == o.v[2] && v[3] == o.v[3]; }
    };
    auto hash = [](const PlaneKey &k) {
        uint64_t h = 0x9E3779B97F4A7C15ull;
        for (long long x : k.v) h = (h ^ (uint64_t)x) * 0xBF58476D1CE4E5B9ull + (h >> 29);
        return h ^ (h >> 31);
    };
    std::vector<PlaneKey> keys((size_t)hs.ntri);
    std::vector<uint64_t> khash((size_t)hs.ntri);
    parallel_chunks((size_t)hs.ntri, 65536, [&](size_t i0, size_t i1) {
        for (size_t i = i0; i < i1; ++i) {
            const double *t = &hs.tri64[9 * i];
            D3 n = unit(cross(D3{t[3], t[4], t[5]}, D3{t[6], t[7], t[8]}));
            if (n.x < 0 || (n.x == 0 && (n.y < 0 || (n.y == 0 && n.z < 0)))) n = mul(n, -1);
            double off = dot(n, D3{t[0], t[1], t[2]}) / hs.scale;
            keys[i] = PlaneKey{{std::llround(n.x * 1e6), std::llround(n.y * 1e6), std::llround(n.z * 1e6),
                                std::llround(off * 1e6)}};
            khash[i] = hash(keys[i]);
        }
    });
    const int shards = hs.ntri >= 65536 ? 16 : 1;
    std::vector<int> first((size_t)hs.ntri);
    parallel_chunks((size_t)shards, 1, [&](size_t s0, size_t s1) {
        for (size_t s = s0; s < s1; ++s) {
            auto mine = [&](size_t i) { return shards == 1 || (khash[i] >> 60) == s; };
            size_t count = 0;
            for (size_t i = 0; i < (size_t)hs.ntri; ++i) count += mine(i);
            size_t cap = 16;
            while (cap < 2 * count) cap <<= 1;
            std::vector<int> slot(cap, -1);  // first triangle of the slot's group
            for (size_t i = 0; i < (size_t)hs.ntri; ++i) {
                if (!mine(i)) continue;
                size_t h = (size_t)khash[i] & (cap - 1);
                while (slot[h] >= 0 && !(keys[(size_t)slot[h]] == keys[i])) h = (h + 1) & (cap - 1);
                if (slot[h] < 0) slot[h] = (int)i;
                first[i] = slot[h];
            }
        }
    });
    hs.tri_plane.resize(hs.ntri);
    int n_planes = 0;
    for (int i = 0; i < hs.ntri; ++i) hs.tri_plane[i] = first[i] == i ? n_planes++ : hs.tri_plane[first[i]];

    build_bvh(hs, d->bvh_leaf_max);
    quantize_bvh(hs);

    medium_properties(d->temp_c, d->rel_humidity, d->pressure_hpa, d->air_choice, d->edge_correction, hs.atten,
                      &hs.c, &hs.rho);
    hs.rho_c = hs.rho * hs.c;
    if (!(hs.c > 0)) { err = "scene: non-positive sound speed"; return false; }
    return true;
}

}  // namespace pach
