// venu_oracle.cpp -- CPU oracle for the Venusaur-GB300 path tracer.
//
// TEST INFRASTRUCTURE ONLY (see venu_oracle.h).  Compiled with
// -ffp-contract=off so every float operation rounds exactly once, as written;
// fmaf() appears only where the GB300 kernels use an explicit fused
// multiply-add.  The product library never links or calls this file.
//
// Reference citations are relative to the reference project root.

#include "venu_oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <random>
#include <thread>
#include <vector>

namespace {

// ---------------------------------------------------------------------------
// float3 with the reference's vec_math.h semantics (Core/vec_math.h:479-569):
// plain IEEE single-precision operations, left-to-right.
// ---------------------------------------------------------------------------
struct f3 {
    float x, y, z;
};
inline f3 mk(float x, float y, float z) { return f3{x, y, z}; }
inline f3 operator+(f3 a, f3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
inline f3 operator-(f3 a, f3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
inline f3 operator-(f3 a) { return mk(-a.x, -a.y, -a.z); }
inline f3 operator*(f3 a, f3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
inline f3 operator*(f3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
inline f3 operator*(float s, f3 a) { return mk(a.x * s, a.y * s, a.z * s); }
// Core/vec_math.h:483-487: division by a scalar multiplies by its reciprocal.
inline f3 divs(f3 a, float s) {
    float inv = 1.0f / s;
    return a * inv;
}
inline float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }  // :527-530
inline f3 normalize(f3 v) {                                                 // :544-549
    float inv = 1.0f / std::sqrt(dot(v, v));
    return v * inv;
}
inline f3 reflect(f3 i, f3 n) { return i - (2.0f * n) * dot(n, i); }  // :557-561
inline f3 refract(f3 uv, f3 n, float eta) {                           // :563-569
    float cos_theta = std::fmin(dot(-uv, n), 1.0f);
    f3 r_perp = eta * (uv + cos_theta * n);
    f3 r_par = (-std::sqrt(std::fabs(1.0f - dot(r_perp, r_perp)))) * n;
    return r_perp + r_par;
}
inline f3 lerp3(f3 a, f3 b, float t) { return a + t * (b - a); }  // :499-503
inline float clampf(float f, float a, float b) { return std::fmax(a, std::fmin(f, b)); }

// ---------------------------------------------------------------------------
// RNG: Core/random.cuh:31-67 restated.
// ---------------------------------------------------------------------------
inline uint32_t tea4(uint32_t val0, uint32_t val1) {  // random.cuh:31-46, N = 4
    uint32_t v0 = val0, v1 = val1, s0 = 0;
    for (int n = 0; n < 4; ++n) {
        s0 += 0x9e3779b9u;
        v0 += ((v1 << 4) + 0xa341316cu) ^ (v1 + s0) ^ ((v1 >> 5) + 0xc8013ea4u);
        v1 += ((v0 << 4) + 0xad90777du) ^ (v0 + s0) ^ ((v0 >> 5) + 0x7e95761eu);
    }
    return v0;
}
inline float rnd(uint32_t& prev) {  // random.cuh:49-55 (lcg) and :64-67 (rnd)
    prev = 1664525u * prev + 1013904223u;
    return (float)(prev & 0x00FFFFFFu) / (float)0x01000000;
}
// Core/RayTracer.cu:93-97 (random_float with range), left-to-right draws.
inline float rnd_range(uint32_t& s, float lo, float hi) { return lo + (hi - lo) * rnd(s); }
// Core/RayTracer.cu:117-125: rejection sampling, x then y then z per try.
// Capped at 4096 candidates like the CUDA kernels (an unreachable bound at
// a 52% / 79% acceptance rate that only guarantees termination).
const int kMaxTries = 4096;
inline f3 random_in_unit_sphere(uint32_t& s) {
    f3 p{0, 0, 0};
    for (int i = 0; i < kMaxTries; ++i) {
        float x = rnd_range(s, -1.0f, 1.0f);
        float y = rnd_range(s, -1.0f, 1.0f);
        float z = rnd_range(s, -1.0f, 1.0f);
        p = mk(x, y, z);
        if (!(dot(p, p) >= 1.0f)) break;
    }
    return p;
}
// Core/RayTracer.cu:141-149
inline f3 random_in_unit_disk(uint32_t& s) {
    f3 p{0, 0, 0};
    for (int i = 0; i < kMaxTries; ++i) {
        float x = rnd_range(s, -1.0f, 1.0f);
        float y = rnd_range(s, -1.0f, 1.0f);
        p = mk(x, y, 0.0f);
        if (!(dot(p, p) >= 1.0f)) break;
    }
    return p;
}
// Core/RayTracer.cu:8-13: |e_i| < 1e-8 (a double constant) for all i.  For a
// float x, (double)x < 1e-8 holds exactly when x <= 1e-8f.
inline bool near_zero(f3 e) {
    return std::fabs(e.x) <= 1e-8f && std::fabs(e.y) <= 1e-8f && std::fabs(e.z) <= 1e-8f;
}

// ---------------------------------------------------------------------------
// Deterministic exp/log in double from +,-,*,/ only (no libm), so a scene
// generated on one machine is bit-identical on another.
// ---------------------------------------------------------------------------
const double kLn2Hi = 6.93147180369123816490e-01;
const double kLn2Lo = 1.90821492927058770002e-10;
double det_exp(double x) {
    double kf = std::floor(x * 1.44269504088896338700 + 0.5);
    double r = (x - kf * kLn2Hi) - kf * kLn2Lo;
    double term = 1.0, sum = 1.0;
    for (int i = 1; i < 24; ++i) {
        term = term * r / (double)i;
        sum = sum + term;
    }
    int k = (int)kf;
    return std::ldexp(sum, k);
}
double det_log(double x) {
    int e = 0;
    double m = std::frexp(x, &e);  // x = m * 2^e, m in [0.5, 1)
    if (m < 0.70710678118654752440) {
        m = m * 2.0;
        e -= 1;
    }
    double s = (m - 1.0) / (m + 1.0);
    double s2 = s * s, term = s, sum = 0.0;
    for (int i = 1; i < 60; i += 2) {
        sum = sum + term / (double)i;
        term = term * s2;
    }
    return 2.0 * sum + (double)e * kLn2Hi + (double)e * kLn2Lo;
}

// Scene RNG: std::mt19937 (fully specified by the C++ standard) with a
// documented canonical float u = (x >> 8) * 2^-24.
struct SceneRng {
    std::mt19937 g;
    explicit SceneRng(uint32_t seed) : g(seed) {}
    float U() { return (float)(g() >> 8) * (1.0f / 16777216.0f); }
};

vo_sphere make_sphere(f3 c, float r, uint32_t mat, f3 albedo, float fuzz, float ir) {
    vo_sphere s;
    std::memset(&s, 0, sizeof(s));
    s.center[0] = c.x;
    s.center[1] = c.y;
    s.center[2] = c.z;
    s.radius = r;
    s.albedo[0] = albedo.x;
    s.albedo[1] = albedo.y;
    s.albedo[2] = albedo.z;
    s.fuzz = fuzz;
    s.ir = ir;
    s.material = mat;
    return s;
}

// Material draws shared by both generators (Core/Scene.h:28-64).
vo_sphere draw_material(SceneRng& R, float choose, f3 center, float radius) {
    if ((double)choose < 0.8) {
        float a0 = R.U(), a1 = R.U(), a2 = R.U();
        float b0 = R.U(), b1 = R.U(), b2 = R.U();
        return make_sphere(center, radius, 0, mk(a0 * b0, a1 * b1, a2 * b2), 0.0f, 0.0f);
    } else if ((double)choose < 0.95) {
        float a0 = 0.5f + (1.0f - 0.5f) * R.U();
        float a1 = 0.5f + (1.0f - 0.5f) * R.U();
        float a2 = 0.5f + (1.0f - 0.5f) * R.U();
        float fz = 0.0f + (0.5f - 0.0f) * R.U();
        return make_sphere(center, radius, 1, mk(a0, a1, a2), fz, 0.0f);
    }
    return make_sphere(center, radius, 2, mk(0, 0, 0), 0.0f, 1.5f);
}

// ---------------------------------------------------------------------------
// LBVH (Karras 2012) host build.
// ---------------------------------------------------------------------------
const int32_t kLeaf = (int32_t)0x80000000u;
const int32_t kHoisted = 0x40000000;  // leaf tested before traversal
const int32_t kSlotMask = 0x3fffffff;
const int kMaxHoisted = 4;
const uint32_t kHoistCandidates = 64;

uint32_t spread10(uint32_t v) {  // bit i of v -> bit 3i
    uint32_t r = 0;
    for (int i = 0; i < 10; ++i) r |= ((v >> i) & 1u) << (3 * i);
    return r;
}
uint32_t quant10(float c, float lo, float ext) {
    if (!(ext > 0.0f)) return 0;
    float t = (c - lo) / ext;
    float f = t * 1024.0f;
    f = std::fmin(std::fmax(f, 0.0f), 1023.0f);
    return (uint32_t)f;
}
inline void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    float bp = s - a;
    float ap = s - bp;
    e = (a - ap) + (b - bp);
}
// Round-down of (c - r) and round-up of (c + r), exact via the TwoSum error.
float sub_rd(float c, float r) {
    float s, e;
    two_sum(c, -r, s, e);
    return e < 0.0f ? std::nextafter(s, -INFINITY) : s;
}
float add_ru(float c, float r) {
    float s, e;
    two_sum(c, r, s, e);
    return e > 0.0f ? std::nextafter(s, INFINITY) : s;
}

struct Bvh {
    uint32_t n = 0;
    std::vector<uint32_t> keys;  // sorted Morton codes
    std::vector<uint32_t> ids;   // sorted slot -> original sphere index
    std::vector<vo_node> nodes;  // n-1 internal nodes, root = 0
    std::vector<f3> center;      // sorted slot data
    std::vector<float> radius;
    float bounds[6] = {0, 0, 0, 0, 0, 0};
    uint32_t depth = 0;
    std::vector<int32_t> hoist;  // slots of huge spheres tested first
};

int delta(const std::vector<uint32_t>& k, int n, int i, int j) {
    if (j < 0 || j > n - 1) return -1;
    uint32_t a = k[i], b = k[j];
    if (a == b) return 32 + __builtin_clz((uint32_t)i ^ (uint32_t)j);
    return __builtin_clz(a ^ b);
}

// Refit: post-order DFS from the root; a node's box is the union of its
// children's (leaf boxes from the slot's sphere, rounded outward).  Leaf words
// may carry the hoisted flag.  Also records the tree depth.
void refit_bvh(Bvh& B) {
    const int N = (int)B.n;
    if (N < 2) return;
    struct Item { int node; int state; };
    std::vector<Item> st;
    st.push_back({0, 0});
    uint32_t maxdepth = 0;
    std::vector<uint32_t> dep(N - 1, 0);
    dep[0] = 1;
    auto child_box = [&](int c, float* blo, float* bhi) {
        if (c & kLeaf) {
            int k = c & kSlotMask;
            float r = std::fabs(B.radius[k]);
            blo[0] = sub_rd(B.center[k].x, r);
            blo[1] = sub_rd(B.center[k].y, r);
            blo[2] = sub_rd(B.center[k].z, r);
            bhi[0] = add_ru(B.center[k].x, r);
            bhi[1] = add_ru(B.center[k].y, r);
            bhi[2] = add_ru(B.center[k].z, r);
        } else {
            for (int a = 0; a < 3; ++a) {
                blo[a] = B.nodes[c].lo[a];
                bhi[a] = B.nodes[c].hi[a];
            }
        }
    };
    while (!st.empty()) {
        Item it = st.back();
        st.pop_back();
        vo_node& nd = B.nodes[it.node];
        if (it.state == 0) {
            st.push_back({it.node, 1});
            for (int c : {nd.left, nd.right}) {
                if (!(c & kLeaf)) {
                    dep[c] = dep[it.node] + 1;
                    st.push_back({c, 0});
                } else {
                    maxdepth = std::max(maxdepth, dep[it.node] + 1);
                }
            }
        } else {
            float l0[3], h0[3], l1[3], h1[3];
            child_box(nd.left, l0, h0);
            child_box(nd.right, l1, h1);
            for (int a = 0; a < 3; ++a) {
                nd.lo[a] = std::fmin(l0[a], l1[a]);
                nd.hi[a] = std::fmax(h0[a], h1[a]);
            }
        }
    }
    B.depth = maxdepth;
}

// Treelet restructuring: one bottom-up pass over the Karras tree after the
// refit (Karras & Aila, "Fast Parallel Construction of High-Quality Bounding
// Volume Hierarchies", HPG 2013).  At every internal node N (children before
// parents) a treelet of up to 7 leaves is grown from N's two children by
// repeatedly opening the internal treelet leaf with the largest surface area
// (first such on ties); a dynamic program over all subsets of the treelet
// leaves finds the binary topology with the least total internal surface
// area, and the treelet is rewired that way when that is strictly less than
// its current total.  The leaves keep their Morton slots; N stays the
// treelet root; its internal nodes are reused in the order they were opened,
// handed out in depth-first order of the new topology.  Mirrors
// k_treelets in lbvh.cu operation for operation.
struct TBox {
    float lo[3], hi[3];
};
float tbox_area(const TBox& b) {
    const float dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
    return 2.0f * ((dx * dy + dy * dz) + dz * dx);
}
TBox tbox_of(const Bvh& B, int32_t c) {
    TBox b;
    if (c & kLeaf) {
        const int k = c & kSlotMask;
        const float r = std::fabs(B.radius[k]);
        const float cc[3] = {B.center[k].x, B.center[k].y, B.center[k].z};
        for (int a = 0; a < 3; ++a) {
            b.lo[a] = sub_rd(cc[a], r);
            b.hi[a] = add_ru(cc[a], r);
        }
    } else {
        for (int a = 0; a < 3; ++a) {
            b.lo[a] = B.nodes[c].lo[a];
            b.hi[a] = B.nodes[c].hi[a];
        }
    }
    return b;
}

void restructure_treelet(Bvh& B, int32_t N, std::vector<int32_t>& parent_internal,
                         std::vector<int32_t>& parent_leaf) {
    constexpr int kMaxTreeletLeaves = 7;
    int32_t L[kMaxTreeletLeaves];
    int32_t internals[kMaxTreeletLeaves - 1];
    int nl = 0, ni = 0;
    L[nl++] = B.nodes[N].left;
    L[nl++] = B.nodes[N].right;
    internals[ni++] = N;
    while (nl < kMaxTreeletLeaves) {
        int pick = -1;
        float pa = -1.0f;
        for (int i = 0; i < nl; ++i)
            if (!(L[i] & kLeaf)) {
                const float a = tbox_area(tbox_of(B, L[i]));
                if (a > pa) {
                    pa = a;
                    pick = i;
                }
            }
        if (pick < 0) break;
        const int32_t c = L[pick];
        internals[ni++] = c;
        L[pick] = B.nodes[c].left;
        L[nl++] = B.nodes[c].right;
    }
    if (nl < 3) return;
    const int full = (1 << nl) - 1;
    TBox bx[kMaxTreeletLeaves];
    for (int i = 0; i < nl; ++i) bx[i] = tbox_of(B, L[i]);
    float area[1 << kMaxTreeletLeaves], cost[1 << kMaxTreeletLeaves];
    uint8_t split[1 << kMaxTreeletLeaves];
    for (int S = 1; S <= full; ++S) {
        TBox u;
        for (int a = 0; a < 3; ++a) {
            u.lo[a] = INFINITY;
            u.hi[a] = -INFINITY;
        }
        for (int i = 0; i < nl; ++i)
            if (S >> i & 1)
                for (int a = 0; a < 3; ++a) {
                    u.lo[a] = std::fmin(u.lo[a], bx[i].lo[a]);
                    u.hi[a] = std::fmax(u.hi[a], bx[i].hi[a]);
                }
        area[S] = tbox_area(u);
    }
    for (int S = 1; S <= full; ++S) {
        split[S] = 0;
        if ((S & (S - 1)) == 0) {
            cost[S] = 0.0f;
            continue;
        }
        const int low = S & -S, rest = S ^ low;
        float bc = INFINITY;
        int bp = 0;
        // P = low | Q over the subsets Q of rest except rest itself,
        // enumerated from the largest down
        for (int Q = (rest - 1) & rest;; Q = (Q - 1) & rest) {
            const int P = Q | low;
            const float c = cost[P] + cost[S ^ P];
            if (c < bc) {
                bc = c;
                bp = P;
            }
            if (Q == 0) break;
        }
        cost[S] = area[S] + bc;
        split[S] = (uint8_t)bp;
    }
    float current = 0.0f;
    for (int i = 0; i < ni; ++i) current = current + tbox_area(tbox_of(B, internals[i]));
    if (!(cost[full] < current)) return;
    // Rewire.  The treelet's internal nodes are handed out in depth-first
    // preorder of the chosen splits (left part first); children are wired in
    // that order and boxes computed in the reverse order (children first).
    int order[kMaxTreeletLeaves - 1];
    int32_t node_of[1 << kMaxTreeletLeaves];
    int no = 0;
    {
        int stack[kMaxTreeletLeaves];
        int sp = 0;
        stack[sp++] = full;
        while (sp > 0) {
            const int S = stack[--sp];
            if ((S & (S - 1)) == 0) continue;
            node_of[S] = internals[no];
            order[no++] = S;
            stack[sp++] = S ^ split[S];
            stack[sp++] = split[S];
        }
    }
    auto word = [&](int T) { return (T & (T - 1)) == 0 ? L[__builtin_ctz(T)] : node_of[T]; };
    for (int i = 0; i < no; ++i) {
        const int S = order[i];
        const int32_t me = node_of[S], l = word(split[S]), r = word(S ^ split[S]);
        B.nodes[me].left = l;
        B.nodes[me].right = r;
        for (int32_t c : {l, r}) {
            if (c & kLeaf) parent_leaf[c & kSlotMask] = me;
            else parent_internal[c] = me;
        }
    }
    for (int i = no - 1; i >= 0; --i) {
        const int32_t me = node_of[order[i]];
        const TBox bl = tbox_of(B, B.nodes[me].left), br = tbox_of(B, B.nodes[me].right);
        for (int a = 0; a < 3; ++a) {
            B.nodes[me].lo[a] = std::fmin(bl.lo[a], br.lo[a]);
            B.nodes[me].hi[a] = std::fmax(bl.hi[a], br.hi[a]);
        }
    }
}

// One pass over every internal node, children before parents (post-order).
void optimize_treelets(Bvh& B, std::vector<int32_t>& parent_internal, std::vector<int32_t>& parent_leaf) {
    if (B.n < 3) return;
    struct Item {
        int32_t node;
        bool expanded;
    };
    std::vector<Item> st;
    st.push_back({0, false});
    while (!st.empty()) {
        Item it = st.back();
        st.pop_back();
        if (it.expanded) {
            restructure_treelet(B, it.node, parent_internal, parent_leaf);
            continue;
        }
        st.push_back({it.node, true});
        for (int32_t c : {B.nodes[it.node].right, B.nodes[it.node].left})
            if (!(c & kLeaf)) st.push_back({c, false});
    }
}

// Moving spheres: the same topology, slot order and hoisted set, with every
// slot's sphere taken from the new array (same original indices) and the
// boxes refit bottom-up.  Mirrors venu_scene_update.
void update_bvh(Bvh& B, const vo_sphere* s) {
    for (uint32_t k = 0; k < B.n; ++k) {
        const vo_sphere& sp = s[B.ids[k]];
        B.center[k] = mk(sp.center[0], sp.center[1], sp.center[2]);
        B.radius[k] = sp.radius;
    }
    refit_bvh(B);
}

void build_bvh(const vo_sphere* s, uint32_t n, Bvh& B) {
    B.n = n;
    B.keys.assign(n, 0);
    B.ids.assign(n, 0);
    B.center.assign(n, f3{0, 0, 0});
    B.radius.assign(n, 0);
    B.nodes.assign(n > 1 ? n - 1 : 0, vo_node{});
    if (n == 0) return;
    // Centroid bounds; Morton codes use one quantisation scale for all axes
    // (the largest extent: cubic cells).  A sphere is huge -- hoisted, below --
    // when its radius exceeds a quarter of that extent.
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t i = 0; i < n; ++i)
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::fmin(lo[a], s[i].center[a]);
            hi[a] = std::fmax(hi[a], s[i].center[a]);
        }
    float ext = 0.0f;
    for (int a = 0; a < 3; ++a) {
        ext = std::fmax(ext, hi[a] - lo[a]);
        B.bounds[a] = lo[a];
        B.bounds[3 + a] = hi[a];
    }
    const float thr = 0.25f * ext;
    std::vector<uint32_t> key(n), idx(n);
    for (uint32_t i = 0; i < n; ++i) {
        uint32_t qx = quant10(s[i].center[0], lo[0], ext);
        uint32_t qy = quant10(s[i].center[1], lo[1], ext);
        uint32_t qz = quant10(s[i].center[2], lo[2], ext);
        key[i] = (spread10(qx) << 2) | (spread10(qy) << 1) | spread10(qz);
        idx[i] = i;
    }
    // Stable sort by key: equal keys keep ascending original index.
    std::stable_sort(idx.begin(), idx.end(), [&](uint32_t a, uint32_t b) { return key[a] < key[b]; });
    for (uint32_t k = 0; k < n; ++k) {
        B.keys[k] = key[idx[k]];
        B.ids[k] = idx[k];
        const vo_sphere& sp = s[idx[k]];
        B.center[k] = mk(sp.center[0], sp.center[1], sp.center[2]);
        B.radius[k] = sp.radius;
    }
    if (n == 1) {
        B.depth = 1;
        return;
    }
    const int N = (int)n;
    std::vector<int32_t> parent_internal(N - 1, -1), parent_leaf(N, -1);
    for (int i = 0; i < N - 1; ++i) {
        int d = (delta(B.keys, N, i, i + 1) - delta(B.keys, N, i, i - 1)) >= 0 ? 1 : -1;
        int dmin = delta(B.keys, N, i, i - d);
        int lmax = 2;
        while (delta(B.keys, N, i, i + lmax * d) > dmin) lmax *= 2;
        int l = 0;
        for (int t = lmax / 2; t >= 1; t /= 2)
            if (delta(B.keys, N, i, i + (l + t) * d) > dmin) l += t;
        int j = i + l * d;
        int dnode = delta(B.keys, N, i, j);
        int s_ = 0;
        for (int div = 2;; div *= 2) {
            int t = (l + div - 1) / div;  // ceil(l / div)
            if (delta(B.keys, N, i, i + (s_ + t) * d) > dnode) s_ += t;
            if (t == 1) break;
        }
        int gamma = i + s_ * d + std::min(d, 0);
        int left = (std::min(i, j) == gamma) ? (gamma | kLeaf) : gamma;
        int right = (std::max(i, j) == gamma + 1) ? ((gamma + 1) | kLeaf) : gamma + 1;
        B.nodes[i].left = left;
        B.nodes[i].right = right;
        if (left & kLeaf) parent_leaf[left & ~kLeaf] = i; else parent_internal[left] = i;
        if (right & kLeaf) parent_leaf[right & ~kLeaf] = i; else parent_internal[right] = i;
    }
    refit_bvh(B);
    optimize_treelets(B, parent_internal, parent_leaf);
    refit_bvh(B);  // boxes unchanged; the depth of the rewired tree
    // Hoisted spheres: the (at most 4) lowest huge slots, if there are at
    // most 64 huge spheres; their leaf words are flagged.
    std::vector<int32_t> cand;
    for (uint32_t k = 0; k < n; ++k)
        if (std::fabs(B.radius[k]) > thr) cand.push_back((int32_t)k);
    if (!cand.empty() && cand.size() <= kHoistCandidates) {
        const size_t nh = std::min(cand.size(), (size_t)kMaxHoisted);
        for (size_t i = 0; i < nh; ++i) {
            const int32_t k = cand[i];
            B.hoist.push_back(k);
            const int32_t p = parent_leaf[k];
            if (p < 0) continue;
            if (B.nodes[p].left == (k | kLeaf)) B.nodes[p].left |= kHoisted;
            else if (B.nodes[p].right == (k | kLeaf)) B.nodes[p].right |= kHoisted;
        }
    }
}

// ---------------------------------------------------------------------------
// GB300-mode ray/box and ray/sphere tests (the CUDA traversal kernel's
// arithmetic).  Explicit fmaf where the kernel uses one.
// ---------------------------------------------------------------------------
// Slab offsets.  The offset -(o inv) of each axis is rounded; a margin of
// |o inv| 2^-21 per axis covers it.  Shared margin (almost every ray): the
// offsets unchanged and the largest margin of the three added to the exit
// parameter.  When that margin exceeds 1 (a near-zero direction component,
// whose margin would switch off the culling on the other axes) each axis
// carries its own margin, moved outwards: nlo for the lo plane, nhi for the
// hi plane (the entry plane is lo when inv >= 0).
constexpr float kSharedMarginMax = 1.0f;
struct RayPre {
    f3 o, d, inv, nlo, nhi;
    float a, inv_a, slack;  // slack: the shared margin (0 with per-axis margins)
    bool axis;
};
inline RayPre prep(f3 o, f3 d) {
    RayPre R;
    R.o = o;
    R.d = d;
    float dd[3] = {d.x, d.y, d.z}, oo[3] = {o.x, o.y, o.z}, inv[3], p[3], m[3], nlo[3], nhi[3];
    for (int a = 0; a < 3; ++a) {
        float di = dd[a];
        if (std::fabs(di) < 1e-20f) di = std::copysign(1e-20f, di);
        inv[a] = 1.0f / di;
        p[a] = oo[a] * inv[a];
        m[a] = std::fabs(p[a]) * 4.76837158203125e-07f;  // 2^-21
    }
    const float mm = std::fmax(std::fmax(m[0], m[1]), m[2]);
    R.axis = mm > kSharedMarginMax;
    for (int a = 0; a < 3; ++a) {
        if (!R.axis) {
            nlo[a] = nhi[a] = -p[a];
        } else {
            const float lo = -p[a] - m[a], hi = -p[a] + m[a];
            nlo[a] = inv[a] >= 0.0f ? lo : hi;
            nhi[a] = inv[a] >= 0.0f ? hi : lo;
        }
    }
    R.slack = R.axis ? 0.0f : mm;
    R.inv = mk(inv[0], inv[1], inv[2]);
    R.nlo = mk(nlo[0], nlo[1], nlo[2]);
    R.nhi = mk(nhi[0], nhi[1], nhi[2]);
    R.a = std::fma(d.x, d.x, std::fma(d.y, d.y, d.z * d.z));
    R.inv_a = 1.0f / R.a;
    return R;
}
inline bool box_test(const RayPre& R, const vo_node& nd, float tmin, float tfar_cap, float& tnear) {
    float t0x = std::fma(nd.lo[0], R.inv.x, R.nlo.x), t1x = std::fma(nd.hi[0], R.inv.x, R.nhi.x);
    float t0y = std::fma(nd.lo[1], R.inv.y, R.nlo.y), t1y = std::fma(nd.hi[1], R.inv.y, R.nhi.y);
    float t0z = std::fma(nd.lo[2], R.inv.z, R.nlo.z), t1z = std::fma(nd.hi[2], R.inv.z, R.nhi.z);
    float tn = std::fmax(std::fmax(std::fmin(t0x, t1x), std::fmin(t0y, t1y)),
                         std::fmax(std::fmin(t0z, t1z), tmin));
    float tf = std::fmin(std::fmin(std::fmax(t0x, t1x), std::fmax(t0y, t1y)),
                         std::fmin(std::fmax(t0z, t1z), tfar_cap));
    tnear = tn;
    if (R.axis) return tn <= tf * 1.00000095367431640625f;  // tf * (1 + 2^-20)
    return tn <= std::fma(tf, 1.00000095367431640625f, R.slack);  // tf * (1 + 2^-20) + shared margin
}
// GB300 ray/sphere: perpendicular-distance discriminant (Ray Tracing Gems
// ch. 7), q-form roots, and an exactly refined c and h when the origin is
// within ~r/16 of the surface.  Same operation sequence as the CUDA kernel.
inline bool sphere_gb300(const RayPre& R, f3 C, float r, float tmin, float tmax, float& tout) {
    float hx = R.o.x - C.x, hy = R.o.y - C.y, hz = R.o.z - C.z;
    float hb = std::fma(hx, R.d.x, std::fma(hy, R.d.y, hz * R.d.z));
    float hh = std::fma(hx, hx, std::fma(hy, hy, hz * hz));
    float r2 = r * r;
    float c = hh - r2;
    // origin clearly outside and moving away from the centre: no hit
    if (hb > 0.0f && c > (hh + r2) * 9.5367431640625e-07f) return false;  // 2^-20
    float discp;
    if (std::fabs(c) < (hh + r2) * 0.0625f) {
        // exact residuals of h = o - C (TwoDiff)
        float bvx = R.o.x - hx, bvy = R.o.y - hy, bvz = R.o.z - hz;
        float ex = (R.o.x - (hx + bvx)) + (bvx - C.x);
        float ey = (R.o.y - (hy + bvy)) + (bvy - C.y);
        float ez = (R.o.z - (hz + bvz)) + (bvz - C.z);
        // c = |h + e|^2 - r^2 from exact squares and compensated sums
        float px = hx * hx, py = hy * hy, pz = hz * hz;
        float qx = std::fma(hx, hx, -px), qy = std::fma(hy, hy, -py), qz = std::fma(hz, hz, -pz);
        float qr = std::fma(r, r, -r2);
        float s1, e1, s2, e2, s3, e3;
        two_sum(px, py, s1, e1);
        two_sum(s1, pz, s2, e2);
        two_sum(s2, -r2, s3, e3);
        float lo = (e1 + e2) + e3;
        lo = lo + ((qx + qy) + qz);
        lo = lo - qr;
        float he = std::fma(hx, ex, std::fma(hy, ey, hz * ez));
        lo = std::fma(2.0f, he, lo);
        c = s3 + lo;
        hb = hb + std::fma(ex, R.d.x, std::fma(ey, R.d.y, ez * R.d.z));
        // f = (h + e) - s d as head + tail, then r^2 - |f|^2 compensated
        const float s = hb * R.inv_a;
        float mx = s * R.d.x, my = s * R.d.y, mz = s * R.d.z;
        float mex = std::fma(s, R.d.x, -mx), mey = std::fma(s, R.d.y, -my), mez = std::fma(s, R.d.z, -mz);
        float fx, fy, fz, fex, fey, fez;
        two_sum(hx, -mx, fx, fex);
        two_sum(hy, -my, fy, fey);
        two_sum(hz, -mz, fz, fez);
        float tx = (fex - mex) + ex, ty = (fey - mey) + ey, tz = (fez - mez) + ez;
        float gx = fx * fx, gy = fy * fy, gz = fz * fz;
        float gex = std::fma(fx, fx, -gx), gey = std::fma(fy, fy, -gy), gez = std::fma(fz, fz, -gz);
        float u1, v1, u2, v2, w, we;
        two_sum(gx, gy, u1, v1);
        two_sum(u1, gz, u2, v2);
        two_sum(r2, -u2, w, we);
        float dl = (we + qr) - (v1 + v2);
        dl = dl - ((gex + gey) + gez);
        dl = std::fma(-2.0f, std::fma(fx, tx, std::fma(fy, ty, fz * tz)), dl);
        discp = w + dl;
    } else {
        const float s = hb * R.inv_a;
        const float fx = std::fma(-s, R.d.x, hx);
        const float fy = std::fma(-s, R.d.y, hy);
        const float fz = std::fma(-s, R.d.z, hz);
        const float ff = std::fma(fx, fx, std::fma(fy, fy, fz * fz));
        discp = std::fma(r, r, -ff);
    }
    if (!(discp >= 0.0f)) return false;
    const float sd = std::sqrt(R.a * discp);
    const float q = -(hb + std::copysign(sd, hb));
    if (q == 0.0f) return false;
    const float ta = q * R.inv_a;
    const float tb = c / q;
    const float t0 = std::fmin(ta, tb), t1 = std::fmax(ta, tb);
    if (t0 >= tmin && t0 <= tmax) {
        tout = t0;
        return true;
    }
    if (t1 >= tmin && t1 <= tmax) {
        tout = t1;
        return true;
    }
    return false;
}

struct Hit {
    int32_t k;  // sorted slot (GB300) or original index (REF); -1 = miss
    float t;
};

const int32_t kNone = 0x7fffffff;

// The LBVH walk shared by both arithmetic modes: test-children-at-parent,
// near child first, far child's child pair pushed with its entry distance;
// popped entries culled against the current closest hit (best_t, which the
// leaf callback lowers).  Tested first: the sphere the ray leaves (`from`,
// GB300 mode only; -1 for none), then the hoisted huge spheres but that one;
// neither is tested again during the walk (the kernels' from_first,
// venusaur_gb300/csrc/venu_device.cuh).
// Deepest traversal stack of the walks on this thread since it was last reset
// (the kernels keep the top entries of the same stack in shared memory).
thread_local int tl_max_stack = 0;

template <class Leaf>
void walk_bvh(const Bvh& B, const RayPre& R, float tmin, const float& best_t, uint64_t* nv, Leaf leaf,
              int32_t from = -1) {
    if (from >= 0) leaf(from);
    for (int32_t k : B.hoist)  // huge spheres (the ground)
        if (k != from) leaf(k);
    if (B.n == 1) {
        if (from != 0) leaf(0);
        return;
    }
    float tn;
    if (nv) ++*nv;
    if (!box_test(R, B.nodes[0], tmin, best_t, tn)) return;
    struct Ent { int32_t l, r; float tn; };
    Ent stack[128];
    int sp = 0;
    int32_t pl = B.nodes[0].left, pr = B.nodes[0].right;
    for (;;) {
        bool h0 = false, h1 = false;
        float tn0 = 0, tn1 = 0;
        int32_t c0l = 0, c0r = 0, c1l = 0, c1r = 0;
        if (pl & kLeaf) {
            if (!(pl & kHoisted) && (pl & kSlotMask) != from) leaf(pl & kSlotMask);
        } else {
            const vo_node& nd = B.nodes[pl];
            if (nv) ++*nv;
            h0 = box_test(R, nd, tmin, best_t, tn0);
            c0l = nd.left;
            c0r = nd.right;
        }
        if (pr & kLeaf) {
            if (!(pr & kHoisted) && (pr & kSlotMask) != from) leaf(pr & kSlotMask);
        } else {
            const vo_node& nd = B.nodes[pr];
            if (nv) ++*nv;
            h1 = box_test(R, nd, tmin, best_t, tn1);
            c1l = nd.left;
            c1r = nd.right;
        }
        if (h0 && h1) {
            if (tn1 < tn0) {
                stack[sp++] = Ent{c0l, c0r, tn0};
                pl = c1l;
                pr = c1r;
            } else {
                stack[sp++] = Ent{c1l, c1r, tn1};
                pl = c0l;
                pr = c0r;
            }
            if (sp > tl_max_stack) tl_max_stack = sp;
        } else if (h0) {
            pl = c0l;
            pr = c0r;
        } else if (h1) {
            pl = c1l;
            pr = c1r;
        } else {
            bool found = false;
            while (sp > 0) {
                --sp;
                if (stack[sp].tn <= best_t) {
                    pl = stack[sp].l;
                    pr = stack[sp].r;
                    found = true;
                    break;
                }
            }
            if (!found) return;
        }
    }
}

// GB300 closest hit: the LBVH walk with the GB300 sphere test.  Ties on t go
// to the smaller sorted slot.  from: sorted slot of the sphere the ray
// leaves (-1: none), tested first.
Hit trace_gb300(const Bvh& B, f3 o, f3 d, float tmin, float tmax, uint64_t* nv, uint64_t* ns,
                int32_t from = -1) {
    Hit h{-1, tmax};
    if (B.n == 0) return h;
    RayPre R = prep(o, d);
    float best_t = tmax;
    int32_t best = kNone;
    walk_bvh(B, R, tmin, best_t, nv, [&](int k) {
        float t;
        if (ns) ++*ns;
        if (sphere_gb300(R, B.center[k], B.radius[k], tmin, tmax, t) &&
            (t < best_t || (t == best_t && k < best))) {
            best_t = t;
            best = k;
        }
    }, from);
    if (best != kNone) {
        h.k = best;
        h.t = best_t;
    }
    return h;
}

// REF-mode intersection: Core/RayTracer.cu:229-270 literally (float), with
// the OptiX interval semantics tmin <= t <= tmax checked by the program.
inline bool sphere_ref(f3 o, f3 d, f3 C, float r, float tmin, float tmax, float& root_out) {
    f3 oc = o - C;
    float a = dot(d, d);
    float half_b = dot(oc, d);
    float c = dot(oc, oc) - r * r;
    float disc = half_b * half_b - a * c;
    if (disc < 0) return false;
    float sqrtd = std::sqrt(disc);
    float root = (-half_b - sqrtd) / a;
    if (root < tmin || tmax < root) {
        root = (-half_b + sqrtd) / a;
        if (root < tmin || tmax < root) return false;
    }
    root_out = root;
    return true;
}
// Brute force in index order; an intersection is accepted when it is closer
// than the current one (the earlier sphere keeps exact ties).
Hit trace_ref(const vo_sphere* s, uint32_t ns, f3 o, f3 d, float tmin, float tmax) {
    Hit h{-1, tmax};
    float cur = tmax;
    for (uint32_t i = 0; i < ns; ++i) {
        float root;
        f3 C = mk(s[i].center[0], s[i].center[1], s[i].center[2]);
        if (sphere_ref(o, d, C, s[i].radius, tmin, cur, root)) {
            if (h.k < 0 || root < cur) {
                h.k = (int32_t)i;
                h.t = root;
                cur = root;
            }
        }
    }
    return h;
}

// REF-mode closest hit through the LBVH: the reference's intersection
// program (sphere_ref, Core/RayTracer.cu:229-270) on the spheres the walk
// reaches, in place of OptiX's hardware traversal.  The accepted hit is the
// brute force's: the smallest root, exact ties to the smaller original index
// (the sphere a brute-force loop in index order keeps).  Returns the
// original index.
Hit trace_ref_bvh(const Bvh& B, f3 o, f3 d, float tmin, float tmax, uint64_t* nv, uint64_t* ns) {
    Hit h{-1, tmax};
    if (B.n == 0) return h;
    RayPre R = prep(o, d);
    float best_t = tmax;
    int32_t best = -1;
    walk_bvh(B, R, tmin, best_t, nv, [&](int k) {
        float root;
        if (ns) ++*ns;
        const int32_t id = (int32_t)B.ids[k];
        if (sphere_ref(o, d, B.center[k], B.radius[k], tmin, best_t, root) &&
            (best < 0 || root < best_t || (root == best_t && id < best))) {
            best_t = root;
            best = id;
        }
    });
    if (best >= 0) {
        h.k = best;
        h.t = best_t;
    }
    return h;
}

// ---------------------------------------------------------------------------
// Camera ray: Core/RayTracer.cu:151-161 and :173-177.
// ---------------------------------------------------------------------------
struct Cam {
    f3 origin, u, v, w, un, vn;
    float lens;
};
Cam load_cam(const vo_camera* c) {
    Cam k;
    k.origin = mk(c->origin[0], c->origin[1], c->origin[2]);
    k.u = mk(c->u[0], c->u[1], c->u[2]);
    k.v = mk(c->v[0], c->v[1], c->v[2]);
    k.w = mk(c->w[0], c->w[1], c->w[2]);
    k.un = normalize(k.u);
    k.vn = normalize(k.v);
    k.lens = c->lens_radius;
    return k;
}
inline void camera_ray(const Cam& C, uint32_t x, uint32_t y, uint32_t W, uint32_t H, uint32_t& seed,
                       f3& o, f3& d) {
    float r1 = rnd(seed);
    float s = 2.0f * ((float)x + r1) / (float)(W - 1) - 1.0f;
    float r2 = rnd(seed);
    float t = 2.0f * ((float)y + r2) / (float)(H - 1) - 1.0f;
    f3 rd = C.lens * random_in_unit_disk(seed);
    f3 offset = C.un * rd.x + C.vn * rd.y;
    o = C.origin + offset;
    d = C.w + (s * C.u) * 0.5f + (t * C.v) * 0.5f - offset;
}

// Sky: Core/RayTracer.cu:442-449.
inline f3 sky_ref(f3 d) {
    f3 ud = normalize(d);
    double t = 0.5 * ((double)ud.y + 1.0);
    return lerp3(mk(1.0f, 1.0f, 1.0f), mk(0.5f, 0.7f, 1.0f), (float)t);
}
inline f3 sky_gb300(f3 d) {
    f3 ud = normalize(d);
    float t = std::fma(0.5f, ud.y, 0.5f);  // == (float)(0.5 * ((double)y + 1.0))
    return lerp3(mk(1.0f, 1.0f, 1.0f), mk(0.5f, 0.7f, 1.0f), t);
}

inline float reflectance_ref(float cosine, float ref_idx) {  // :373-379 (pow for __powf)
    float r0 = (1 - ref_idx) / (1 + ref_idx);
    r0 = r0 * r0;
    return r0 + (1 - r0) * std::pow((1 - cosine), 5.0f);
}
inline float reflectance_gb300(float cosine, float ref_idx) {
    float r0 = (1.0f - ref_idx) / (1.0f + ref_idx);
    r0 = r0 * r0;
    float x = 1.0f - cosine;
    float x2 = x * x;
    float x5 = (x2 * x2) * x;
    return r0 + (1.0f - r0) * x5;
}

struct Scene {
    const vo_sphere* s;
    uint32_t n;
    bool ref_bvh = false;  // REF mode: closest hit through the LBVH, not brute force
    Bvh bvh;
    std::vector<vo_sphere> sorted;  // materials in BVH slot order
};

struct Counters {
    uint64_t segs = 0, nv = 0, ns = 0;
};

// One path in REF mode: the recursion of Core/RayTracer.cu:163-449 unrolled;
// attenuation multiplied on the way back up (innermost albedo first).
f3 path_ref(const Scene& S, f3 o, f3 d, uint32_t seed, int depth, Counters& K) {
    f3 chain[256];
    int nchain = 0;
    f3 att;
    for (;;) {
        Hit h = S.ref_bvh ? trace_ref_bvh(S.bvh, o, d, 0.001f, 1e16f, &K.nv, &K.ns)
                          : trace_ref(S.s, S.n, o, d, 0.001f, 1e16f);
        ++K.segs;
        if (h.k < 0) {
            att = sky_ref(d);
            break;
        }
        const vo_sphere& sp = S.s[h.k];
        f3 C = mk(sp.center[0], sp.center[1], sp.center[2]);
        f3 p = o + d * h.t;
        f3 normal = divs(p - C, sp.radius);
        bool front = dot(d, normal) < 0;
        normal = front ? normal : -normal;
        if (!(depth > 0)) {
            att = mk(0, 0, 0);
            break;
        }
        f3 albedo = mk(sp.albedo[0], sp.albedo[1], sp.albedo[2]);
        if (sp.material == 0) {
            f3 dir = normal + normalize(random_in_unit_sphere(seed));
            if (near_zero(dir)) dir = normal;
            o = p;
            d = dir;
            depth -= 1;
            chain[nchain++] = albedo;
        } else if (sp.material == 1) {
            f3 refl = reflect(normalize(d), normal);
            o = p;
            d = refl + sp.fuzz * random_in_unit_sphere(seed);
            if (dot(d, normal) > 0) {
                depth -= 1;
                chain[nchain++] = albedo;
            } else {
                att = mk(0, 0, 0);
                break;
            }
        } else {
            float ratio = sp.ir;
            if (front) ratio = 1.0f / sp.ir;
            f3 ud = normalize(d);
            double cos_theta = std::fmin(dot(-ud, normal), 1.0f);
            double sin_theta = std::sqrt(1.0 - cos_theta * cos_theta);
            bool cannot = (double)ratio * sin_theta > 1.0;
            f3 dir;
            if (cannot || reflectance_ref((float)cos_theta, ratio) > rnd(seed))
                dir = reflect(ud, normal);
            else
                dir = refract(ud, normal, ratio);
            o = p;
            d = dir;
            depth -= 1;
            chain[nchain++] = mk(NAN, 0, 0);  // no attenuation multiply
        }
        if (nchain >= 256) {
            att = mk(0, 0, 0);
            break;
        }
    }
    for (int i = nchain - 1; i >= 0; --i)
        if (!std::isnan(chain[i].x)) att = att * chain[i];
    return att;
}

// One path in GB300 mode: forward throughput, LBVH closest hit.
f3 path_gb300(const Scene& S, f3 o, f3 d, uint32_t seed, int depth, Counters& K) {
    f3 T = mk(1.0f, 1.0f, 1.0f);
    int32_t from = -1;  // the sphere the ray leaves
    for (;;) {
        Hit h = trace_gb300(S.bvh, o, d, 0.001f, 1e16f, &K.nv, &K.ns, from);
        // carried for slots up to 2^24 - 2 (the kernels keep 1 + slot in 24 bits)
        from = (h.k >= 0 && h.k <= (1 << 24) - 2) ? h.k : -1;
        ++K.segs;
        if (h.k < 0) return T * sky_gb300(d);
        if (!(depth > 0)) return mk(0, 0, 0);
        const vo_sphere& sp = S.sorted[h.k];
        f3 C = mk(sp.center[0], sp.center[1], sp.center[2]);
        f3 p = o + d * h.t;
        f3 outward = divs(p - C, sp.radius);
        bool front = dot(d, outward) < 0;
        f3 n = front ? outward : -outward;
        f3 albedo = mk(sp.albedo[0], sp.albedo[1], sp.albedo[2]);
        if (sp.material == 0) {
            f3 dir = n + normalize(random_in_unit_sphere(seed));
            if (near_zero(dir)) dir = n;
            o = p;
            d = dir;
            depth -= 1;
            T = T * albedo;
        } else if (sp.material == 1) {
            f3 refl = reflect(normalize(d), n);
            f3 dir = refl + sp.fuzz * random_in_unit_sphere(seed);
            if (dot(dir, n) > 0) {
                o = p;
                d = dir;
                depth -= 1;
                T = T * albedo;
            } else {
                return mk(0, 0, 0);
            }
        } else {
            float ratio = front ? (1.0f / sp.ir) : sp.ir;
            f3 ud = normalize(d);
            float cos_t = std::fmin(dot(-ud, n), 1.0f);
            float sin_t = std::sqrt(1.0f - cos_t * cos_t);
            bool cannot = ratio * sin_t > 1.0f;
            f3 dir;
            if (cannot || reflectance_gb300(cos_t, ratio) > rnd(seed))
                dir = reflect(ud, n);
            else
                dir = refract(ud, n, ratio);
            o = p;
            d = dir;
            depth -= 1;
        }
    }
}

// x^(1/2.4) for x in [2^-126, 1]: the sRGB encode's power in the GB300
// arithmetic, restating the CUDA kernel's routine operation by operation
// (IEEE +, -, *, / and fma only, so host and device round identically).
// x = m 2^e with m in [sqrt(1/2), sqrt(2)); log2 m = s (c1 + c3 s^2 + ...),
// s = (m-1)/(m+1), the atanh series of ln m = 2 atanh s scaled by 1/ln 2;
// t = y (e + log2 m) with y e split exactly (TwoProduct); 2^t = 2^n 2^f,
// n = rint(t), 2^f by its Taylor series to f^7.
inline float srgb_pow(float x) {
    uint32_t b;
    std::memcpy(&b, &x, 4);
    int e = (int)(b >> 23) - 127;
    const uint32_t mb = (b & 0x007fffffu) | 0x3f800000u;
    float m;
    std::memcpy(&m, &mb, 4);
    if (m > 1.41421353816986083984375f) {
        m = m * 0.5f;
        e += 1;
    }
    const float s = (m - 1.0f) / (m + 1.0f);
    const float z = s * s;
    float tail = std::fma(z, 0.32059890031814575f, 0.41219857335090637f);
    tail = std::fma(z, tail, 0.5770780444145203f);
    tail = std::fma(z, tail, 0.9617967009544373f);
    tail = std::fma(z, tail, 3.8519259e-08f);
    const float L = std::fma(s, 2.885390043258667f, s * tail);
    const float y = 0.4166666567325592f;
    const float fe = (float)e;
    const float ph = fe * y;
    const float pl = std::fma(fe, y, -ph);
    const float q = std::fma(y, L, pl);
    const float n = std::rint(ph + q);
    const float f = (ph - n) + q;
    float p = std::fma(f, 1.5252733646775596e-05f, 1.540352968731895e-04f);
    p = std::fma(f, p, 1.3333557872101665e-03f);
    p = std::fma(f, p, 9.618128649890423e-03f);
    p = std::fma(f, p, 5.550410971045494e-02f);
    p = std::fma(f, p, 2.4022650718688965e-01f);
    p = std::fma(f, p, 6.931471824645996e-01f);
    p = std::fma(f, p, 1.0f);
    const uint32_t sb = (uint32_t)(127 + (int)n) << 23;
    float scale;
    std::memcpy(&scale, &sb, 4);
    return p * scale;
}

// Core/RayTracer.cu:16-47
inline uint8_t quant8(float x) {
    x = clampf(x, 0.0f, 1.0f);
    uint32_t q = (uint32_t)(x * 256.0f);
    return (uint8_t)(q < 255u ? q : 255u);
}
// ref = false: the GB300 arithmetic's own power routine in place of pow().
inline void make_color(f3 c, uint8_t* out, bool ref = true) {
    c = mk(clampf(c.x, 0.0f, 1.0f), clampf(c.y, 0.0f, 1.0f), clampf(c.z, 0.0f, 1.0f));
    float inv_gamma = 1.0f / 2.4f;
    float p[3] = {std::pow(c.x, inv_gamma), std::pow(c.y, inv_gamma), std::pow(c.z, inv_gamma)};
    if (!ref) {
        p[0] = c.x < 0.0031308f ? 0.0f : srgb_pow(c.x);
        p[1] = c.y < 0.0031308f ? 0.0f : srgb_pow(c.y);
        p[2] = c.z < 0.0031308f ? 0.0f : srgb_pow(c.z);
    }
    float v[3] = {c.x, c.y, c.z};
    for (int i = 0; i < 3; ++i) {
        float srgb = v[i] < 0.0031308f ? 12.92f * v[i] : 1.055f * p[i] - 0.055f;
        out[i] = quant8(srgb);
    }
    out[3] = 255;
}

}  // namespace

extern "C" {

uint32_t vo_tea4(uint32_t v0, uint32_t v1) { return tea4(v0, v1); }

void vo_rnd_stream(uint32_t seed, uint32_t n, float* out, uint32_t* states_out) {
    for (uint32_t i = 0; i < n; ++i) {
        out[i] = rnd(seed);
        if (states_out) states_out[i] = seed;
    }
}

uint32_t vo_scene_rtiow(uint32_t seed, vo_sphere* out, uint32_t cap) {
    std::vector<vo_sphere> v;
    SceneRng R(seed);
    v.push_back(make_sphere(mk(0.0f, -1000.0f, 0.0f), 1000.0f, 0, mk(0.5f, 0.5f, 0.5f), 0.0f, 0.0f));
    for (int a = -11; a < 11; a++) {
        for (int b = -11; b < 11; b++) {
            float choose = R.U();
            float ux = R.U();
            float cx = (float)((double)a + 0.9 * (double)ux);
            float uz = R.U();
            float cz = (float)((double)b + 0.9 * (double)uz);
            f3 center = mk(cx, 0.2f, cz);
            f3 dd = center - mk(4.0f, 0.2f, 0.0f);
            float len = std::sqrt(dot(dd, dd));
            if ((double)len > 0.9) v.push_back(draw_material(R, choose, center, 0.2f));
        }
    }
    v.push_back(make_sphere(mk(0, 1, 0), 1.0f, 2, mk(0, 0, 0), 0.0f, 1.5f));
    v.push_back(make_sphere(mk(-4, 1, 0), 1.0f, 0, mk(0.4f, 0.2f, 0.1f), 0.0f, 0.0f));
    v.push_back(make_sphere(mk(4, 1, 0), 1.0f, 1, mk(0.7f, 0.6f, 0.5f), 0.0f, 0.0f));
    uint32_t n = (uint32_t)v.size();
    if (out) std::memcpy(out, v.data(), sizeof(vo_sphere) * std::min(n, cap));
    return n;
}

uint32_t vo_scene_random(uint32_t n, uint32_t seed, const float box_lo[3], const float box_hi[3],
                         float rmin, float rmax, vo_sphere* out) {
    if (n == 0) return 0;
    SceneRng R(seed);
    out[0] = make_sphere(mk(0.0f, -1000.0f, 0.0f), 1000.0f, 0, mk(0.5f, 0.5f, 0.5f), 0.0f, 0.0f);
    double lrat = det_log((double)rmax / (double)rmin);
    for (uint32_t i = 1; i < n; ++i) {
        float choose = R.U();
        float cx = box_lo[0] + (box_hi[0] - box_lo[0]) * R.U();
        float cy = box_lo[1] + (box_hi[1] - box_lo[1]) * R.U();
        float cz = box_lo[2] + (box_hi[2] - box_lo[2]) * R.U();
        float ur = R.U();
        float r = (float)((double)rmin * det_exp((double)ur * lrat));
        out[i] = draw_material(R, choose, mk(cx, cy, cz), r);
    }
    return n;
}

void vo_camera_look_at(const float eye[3], const float lookat[3], float vfov_deg, float aspect,
                       float aperture, float focal, vo_camera* out) {
    // glm semantics: normalize(v) = v * (1 / sqrt(dot)), dot = (x*x + y*y) + z*z.
    auto gnorm = [](f3 v) {
        float inv = 1.0f / std::sqrt(dot(v, v));
        return v * inv;
    };
    auto gcross = [](f3 x, f3 y) {
        return mk(x.y * y.z - y.y * x.z, x.z * y.x - y.z * x.x, x.x * y.y - y.x * x.y);
    };
    f3 fwd = gnorm(mk(lookat[0] - eye[0], lookat[1] - eye[1], lookat[2] - eye[2]));
    f3 w = fwd * focal;
    f3 u = gnorm(gcross(w, mk(0.0f, 1.0f, 0.0f)));
    f3 v = gnorm(gcross(u, w));
    float theta = vfov_deg * 0.01745329251994329576923690768489f;
    float h = std::tan(theta * 0.5f);
    float vh = 2.0f * h;
    float vw = aspect * vh;
    u = u * (focal * vw);
    v = v * (focal * vh);
    for (int i = 0; i < 3; ++i) out->origin[i] = eye[i];
    out->u[0] = u.x; out->u[1] = u.y; out->u[2] = u.z;
    out->v[0] = v.x; out->v[1] = v.y; out->v[2] = v.z;
    out->w[0] = w.x; out->w[1] = w.y; out->w[2] = w.z;
    out->lens_radius = aperture * 0.5f;
}

int vo_lbvh_build(const vo_sphere* s, uint32_t n, uint32_t* morton_sorted, uint32_t* sorted_ids,
                  vo_node* nodes, float bounds[6], uint32_t* depth_out) {
    Bvh B;
    build_bvh(s, n, B);
    if (morton_sorted) std::memcpy(morton_sorted, B.keys.data(), 4 * (size_t)n);
    if (sorted_ids) std::memcpy(sorted_ids, B.ids.data(), 4 * (size_t)n);
    if (nodes && n > 1) std::memcpy(nodes, B.nodes.data(), sizeof(vo_node) * (size_t)(n - 1));
    if (bounds) std::memcpy(bounds, B.bounds, sizeof(B.bounds));
    if (depth_out) *depth_out = B.depth;
    return 0;
}

int vo_lbvh_refit(const vo_sphere* s_build, const vo_sphere* s_new, uint32_t n, vo_node* nodes) {
    Bvh B;
    build_bvh(s_build, n, B);
    update_bvh(B, s_new);
    if (nodes && n > 1) std::memcpy(nodes, B.nodes.data(), sizeof(vo_node) * (size_t)(n - 1));
    return 0;
}

void vo_trace_fp64(const vo_sphere* s, uint32_t ns, const float* rays, uint32_t n, float tmin,
                   float tmax, int32_t* id, double* t, double* disc_rel, double* t_second) {
    for (uint32_t i = 0; i < n; ++i) {
        const float* r = rays + 6 * (size_t)i;
        double o[3] = {r[0], r[1], r[2]}, d[3] = {r[3], r[4], r[5]};
        double a = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        int32_t best = -1;
        double bt = INFINITY, b2 = INFINITY, bdisc = 0;
        for (uint32_t k = 0; k < ns; ++k) {
            double oc[3] = {o[0] - (double)s[k].center[0], o[1] - (double)s[k].center[1],
                            o[2] - (double)s[k].center[2]};
            double rr = (double)s[k].radius;
            double hb = oc[0] * d[0] + oc[1] * d[1] + oc[2] * d[2];
            double c = oc[0] * oc[0] + oc[1] * oc[1] + oc[2] * oc[2] - rr * rr;
            double disc = hb * hb - a * c;
            if (disc < 0) continue;
            double sd = std::sqrt(disc);
            double q = -(hb + std::copysign(sd, hb));
            if (q == 0) continue;
            double r0 = q / a, r1 = c / q;
            double lo = std::min(r0, r1), hi = std::max(r0, r1), tt;
            if (lo >= tmin && lo <= tmax) tt = lo;
            else if (hi >= tmin && hi <= tmax) tt = hi;
            else continue;
            if (tt < bt) {
                b2 = bt;
                bt = tt;
                best = (int32_t)k;
                bdisc = disc / (a * rr * rr);
            } else if (tt < b2) {
                b2 = tt;
            }
        }
        id[i] = best;
        if (t) t[i] = best >= 0 ? bt : INFINITY;
        if (disc_rel) disc_rel[i] = bdisc;
        if (t_second) t_second[i] = b2;
    }
}

void vo_trace_bvh(const vo_sphere* s, uint32_t ns, const float* rays, uint32_t n, float tmin,
                  float tmax, int32_t* id, float* t, uint32_t* front, uint32_t* nodes_visited,
                  uint32_t* spheres_tested) {
    Bvh B;
    build_bvh(s, ns, B);
    for (uint32_t i = 0; i < n; ++i) {
        const float* r = rays + 6 * (size_t)i;
        f3 o = mk(r[0], r[1], r[2]), d = mk(r[3], r[4], r[5]);
        uint64_t nv = 0, nsph = 0;
        Hit h = trace_gb300(B, o, d, tmin, tmax, &nv, &nsph);
        if (h.k >= 0) {
            id[i] = (int32_t)B.ids[h.k];
            t[i] = h.t;
            if (front) {
                f3 C = B.center[h.k];
                f3 p = o + d * h.t;
                f3 outward = divs(p - C, B.radius[h.k]);
                front[i] = dot(d, outward) < 0 ? 1u : 0u;
            }
        } else {
            id[i] = -1;
            t[i] = tmax;
            if (front) front[i] = 0;
        }
        if (nodes_visited) nodes_visited[i] = (uint32_t)nv;
        if (spheres_tested) spheres_tested[i] = (uint32_t)nsph;
    }
}

void vo_trace_bvh_stack(const vo_sphere* s, uint32_t ns, const float* rays, uint32_t n, float tmin, float tmax,
                        uint32_t* max_stack) {
    Bvh B;
    build_bvh(s, ns, B);
    for (uint32_t i = 0; i < n; ++i) {
        const float* r = rays + 6 * (size_t)i;
        tl_max_stack = 0;
        trace_gb300(B, mk(r[0], r[1], r[2]), mk(r[3], r[4], r[5]), tmin, tmax, nullptr, nullptr);
        max_stack[i] = (uint32_t)tl_max_stack;
    }
}

void vo_trace_ref(const vo_sphere* s, uint32_t ns, const float* rays, uint32_t n, float tmin,
                  float tmax, int32_t* id, float* t) {
    for (uint32_t i = 0; i < n; ++i) {
        const float* r = rays + 6 * (size_t)i;
        Hit h = trace_ref(s, ns, mk(r[0], r[1], r[2]), mk(r[3], r[4], r[5]), tmin, tmax);
        id[i] = h.k;
        t[i] = h.t;
    }
}

uint64_t vo_render(const vo_sphere* s, uint32_t ns, const vo_camera* cam, const vo_render_opts* opts,
                   float* accum, float* image_f, uint8_t* image8, float* samples_out,
                   uint64_t* nodes_visited, uint64_t* spheres_tested) {
    return vo_render_refit(nullptr, s, ns, cam, opts, accum, image_f, image8, samples_out, nodes_visited,
                           spheres_tested);
}

uint64_t vo_render_refit(const vo_sphere* s_build, const vo_sphere* s, uint32_t ns, const vo_camera* cam,
                         const vo_render_opts* opts, float* accum, float* image_f, uint8_t* image8,
                         float* samples_out, uint64_t* nodes_visited, uint64_t* spheres_tested) {
    Scene S;
    S.s = s;
    S.n = ns;
    const bool gb = opts->mode == VO_MODE_GB300;
    S.ref_bvh = opts->mode == VO_MODE_REF_BVH;
    if (gb || S.ref_bvh) {
        build_bvh(s_build ? s_build : s, ns, S.bvh);
        if (s_build) update_bvh(S.bvh, s);
    }
    if (gb) {
        S.sorted.resize(ns);
        for (uint32_t k = 0; k < ns; ++k) S.sorted[k] = s[S.bvh.ids[k]];
    }
    const Cam C = load_cam(cam);
    const uint32_t W = opts->width, H = opts->height, spp = opts->spp;
    const uint32_t r0 = (opts->row_end > opts->row_begin) ? opts->row_begin : 0;
    const uint32_t r1 = (opts->row_end > opts->row_begin) ? std::min(opts->row_end, H) : H;
    const int maxd = (int)opts->max_depth;
    unsigned nt = opts->nthreads ? opts->nthreads : std::max(1u, std::thread::hardware_concurrency());
    std::atomic<uint32_t> next_row{r0};
    std::vector<Counters> counters(nt);
    const size_t rows_px = (size_t)(r1 - r0) * W;
    auto worker = [&](unsigned tid) {
        Counters& K = counters[tid];
        for (;;) {
            uint32_t y = next_row.fetch_add(1);
            if (y >= r1) break;
            for (uint32_t x = 0; x < W; ++x) {
                const uint32_t idx = y * W + x;
                uint32_t seed = tea4(idx, opts->subframe_index);
                if (gb) {
                    float* a = accum + 8 * (size_t)idx;
                    float sum[3] = {a[0], a[1], a[2]}, comp[3] = {a[4], a[5], a[6]};
                    float cnt = a[3];
                    for (uint32_t smp = 0; smp < spp; ++smp) {
                        f3 o, d;
                        camera_ray(C, x, y, W, H, seed, o, d);
                        f3 L = path_gb300(S, o, d, seed, maxd - 1, K);
                        if (samples_out) {
                            float* so = samples_out + 3 * ((size_t)smp * rows_px + (size_t)(y - r0) * W + x);
                            so[0] = L.x; so[1] = L.y; so[2] = L.z;
                        }
                        float v[3] = {L.x, L.y, L.z};
                        for (int c = 0; c < 3; ++c) {  // Kahan
                            float yk = v[c] - comp[c];
                            float tk = sum[c] + yk;
                            comp[c] = (tk - sum[c]) - yk;
                            sum[c] = tk;
                        }
                        cnt = cnt + 1.0f;
                    }
                    a[0] = sum[0]; a[1] = sum[1]; a[2] = sum[2]; a[3] = cnt;
                    a[4] = comp[0]; a[5] = comp[1]; a[6] = comp[2]; a[7] = 0.0f;
                    f3 mean = mk(sum[0] / cnt, sum[1] / cnt, sum[2] / cnt);
                    if (image_f) {
                        float* f = image_f + 4 * (size_t)idx;
                        f[0] = mean.x; f[1] = mean.y; f[2] = mean.z; f[3] = 1.0f;
                    }
                    if (image8) make_color(mean, image8 + 4 * (size_t)idx, false);
                } else {
                    f3 pc = mk(0, 0, 0);
                    for (uint32_t smp = 0; smp < spp; ++smp) {
                        f3 o, d;
                        camera_ray(C, x, y, W, H, seed, o, d);
                        f3 L = path_ref(S, o, d, seed, maxd - 1, K);
                        if (samples_out) {
                            float* so = samples_out + 3 * ((size_t)smp * rows_px + (size_t)(y - r0) * W + x);
                            so[0] = L.x; so[1] = L.y; so[2] = L.z;
                        }
                        pc = pc + L;
                    }
                    f3 ac = divs(pc, (float)spp);
                    float* a = accum + 4 * (size_t)idx;
                    if (opts->subframe_index > 0) {
                        float al = 1.0f / (float)(opts->subframe_index + 1);
                        ac = lerp3(mk(a[0], a[1], a[2]), ac, al);
                    }
                    a[0] = ac.x; a[1] = ac.y; a[2] = ac.z; a[3] = 1.0f;
                    if (image_f) {
                        float* f = image_f + 4 * (size_t)idx;
                        f[0] = ac.x; f[1] = ac.y; f[2] = ac.z; f[3] = 1.0f;
                    }
                    if (image8) make_color(ac, image8 + 4 * (size_t)idx);
                }
            }
        }
    };
    std::vector<std::thread> th;
    for (unsigned i = 1; i < nt; ++i) th.emplace_back(worker, i);
    worker(0);
    for (auto& t : th) t.join();
    uint64_t segs = 0, nv = 0, nsph = 0;
    for (auto& k : counters) {
        segs += k.segs;
        nv += k.nv;
        nsph += k.ns;
    }
    if (nodes_visited) *nodes_visited = nv;
    if (spheres_tested) *spheres_tested = nsph;
    return segs;
}

void vo_make_color(const float* rgb, uint32_t n, uint8_t* out4) {
    for (uint32_t i = 0; i < n; ++i) make_color(mk(rgb[3 * i], rgb[3 * i + 1], rgb[3 * i + 2]), out4 + 4 * i);
}

void vo_make_color_gb300(const float* rgb, uint32_t n, uint8_t* out4) {
    for (uint32_t i = 0; i < n; ++i)
        make_color(mk(rgb[3 * i], rgb[3 * i + 1], rgb[3 * i + 2]), out4 + 4 * i, false);
}

void vo_srgb_pow(const float* x, uint64_t n, float* out) {
    for (uint64_t i = 0; i < n; ++i) out[i] = srgb_pow(x[i]);
}

}  // extern "C"
