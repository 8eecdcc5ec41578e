/*
 * oracle.cpp -- CPU oracle for the RaySpace3D query path (TEST INFRASTRUCTURE).
 * See oracle.h for what it restates and who may call it.
 *
 * Compile with -ffp-contract=off: the hit-distance formula is a fixed sequence of
 * individually rounded IEEE float operations, shared as a contract with the GPU.
 */
#include "oracle.h"

#include <algorithm>
#include <array>
#include <atomic>
#include <map>
#include <unordered_map>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

namespace {

// ---------------------------------------------------------------------------
// Exact big-integer arithmetic.  A finite float f is the integer f * 2^149
// (2^-149 is the smallest subnormal), so every predicate below is a
// homogeneous integer polynomial whose sign is computed exactly.
// ---------------------------------------------------------------------------
constexpr int kLimbs = 36;  // 1152 bits; degree-3 products of 2^278 values need < 840

struct Big {
    int neg = 0;
    int len = 0;  // number of significant limbs
    uint32_t w[kLimbs];
};

static void big_zero(Big& r) { r.neg = 0; r.len = 0; }

static void big_trim(Big& r) {
    while (r.len > 0 && r.w[r.len - 1] == 0) r.len--;
    if (r.len == 0) r.neg = 0;
}

static void big_from_float(Big& r, float f) {
    uint32_t bits;
    std::memcpy(&bits, &f, 4);
    big_zero(r);
    uint32_t e = (bits >> 23) & 0xffu;
    uint64_t m = bits & 0x7fffffu;
    int shift = 0;
    if (e != 0) { m |= 0x800000u; shift = (int)e - 1; }
    if (m == 0) return;
    int limb = shift / 32, off = shift % 32;
    uint64_t v = m << off;
    for (int i = 0; i < limb + 3 && i < kLimbs; ++i) r.w[i] = 0;
    r.w[limb] = (uint32_t)v;
    r.w[limb + 1] = (uint32_t)(v >> 32);
    r.len = limb + 2;
    r.neg = (int)(bits >> 31);
    big_trim(r);
}

static int mag_cmp(const Big& a, const Big& b) {
    if (a.len != b.len) return a.len < b.len ? -1 : 1;
    for (int i = a.len - 1; i >= 0; --i)
        if (a.w[i] != b.w[i]) return a.w[i] < b.w[i] ? -1 : 1;
    return 0;
}

static void mag_add(Big& r, const Big& a, const Big& b) {  // |r| = |a| + |b|
    int n = std::max(a.len, b.len);
    uint64_t carry = 0;
    for (int i = 0; i < n; ++i) {
        uint64_t s = carry + (i < a.len ? a.w[i] : 0u) + (i < b.len ? b.w[i] : 0u);
        r.w[i] = (uint32_t)s;
        carry = s >> 32;
    }
    r.len = n;
    if (carry) r.w[r.len++] = (uint32_t)carry;
}

static void mag_sub(Big& r, const Big& a, const Big& b) {  // |r| = |a| - |b|, |a| >= |b|
    int64_t borrow = 0;
    for (int i = 0; i < a.len; ++i) {
        int64_t s = (int64_t)a.w[i] - (i < b.len ? (int64_t)b.w[i] : 0) - borrow;
        borrow = s < 0;
        r.w[i] = (uint32_t)(s + (borrow ? ((int64_t)1 << 32) : 0));
    }
    r.len = a.len;
}

static void big_add(Big& r, const Big& a, const Big& b) {
    Big t;
    if (a.neg == b.neg) {
        mag_add(t, a, b);
        t.neg = a.neg;
    } else if (mag_cmp(a, b) >= 0) {
        mag_sub(t, a, b);
        t.neg = a.neg;
    } else {
        mag_sub(t, b, a);
        t.neg = b.neg;
    }
    big_trim(t);
    r = t;
}

static void big_sub(Big& r, const Big& a, const Big& b) {
    Big nb = b;
    if (nb.len) nb.neg ^= 1;
    big_add(r, a, nb);
}

static void big_mul(Big& r, const Big& a, const Big& b) {
    Big t;
    big_zero(t);
    if (a.len == 0 || b.len == 0) { r = t; return; }
    int n = a.len + b.len;
    if (n > kLimbs) std::abort();  // cannot happen for float inputs (see kLimbs)
    for (int i = 0; i < n; ++i) t.w[i] = 0;
    for (int i = 0; i < a.len; ++i) {
        uint64_t carry = 0;
        for (int j = 0; j < b.len; ++j) {
            uint64_t cur = (uint64_t)a.w[i] * b.w[j] + t.w[i + j] + carry;
            t.w[i + j] = (uint32_t)cur;
            carry = cur >> 32;
        }
        int k = i + b.len;
        while (carry) {
            uint64_t cur = (uint64_t)t.w[k] + carry;
            t.w[k] = (uint32_t)cur;
            carry = cur >> 32;
            ++k;
        }
    }
    t.len = n;
    t.neg = a.neg ^ b.neg;
    big_trim(t);
    r = t;
}

static int big_sign(const Big& a) { return a.len == 0 ? 0 : (a.neg ? -1 : 1); }

// ---------------------------------------------------------------------------
// Exact predicates.
//   orient(d,o,a,b)   = sign det[d, a-o, b-o]
//   axis_det(d,k,a,b) = sign det[d, e_k, b-a]
// A double-precision filter decides almost every case; the big-integer path
// settles the rest.  The filter bound is generous (32 units of 2^-53).
// ---------------------------------------------------------------------------
static int orient_exact_big(const float d[3], const float o[3], const float a[3], const float b[3]) {
    Big D[3], A[3], B[3], t0, t1;
    for (int k = 0; k < 3; ++k) {
        Big fa, fb, fo;
        big_from_float(D[k], d[k]);
        big_from_float(fa, a[k]);
        big_from_float(fb, b[k]);
        big_from_float(fo, o[k]);
        big_sub(A[k], fa, fo);
        big_sub(B[k], fb, fo);
    }
    Big acc;
    big_zero(acc);
    for (int k = 0; k < 3; ++k) {
        int i = (k + 1) % 3, j = (k + 2) % 3;
        Big c;
        big_mul(t0, A[i], B[j]);
        big_mul(t1, A[j], B[i]);
        big_sub(c, t0, t1);
        big_mul(t0, D[k], c);
        big_add(acc, acc, t0);
    }
    return big_sign(acc);
}

static int orient(const float d[3], const float o[3], const float a[3], const float b[3]) {
    double A[3], B[3];
    for (int k = 0; k < 3; ++k) {
        A[k] = (double)a[k] - (double)o[k];
        B[k] = (double)b[k] - (double)o[k];
    }
    double det = 0.0, mag = 0.0;
    for (int k = 0; k < 3; ++k) {
        int i = (k + 1) % 3, j = (k + 2) % 3;
        double p = A[i] * B[j], q = A[j] * B[i];
        det += (double)d[k] * (p - q);
        mag += std::fabs((double)d[k]) * (std::fabs(p) + std::fabs(q));
    }
    const double bound = 32.0 * std::ldexp(1.0, -53) * mag;
    if (std::isfinite(mag) && mag > 1e-250) {
        if (det > bound) return 1;
        if (det < -bound) return -1;
    }
    return orient_exact_big(d, o, a, b);
}

static int axis_det(const float d[3], int k, const float a[3], const float b[3]) {
    int i = (k + 1) % 3, j = (k + 2) % 3;
    double Ei = (double)b[i] - (double)a[i], Ej = (double)b[j] - (double)a[j];
    double p = (double)d[j] * Ei, q = (double)d[i] * Ej;
    double det = p - q;
    double bound = 8.0 * std::ldexp(1.0, -53) * (std::fabs(p) + std::fabs(q));
    if (std::isfinite(bound) && (std::fabs(p) + std::fabs(q)) > 1e-250) {
        if (det > bound) return 1;
        if (det < -bound) return -1;
    }
    Big D[3], fa, fb, Ei_b, Ej_b, t0, t1, r;
    big_from_float(D[i], d[i]);
    big_from_float(D[j], d[j]);
    big_from_float(fa, a[i]);
    big_from_float(fb, b[i]);
    big_sub(Ei_b, fb, fa);
    big_from_float(fa, a[j]);
    big_from_float(fb, b[j]);
    big_sub(Ej_b, fb, fa);
    big_mul(t0, D[j], Ei_b);
    big_mul(t1, D[i], Ej_b);
    big_sub(r, t0, t1);
    return big_sign(r);
}

static void perturb_axes(const float d[3], int& kx, int& ky) {
    int kz = 2;
    if (std::fabs(d[0]) > std::fabs(d[kz])) kz = 0;
    if (std::fabs(d[1]) > std::fabs(d[kz])) kz = 1;
    kx = (kz + 1) % 3;
    ky = (kz + 2) % 3;
}

// Sign of the edge function of (a,b) for the origin perturbed by
// delta*e_kx + delta^2*e_ky: det[d,a-o,b-o] - delta*det[d,e_kx,b-a] - delta^2*det[d,e_ky,b-a].
static int perturbed_sign(const float d[3], const float o[3], const float a[3], const float b[3], int kx, int ky) {
    int s = orient(d, o, a, b);
    if (s) return s;
    s = -axis_det(d, kx, a, b);
    if (s) return s;
    return -axis_det(d, ky, a, b);
}

// ---------------------------------------------------------------------------
// Ray and the hit contract.
// ---------------------------------------------------------------------------
struct Ray {
    float o[3], d[3], inv[3];
    int zero[3];
    int kx, ky;
    float tmin, tmax;
};

static Ray make_ray(const float o[3], const float d[3], float tmin, float tmax) {
    Ray r;
    for (int k = 0; k < 3; ++k) {
        r.o[k] = o[k];
        r.d[k] = d[k];
        r.zero[k] = 0;
        r.inv[k] = 0.0f;
        if (d[k] == 0.0f) {
            r.zero[k] = 1;
        } else {
            r.inv[k] = 1.0f / d[k];
            if (std::isinf(r.inv[k])) r.zero[k] = 1;
        }
    }
    perturb_axes(d, r.kx, r.ky);
    r.tmin = tmin;
    r.tmax = tmax;
    return r;
}

// Slab interval of a box clipped to [tmin, tmax]; monotone in the box bounds,
// so a box that contains another passes whenever the contained one does.
static bool slab_range(const Ray& r, const float lo[3], const float hi[3], float en, float ex,
                       float& enter, float& exit) {
    for (int k = 0; k < 3; ++k) {
        if (r.zero[k]) {
            if (r.o[k] < lo[k] || r.o[k] > hi[k]) return false;
            continue;
        }
        float t1 = (lo[k] - r.o[k]) * r.inv[k];
        float t2 = (hi[k] - r.o[k]) * r.inv[k];
        float tn = r.inv[k] > 0.0f ? t1 : t2;
        float tf = r.inv[k] > 0.0f ? t2 : t1;
        en = tn > en ? tn : en;
        ex = tf < ex ? tf : ex;
    }
    enter = en;
    exit = ex;
    return en <= ex;
}

static bool slab(const Ray& r, const float lo[3], const float hi[3], float& enter, float& exit) {
    return slab_range(r, lo, hi, r.tmin, r.tmax, enter, exit);
}

// Triangle hit contract: the slab interval of the triangle's own box (not
// clipped to the query range) is non-empty, the perturbed origin lies strictly
// inside the triangle's projection along d (exact signs), and t -- the
// fixed-sequence float distance clamped to that slab interval -- lies in
// [tmin, tmax].  Every box containing an accepted triangle's box passes the
// clipped slab test, so BVH culling never changes the hit set.
static bool hit_triangle(const Ray& r, const float* a, const float* b, const float* c, float& t) {
    float lo[3], hi[3];
    for (int k = 0; k < 3; ++k) {
        float mn = a[k] < b[k] ? a[k] : b[k];
        mn = c[k] < mn ? c[k] : mn;
        float mx = a[k] > b[k] ? a[k] : b[k];
        mx = c[k] > mx ? c[k] : mx;
        lo[k] = mn;
        hi[k] = mx;
    }
    float en, ex;
    if (!slab_range(r, lo, hi, -INFINITY, INFINITY, en, ex)) return false;
    int s0 = perturbed_sign(r.d, r.o, a, b, r.kx, r.ky);
    if (s0 == 0) return false;
    int s1 = perturbed_sign(r.d, r.o, b, c, r.kx, r.ky);
    if (s1 != s0) return false;
    int s2 = perturbed_sign(r.d, r.o, c, a, r.kx, r.ky);
    if (s2 != s0) return false;
    // Fixed operation sequence (each operation rounded to float).
    float e1x = b[0] - a[0], e1y = b[1] - a[1], e1z = b[2] - a[2];
    float e2x = c[0] - a[0], e2y = c[1] - a[1], e2z = c[2] - a[2];
    float nx = e1y * e2z - e1z * e2y;
    float ny = e1z * e2x - e1x * e2z;
    float nz = e1x * e2y - e1y * e2x;
    float wx = a[0] - r.o[0], wy = a[1] - r.o[1], wz = a[2] - r.o[2];
    float num = (wx * nx + wy * ny) + wz * nz;
    float den = (r.d[0] * nx + r.d[1] * ny) + r.d[2] * nz;
    float traw = num / den;
    t = (traw >= en) ? ((traw <= ex) ? traw : ex) : en;
    return t >= r.tmin && t <= r.tmax;
}

// ---------------------------------------------------------------------------
// Mesh view and a CPU BVH (median split on centroids, leaves of <= 4).
// ---------------------------------------------------------------------------
struct Mesh {
    const float* V;
    uint64_t nV;
    const uint32_t* I;
    uint64_t nF;
    const int32_t* t2o;
    const float* vtx(uint64_t tri, int corner) const {
        uint32_t vi = I[3 * tri + corner];
        return V + 3 * (uint64_t)vi;
    }
    bool valid(uint64_t tri) const {
        return I[3 * tri] < nV && I[3 * tri + 1] < nV && I[3 * tri + 2] < nV;
    }
};

struct CpuNode {
    float lo[3], hi[3];
    int64_t left;   // child index, or -1 for a leaf
    int64_t right;
    uint64_t first, count;
};

struct CpuBvh {
    std::vector<CpuNode> nodes;
    std::vector<uint64_t> order;
};

static void build_bvh(const Mesh& m, CpuBvh& bvh) {
    bvh.nodes.clear();
    bvh.order.clear();
    std::vector<float> cen;
    std::vector<float> blo, bhi;
    for (uint64_t t = 0; t < m.nF; ++t) {
        if (!m.valid(t)) continue;
        bvh.order.push_back(t);
    }
    uint64_t n = bvh.order.size();
    cen.resize(3 * m.nF);
    blo.resize(3 * m.nF);
    bhi.resize(3 * m.nF);
    for (uint64_t t : bvh.order) {
        const float* a = m.vtx(t, 0);
        const float* b = m.vtx(t, 1);
        const float* c = m.vtx(t, 2);
        for (int k = 0; k < 3; ++k) {
            float mn = std::min(a[k], std::min(b[k], c[k]));
            float mx = std::max(a[k], std::max(b[k], c[k]));
            blo[3 * t + k] = mn;
            bhi[3 * t + k] = mx;
            cen[3 * t + k] = 0.5f * mn + 0.5f * mx;
        }
    }
    if (n == 0) return;
    struct Task { int64_t node; uint64_t first, count; };
    std::vector<Task> stack;
    bvh.nodes.push_back(CpuNode{});
    stack.push_back({0, 0, n});
    while (!stack.empty()) {
        Task tk = stack.back();
        stack.pop_back();
        CpuNode nd;
        for (int k = 0; k < 3; ++k) { nd.lo[k] = INFINITY; nd.hi[k] = -INFINITY; }
        float clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (uint64_t i = tk.first; i < tk.first + tk.count; ++i) {
            uint64_t t = bvh.order[i];
            for (int k = 0; k < 3; ++k) {
                nd.lo[k] = std::min(nd.lo[k], blo[3 * t + k]);
                nd.hi[k] = std::max(nd.hi[k], bhi[3 * t + k]);
                clo[k] = std::min(clo[k], cen[3 * t + k]);
                chi[k] = std::max(chi[k], cen[3 * t + k]);
            }
        }
        nd.first = tk.first;
        nd.count = tk.count;
        nd.left = nd.right = -1;
        if (tk.count > 4) {
            int axis = 0;
            float ext = chi[0] - clo[0];
            for (int k = 1; k < 3; ++k)
                if (chi[k] - clo[k] > ext) { ext = chi[k] - clo[k]; axis = k; }
            uint64_t mid = tk.first + tk.count / 2;
            std::nth_element(bvh.order.begin() + tk.first, bvh.order.begin() + mid,
                             bvh.order.begin() + tk.first + tk.count,
                             [&](uint64_t x, uint64_t y) {
                                 float cx = cen[3 * x + axis], cy = cen[3 * y + axis];
                                 return cx < cy || (cx == cy && x < y);
                             });
            int64_t li = (int64_t)bvh.nodes.size();
            bvh.nodes.push_back(CpuNode{});
            int64_t ri = (int64_t)bvh.nodes.size();
            bvh.nodes.push_back(CpuNode{});
            nd.left = li;
            nd.right = ri;
            stack.push_back({li, tk.first, mid - tk.first});
            stack.push_back({ri, mid, tk.first + tk.count - mid});
        }
        bvh.nodes[tk.node] = nd;
    }
}

struct Hit { float t; uint64_t tri; };

// All triangles accepted by the hit contract for ray r.
static void collect_hits(const Mesh& m, const CpuBvh* bvh, const Ray& r, std::vector<Hit>& hits) {
    hits.clear();
    float t;
    if (!bvh) {
        for (uint64_t tri = 0; tri < m.nF; ++tri) {
            if (!m.valid(tri)) continue;
            if (hit_triangle(r, m.vtx(tri, 0), m.vtx(tri, 1), m.vtx(tri, 2), t)) hits.push_back({t, tri});
        }
        return;
    }
    if (bvh->nodes.empty()) return;
    int64_t stack[256];
    int sp = 0;
    stack[sp++] = 0;
    while (sp) {
        const CpuNode& nd = bvh->nodes[stack[--sp]];
        float en, ex;
        if (!slab(r, nd.lo, nd.hi, en, ex)) continue;
        if (nd.left < 0) {
            for (uint64_t i = nd.first; i < nd.first + nd.count; ++i) {
                uint64_t tri = bvh->order[i];
                if (hit_triangle(r, m.vtx(tri, 0), m.vtx(tri, 1), m.vtx(tri, 2), t)) hits.push_back({t, tri});
            }
        } else {
            stack[sp++] = nd.left;
            stack[sp++] = nd.right;
        }
    }
}

template <class F>
static void parallel_for(uint64_t n, int nthreads, F fn) {
    if (nthreads <= 1 || n < 64) {
        fn(0, n);
        return;
    }
    std::atomic<uint64_t> next(0);
    const uint64_t chunk = std::max<uint64_t>(64, n / ((uint64_t)nthreads * 16));
    std::vector<std::thread> pool;
    for (int t = 0; t < nthreads; ++t) {
        pool.emplace_back([&]() {
            for (;;) {
                uint64_t b = next.fetch_add(chunk);
                if (b >= n) break;
                fn(b, std::min(n, b + chunk));
            }
        });
    }
    for (auto& th : pool) th.join();
}

static void sort_hits(std::vector<Hit>& hits) {
    std::sort(hits.begin(), hits.end(), [](const Hit& x, const Hit& y) {
        return x.t < y.t || (x.t == y.t && x.tri < y.tri);
    });
}

// Point-in-mesh parity (raytracing.cu:22-77): the loop traces from t_min + 1e-6, counts
// the closest hit and sets t_min = t, at most 10000 times.  On the hits sorted by
// (t, triangle id) that is a greedy walk.  When t + 1e-6 rounds back to t, every
// remaining trace finds that hit again, so the count ends at the cap (10000).
static int32_t pim_one(const Mesh& m, const CpuBvh* bvh, const float p[3], const float d[3], std::vector<Hit>& hits) {
    const float eps = 1e-6f, tmax = 1e16f;
    const uint64_t max_iters = 10000;
    Ray r = make_ray(p, d, eps, tmax);
    collect_hits(m, bvh, r, hits);
    sort_hits(hits);
    float thr = eps;
    uint64_t count = 0, first = 0;
    for (const Hit& h : hits) {
        if (count == max_iters) break;
        if (h.t >= thr && h.t < tmax) {
            if (count == 0) first = h.tri;
            ++count;
            const float nt = h.t + eps;
            if (!(nt > h.t)) count = max_iters;
            thr = nt;
        }
    }
    return (count & 1) ? m.t2o[first] : -1;
}

// Edge-ray hit sequence of trace_edge_multi_hits_edges (mesh_overlap_edges.cu:106-178;
// the same loop in mesh_intersection.cu:16-91 and mesh_overlap.cu:13-70): closest-hit
// traces over [t_min, len + 1e-6], t_min = 1e-6 first and t + 1e-6 after a hit at t
// (t + 2e-4 when the float sum does not exceed t), at most max_hits traces.  next_float:
// the edge check of mesh_containment.cu:99-170, where t_min moves to the next float after
// t.  Takes the sorted hits the traces would return; a step that cannot advance ends the
// walk (the remaining traces return the same hit).
static void edge_walk(const std::vector<Hit>& sorted, int max_hits, int next_float, std::vector<uint64_t>& taken) {
    taken.clear();
    float thr = 1e-6f;
    for (const Hit& h : sorted) {
        if ((int)taken.size() >= max_hits) break;
        if (!(h.t >= thr)) continue;
        taken.push_back(h.tri);
        if (next_float) {
            thr = std::nextafter(h.t, INFINITY);
        } else {
            float nt = h.t + 1e-6f;
            if (!(nt > h.t)) nt = h.t + 2e-4f;
            if (!(nt > h.t)) break;
            thr = nt;
        }
    }
}

static void box_mesh(const Mesh& m, std::vector<float>& bv, std::vector<uint32_t>& bi, std::vector<int32_t>& bo) {
    float mn[3], mx[3];
    for (int k = 0; k < 3; ++k) { mn[k] = 3.40282347e38f; mx[k] = -3.40282347e38f; }
    for (uint64_t v = 0; v < m.nV; ++v)
        for (int k = 0; k < 3; ++k) {
            mn[k] = std::min(mn[k], m.V[3 * v + k]);
            mx[k] = std::max(mx[k], m.V[3 * v + k]);
        }
    const float verts[8][3] = {{mn[0], mn[1], mn[2]}, {mx[0], mn[1], mn[2]}, {mx[0], mx[1], mn[2]},
                               {mn[0], mx[1], mn[2]}, {mn[0], mn[1], mx[2]}, {mx[0], mn[1], mx[2]},
                               {mx[0], mx[1], mx[2]}, {mn[0], mx[1], mx[2]}};
    const uint32_t tris[12][3] = {{0, 2, 1}, {0, 3, 2}, {4, 5, 6}, {4, 6, 7}, {0, 1, 5}, {0, 5, 4},
                                  {3, 6, 2}, {3, 7, 6}, {0, 4, 7}, {0, 7, 3}, {1, 2, 6}, {1, 6, 5}};
    bv.assign(&verts[0][0], &verts[0][0] + 24);
    bi.assign(&tris[0][0], &tris[0][0] + 36);
    bo.assign(12, 0);
}

static int32_t first_triangle_vertex(const Mesh& m, uint64_t tri) { return (int32_t)m.I[3 * tri]; }

}  // namespace

extern "C" {

int orc_pim(const float* V, uint64_t nV, const uint32_t* I, uint64_t nF, const int32_t* tri2obj,
            const float* pts, uint64_t n, float dx, float dy, float dz,
            int32_t* out_obj, int nthreads, int use_bvh) {
    Mesh m{V, nV, I, nF, tri2obj};
    CpuBvh bvh;
    if (use_bvh) build_bvh(m, bvh);
    const float d[3] = {dx, dy, dz};
    parallel_for(n, nthreads, [&](uint64_t b, uint64_t e) {
        std::vector<Hit> hits;
        for (uint64_t i = b; i < e; ++i) out_obj[i] = pim_one(m, use_bvh ? &bvh : nullptr, pts + 3 * i, d, hits);
    });
    return 0;
}

int orc_pim_filtered(const float* V, uint64_t nV, const uint32_t* I, uint64_t nF, const int32_t* tri2obj,
                     const float* pts, uint64_t n, float dx, float dy, float dz,
                     int32_t* out_obj, int nthreads, int use_bvh) {
    Mesh m{V, nV, I, nF, tri2obj};
    std::vector<float> bv;
    std::vector<uint32_t> bi;
    std::vector<int32_t> bo;
    if (nV == 0) {
        for (uint64_t i = 0; i < n; ++i) out_obj[i] = -1;
        return 0;
    }
    box_mesh(m, bv, bi, bo);
    Mesh box{bv.data(), 8, bi.data(), 12, bo.data()};
    CpuBvh bvh;
    if (use_bvh) build_bvh(m, bvh);
    const float d[3] = {dx, dy, dz};
    parallel_for(n, nthreads, [&](uint64_t b, uint64_t e) {
        std::vector<Hit> hits;
        for (uint64_t i = b; i < e; ++i) {
            const float* p = pts + 3 * i;
            if (pim_one(box, nullptr, p, d, hits) < 0) {
                out_obj[i] = -1;
                continue;
            }
            out_obj[i] = pim_one(m, use_bvh ? &bvh : nullptr, p, d, hits);
        }
    });
    return 0;
}

int orc_edge_join(const float* starts, const float* ends, const int32_t* offsets, const int32_t* counts,
                  const int32_t* sources, uint64_t nE,
                  const float* V, uint64_t nV, const uint32_t* I, uint64_t nF, const int32_t* tri2obj,
                  int swap, uint64_t** keys, uint64_t* nkeys, int nthreads, int use_bvh, int max_hits,
                  int next_float) {
    if (max_hits <= 0) max_hits = 100;  // mesh_intersection.cu:25-28
    Mesh m{V, nV, I, nF, tri2obj};
    CpuBvh bvh;
    if (use_bvh) build_bvh(m, bvh);
    int nt = std::max(1, nthreads);
    std::vector<uint64_t> all;
    std::mutex mu;
    parallel_for(nE, nt, [&](uint64_t b, uint64_t e) {
        std::vector<uint64_t> mine, taken;
        std::vector<Hit> hits;
        for (uint64_t i = b; i < e; ++i) {
            const float* s = starts + 3 * i;
            const float* en = ends + 3 * i;
            // mesh_overlap_edges.cu:47-60,116-126
            float dxe = en[0] - s[0], dye = en[1] - s[1], dze = en[2] - s[2];
            float len = std::sqrt((dxe * dxe + dye * dye) + dze * dze);
            if (len < 1e-6f) continue;
            const float d[3] = {dxe / len, dye / len, dze / len};
            Ray r = make_ray(s, d, 1e-6f, len + 1e-6f);
            collect_hits(m, use_bvh ? &bvh : nullptr, r, hits);
            sort_hits(hits);
            edge_walk(hits, max_hits, next_float, taken);
            for (uint64_t tri : taken) {
                uint32_t tgt = (uint32_t)m.t2o[tri];
                for (int32_t k = 0; k < counts[i]; ++k) {
                    uint32_t src = (uint32_t)sources[offsets[i] + k];
                    uint64_t key = swap ? (((uint64_t)tgt << 32) | src) : (((uint64_t)src << 32) | tgt);
                    mine.push_back(key);
                }
            }
        }
        std::sort(mine.begin(), mine.end());
        mine.erase(std::unique(mine.begin(), mine.end()), mine.end());
        std::lock_guard<std::mutex> g(mu);
        all.insert(all.end(), mine.begin(), mine.end());
    });
    std::sort(all.begin(), all.end());
    all.erase(std::unique(all.begin(), all.end()), all.end());
    *nkeys = all.size();
    *keys = (uint64_t*)std::malloc(sizeof(uint64_t) * (all.size() ? all.size() : 1));
    if (!all.empty()) std::memcpy(*keys, all.data(), sizeof(uint64_t) * all.size());
    return 0;
}

// Every crossing of the segment start -> end with t in [1e-6, len + 1e-6], testing every
// triangle (no BVH), unsorted: the hits a trace of mesh_overlap_edges.cu:135-145 chooses
// from.  Writes up to cap of them; *n receives the total.
int orc_segment_hits(const float* start, const float* end, const float* V, uint64_t nV, const uint32_t* I,
                     uint64_t nF, const int32_t* tri2obj, float* out_t, uint64_t* out_tri, uint64_t cap,
                     uint64_t* n) {
    Mesh m{V, nV, I, nF, tri2obj};
    float dxe = end[0] - start[0], dye = end[1] - start[1], dze = end[2] - start[2];
    float len = std::sqrt((dxe * dxe + dye * dye) + dze * dze);
    *n = 0;
    if (len < 1e-6f) return 0;
    const float d[3] = {dxe / len, dye / len, dze / len};
    Ray r = make_ray(start, d, 1e-6f, len + 1e-6f);
    std::vector<Hit> hits;
    collect_hits(m, nullptr, r, hits);
    *n = hits.size();
    for (uint64_t k = 0; k < hits.size() && k < cap; ++k) {
        out_t[k] = hits[k].t;
        out_tri[k] = hits[k].tri;
    }
    return 0;
}

// Per-source diagnostics of the tracked containment (PairHitTracking.h:31-150):
// candidates[o] = distinct target objects the ray crossed; odd-parity targets with the
// number of their triangles the ray crossed.
struct ContainDiag {
    std::vector<uint32_t> candidates;
    std::vector<std::vector<std::pair<uint32_t, uint32_t>>> odd;  // (target, hits) per source
};

static void containment_run(const float* srcV, uint64_t srcNV, const uint32_t* srcI, uint64_t srcNF,
                            const int32_t* srcT2O, const float* V, uint64_t nV, const uint32_t* I, uint64_t nF,
                            const int32_t* tri2obj, int swap, std::vector<uint64_t>& all, ContainDiag* diag,
                            int nthreads, int use_bvh) {
    Mesh src{srcV, srcNV, srcI, srcNF, srcT2O};
    Mesh m{V, nV, I, nF, tri2obj};
    // raytracer_intersection_estimated_main.cpp:539-552: lowest triangle index per object.
    int32_t maxObj = -1;
    for (uint64_t t = 0; t < srcNF; ++t) maxObj = std::max(maxObj, srcT2O[t]);
    uint64_t nObj = (uint64_t)(maxObj + 1);
    std::vector<int64_t> firstTri(nObj, -1);
    for (uint64_t t = 0; t < srcNF; ++t) {
        int32_t o = srcT2O[t];
        if (o >= 0 && firstTri[o] < 0) firstTri[o] = (int64_t)t;
    }
    CpuBvh bvh;
    if (use_bvh) build_bvh(m, bvh);
    std::vector<std::vector<uint64_t>> perObj(nObj);
    if (diag) {
        diag->candidates.assign(nObj, 0);
        diag->odd.assign(nObj, {});
    }
    parallel_for(nObj, nthreads, [&](uint64_t b, uint64_t e) {
        std::vector<Hit> hits;
        std::vector<uint32_t> tg;
        for (uint64_t o = b; o < e; ++o) {
            if (firstTri[o] < 0) continue;
            uint32_t vi = (uint32_t)first_triangle_vertex(src, (uint64_t)firstTri[o]);
            if (vi >= srcNV) continue;
            const float* q = srcV + 3 * (uint64_t)vi;
            const float d[3] = {0.0f, 0.0f, 1.0f};
            Ray r = make_ray(q, d, 1e-4f, 1e10f);  // mesh_intersection_anyhit.cu:92-106
            collect_hits(m, use_bvh ? &bvh : nullptr, r, hits);
            tg.clear();
            for (const Hit& h : hits) tg.push_back((uint32_t)m.t2o[h.tri]);
            std::sort(tg.begin(), tg.end());
            for (size_t i = 0; i < tg.size();) {
                size_t j = i;
                while (j < tg.size() && tg[j] == tg[i]) ++j;
                if (diag) ++diag->candidates[o];
                if ((j - i) & 1) {
                    uint64_t key = swap ? (((uint64_t)tg[i] << 32) | (uint32_t)o) : (((uint64_t)o << 32) | tg[i]);
                    perObj[o].push_back(key);
                    if (diag) diag->odd[o].push_back({tg[i], (uint32_t)(j - i)});
                }
                i = j;
            }
        }
    });
    all.clear();
    for (auto& v : perObj) all.insert(all.end(), v.begin(), v.end());
    std::sort(all.begin(), all.end());
    all.erase(std::unique(all.begin(), all.end()), all.end());
}

static void give_keys(const std::vector<uint64_t>& all, uint64_t** keys, uint64_t* nkeys) {
    *nkeys = all.size();
    *keys = (uint64_t*)std::malloc(sizeof(uint64_t) * (all.size() ? all.size() : 1));
    if (!all.empty()) std::memcpy(*keys, all.data(), sizeof(uint64_t) * all.size());
}

int orc_containment(const float* srcV, uint64_t srcNV, const uint32_t* srcI, uint64_t srcNF, const int32_t* srcT2O,
                    const float* V, uint64_t nV, const uint32_t* I, uint64_t nF, const int32_t* tri2obj,
                    int swap, uint64_t** keys, uint64_t* nkeys, int nthreads, int use_bvh) {
    std::vector<uint64_t> all;
    containment_run(srcV, srcNV, srcI, srcNF, srcT2O, V, nV, I, nF, tri2obj, swap, all, nullptr, nthreads, use_bvh);
    give_keys(all, keys, nkeys);
    return 0;
}

int orc_containment_diag(const float* srcV, uint64_t srcNV, const uint32_t* srcI, uint64_t srcNF,
                         const int32_t* srcT2O, const float* V, uint64_t nV, const uint32_t* I, uint64_t nF,
                         const int32_t* tri2obj, uint32_t* out_candidates, uint64_t capacity,
                         uint64_t** odd_keys, uint32_t** odd_hits, uint64_t* n_odd, int nthreads) {
    std::vector<uint64_t> all;
    ContainDiag dg;
    containment_run(srcV, srcNV, srcI, srcNF, srcT2O, V, nV, I, nF, tri2obj, 0, all, &dg, nthreads, 1);
    if (dg.candidates.size() > capacity) return 1;
    std::copy(dg.candidates.begin(), dg.candidates.end(), out_candidates);
    std::vector<std::pair<uint64_t, uint32_t>> flat;
    for (uint64_t o = 0; o < dg.odd.size(); ++o)
        for (auto& th : dg.odd[o]) flat.push_back({(o << 32) | th.first, th.second});
    std::sort(flat.begin(), flat.end());
    *n_odd = flat.size();
    *odd_keys = (uint64_t*)std::malloc(sizeof(uint64_t) * (flat.size() ? flat.size() : 1));
    *odd_hits = (uint32_t*)std::malloc(sizeof(uint32_t) * (flat.size() ? flat.size() : 1));
    for (size_t i = 0; i < flat.size(); ++i) {
        (*odd_keys)[i] = flat[i].first;
        (*odd_hits)[i] = flat[i].second;
    }
    return 0;
}

struct GridCellC { uint32_t center, touch; float avg, ratio; };

double orc_estimate_raw(const void* cellsA, const void* cellsB, uint64_t ncells,
                        float cellVolume, float epsilon, float gamma) {
    const GridCellC* A = (const GridCellC*)cellsA;
    const GridCellC* B = (const GridCellC*)cellsB;
    double sum = 0.0;
    for (uint64_t i = 0; i < ncells; ++i) {
        // estimated_overlap.cu:20-40
        if (A[i].touch == 0 || B[i].touch == 0) continue;
        float cs = A[i].avg + B[i].avg + epsilon;
        float mv = cs * cs * cs;
        float prob = mv / cellVolume;
        float ratio = std::sqrt(A[i].ratio * B[i].ratio);
        float corr = std::pow(ratio, gamma);
        prob *= corr;
        prob = std::fmin(prob, 1.0f);
        sum += (double)((float)A[i].touch * (float)B[i].touch * prob);
    }
    return sum;
}

static void global_means(const GridCellC* c, uint64_t n, float& size, float& ratio) {
    // raytracer_overlap_estimated_main.cpp:129-158
    double ts = 0.0, tr = 0.0;
    long long cnt = 0;
    for (uint64_t i = 0; i < n; ++i) {
        if (c[i].touch > 0) {
            ts += (double)c[i].avg * (double)c[i].touch;
            tr += (double)c[i].ratio * (double)c[i].touch;
            cnt += c[i].touch;
        }
    }
    size = cnt ? (float)(ts / cnt) : 0.0f;
    ratio = cnt ? (float)(tr / cnt) : 1.0f;
}

int64_t orc_estimate_pairs(const void* cellsA, const void* cellsB, uint64_t ncells,
                           const float minA[3], const float maxA[3], const uint32_t resA[3],
                           float epsilon, float gamma, int alpha_correction, double* raw_out) {
    float w = maxA[0] - minA[0], h = maxA[1] - minA[1], dpt = maxA[2] - minA[2];
    float csX = w / resA[0], csY = h / resA[1], csZ = dpt / resA[2];
    float cellVolume = csX * csY * csZ;
    double raw = orc_estimate_raw(cellsA, cellsB, ncells, cellVolume, epsilon, gamma);
    if (raw_out) *raw_out = raw;
    float rawf = (float)raw;
    float alpha = 1.0f;
    if (alpha_correction) {
        float s1, r1, s2, r2;
        global_means((const GridCellC*)cellsA, ncells, s1, r1);
        global_means((const GridCellC*)cellsB, ncells, s2, r2);
        float e1 = s1 * std::cbrt(r1), e2 = s2 * std::cbrt(r2);
        float cs = e1 + e2;
        float mv = cs * cs * cs;
        if (cellVolume < 1e-9f) cellVolume = 1e-9f;
        alpha = mv / cellVolume;
        if (alpha < 1.0f) alpha = 1.0f;
    }
    return (int64_t)(rawf / alpha);
}

int orc_orient(const float d[3], const float o[3], const float a[3], const float b[3]) { return orient(d, o, a, b); }

int orc_perturbed_sign(const float d[3], const float o[3], const float a[3], const float b[3]) {
    int kx, ky;
    perturb_axes(d, kx, ky);
    return perturbed_sign(d, o, a, b, kx, ky);
}

void orc_box_mesh(const float* V, uint64_t nV, float* out_v, uint32_t* out_i) {
    Mesh m{V, nV, nullptr, 0, nullptr};
    std::vector<float> bv;
    std::vector<uint32_t> bi;
    std::vector<int32_t> bo;
    box_mesh(m, bv, bi, bo);
    std::memcpy(out_v, bv.data(), 24 * sizeof(float));
    std::memcpy(out_i, bi.data(), 36 * sizeof(uint32_t));
}

// ---------------------------------------------------------------------------
// Preprocessing payloads.
// ---------------------------------------------------------------------------
int orc_extract_edges(const float* V, uint64_t nV, const uint32_t* I, uint64_t nF, const int32_t* T,
                      float** starts, float** ends, int32_t** offsets, int32_t** counts, int32_t** sources,
                      uint64_t* nE, uint64_t* nS) {
    using Q = std::array<long long, 3>;
    struct Info {
        uint32_t a, b;              // vertex ids of the first occurrence, in its orientation
        std::vector<int32_t> objs;  // distinct, first-seen order
    };
    auto quant = [&](uint32_t v) {
        Q q;
        for (int k = 0; k < 3; ++k) q[k] = std::llround((double)V[3 * (uint64_t)v + k] * 1e5);
        return q;
    };
    std::map<std::pair<Q, Q>, Info> edges;
    for (uint64_t t = 0; t < nF; ++t) {
        const uint32_t v[3] = {I[3 * t], I[3 * t + 1], I[3 * t + 2]};
        if (v[0] >= nV || v[1] >= nV || v[2] >= nV) continue;
        for (int e = 0; e < 3; ++e) {
            const uint32_t a = v[e], b = v[(e + 1) % 3];
            Q qa = quant(a), qb = quant(b);
            if (qb < qa) std::swap(qa, qb);
            auto ins = edges.try_emplace({qa, qb});
            Info& info = ins.first->second;
            if (ins.second) {
                info.a = a;
                info.b = b;
            }
            if (std::find(info.objs.begin(), info.objs.end(), T[t]) == info.objs.end()) info.objs.push_back(T[t]);
        }
    }
    const uint64_t ne = edges.size();
    uint64_t ns = 0;
    for (const auto& kv : edges) ns += kv.second.objs.size();
    *starts = (float*)std::malloc(std::max<uint64_t>(ne, 1) * 3 * sizeof(float));
    *ends = (float*)std::malloc(std::max<uint64_t>(ne, 1) * 3 * sizeof(float));
    *offsets = (int32_t*)std::malloc(std::max<uint64_t>(ne, 1) * sizeof(int32_t));
    *counts = (int32_t*)std::malloc(std::max<uint64_t>(ne, 1) * sizeof(int32_t));
    *sources = (int32_t*)std::malloc(std::max<uint64_t>(ns, 1) * sizeof(int32_t));
    uint64_t i = 0, j = 0;
    for (const auto& kv : edges) {
        const Info& info = kv.second;
        for (int k = 0; k < 3; ++k) {
            (*starts)[3 * i + k] = V[3 * (uint64_t)info.a + k];
            (*ends)[3 * i + k] = V[3 * (uint64_t)info.b + k];
        }
        (*offsets)[i] = (int32_t)j;
        (*counts)[i] = (int32_t)info.objs.size();
        for (int32_t o : info.objs) (*sources)[j++] = o;
        ++i;
    }
    *nE = ne;
    *nS = ns;
    return 0;
}

void orc_grid_stats(const float* V, uint64_t nV, const uint32_t* I, uint64_t nF, const int32_t* T, int res,
                    float world_size, void* cells_out, float* bounds6) {
    struct Cell {
        uint32_t center, touch;
        float avg, ratio;
    };
    struct Obj {
        float mn[3] = {1e30f, 1e30f, 1e30f}, mx[3] = {-1e30f, -1e30f, -1e30f};
        double vol = 0.0;
    };
    float lo[3] = {1e30f, 1e30f, 1e30f}, hi[3] = {-1e30f, -1e30f, -1e30f};
    for (uint64_t v = 0; v < nV; ++v)
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::min(lo[k], V[3 * v + k]);
            hi[k] = std::max(hi[k], V[3 * v + k]);
        }
    if (world_size > 0) {
        for (int k = 0; k < 3; ++k) {
            lo[k] = 0.0f;
            hi[k] = world_size;
        }
    }
    float cs[3];
    for (int k = 0; k < 3; ++k) {
        cs[k] = (hi[k] - lo[k]) / (float)res;
        bounds6[k] = lo[k];
        bounds6[3 + k] = hi[k];
    }
    const uint64_t ncell = (uint64_t)res * res * res;
    Cell* cells = static_cast<Cell*>(cells_out);
    std::memset(cells, 0, ncell * sizeof(Cell));
    auto valid = [&](uint64_t t) { return I[3 * t] < nV && I[3 * t + 1] < nV && I[3 * t + 2] < nV; };
    std::unordered_map<int, Obj> objs;
    for (uint64_t t = 0; t < nF; ++t) {
        if (!valid(t)) continue;
        Obj& o = objs[T[t]];
        for (int c = 0; c < 3; ++c)
            for (int k = 0; k < 3; ++k) {
                const float x = V[3 * (uint64_t)I[3 * t + c] + k];
                o.mn[k] = std::min(o.mn[k], x);
                o.mx[k] = std::max(o.mx[k], x);
            }
    }
    for (uint64_t t = 0; t < nF; ++t) {
        if (!valid(t)) continue;
        Obj& o = objs[T[t]];
        float p[3][3];
        for (int c = 0; c < 3; ++c)
            for (int k = 0; k < 3; ++k) p[c][k] = V[3 * (uint64_t)I[3 * t + c] + k] - (o.mn[k] + o.mx[k]) * 0.5f;
        const float cx = p[0][1] * p[1][2] - p[0][2] * p[1][1];
        const float cy = p[0][2] * p[1][0] - p[0][0] * p[1][2];
        const float cz = p[0][0] * p[1][1] - p[0][1] * p[1][0];
        const float term = cx * p[2][0] + cy * p[2][1] + cz * p[2][2];
        o.vol += term;
    }
    for (const auto& kv : objs) {
        const Obj& o = kv.second;
        const float w = o.mx[0] - o.mn[0], h = o.mx[1] - o.mn[1], d = o.mx[2] - o.mn[2];
        float box = w * h * d;
        if (box < 1e-9f) box = 1e-9f;
        float ratio = (std::fabs((float)o.vol) / 6.0f) / box;
        if (ratio > 1.0f) ratio = 1.0f;
        const float avg = (w + h + d) / 3.0f;
        int a[3], c0[3], c1[3];
        for (int k = 0; k < 3; ++k) {
            a[k] = (int)(((o.mn[k] + o.mx[k]) * 0.5f - lo[k]) / cs[k]);
            c0[k] = std::max(0, (int)((o.mn[k] - lo[k]) / cs[k]));
            c1[k] = std::min(res - 1, (int)((o.mx[k] - lo[k] - 1e-5f) / cs[k]));
        }
        if (a[0] >= 0 && a[0] < res && a[1] >= 0 && a[1] < res && a[2] >= 0 && a[2] < res)
            cells[((uint64_t)a[2] * res + a[1]) * res + a[0]].center++;
        for (int z = c0[2]; z <= c1[2]; ++z)
            for (int y = c0[1]; y <= c1[1]; ++y)
                for (int x = c0[0]; x <= c1[0]; ++x) {
                    Cell& c = cells[((uint64_t)z * res + y) * res + x];
                    c.touch++;
                    c.avg += avg;
                    c.ratio += ratio;
                }
    }
    for (uint64_t i = 0; i < ncell; ++i)
        if (cells[i].touch) {
            cells[i].avg /= (float)cells[i].touch;
            cells[i].ratio /= (float)cells[i].touch;
        }
}

void orc_free(void* p) { std::free(p); }

}  // extern "C"
