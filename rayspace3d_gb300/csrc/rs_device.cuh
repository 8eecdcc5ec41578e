// rs_device.cuh -- device-side geometry of the engine's hit contract.
//
// The reference traces rays with OptiX (query/src/cuda/raytracing.cu:34-46,
// mesh_overlap_edges.cu:135-145, mesh_intersection_anyhit.cu:92-106), whose
// ray/triangle test is closed.  The engine instead fixes an exact contract:
//
//  * a triangle is crossed when the ray origin, perturbed symbolically by
//    delta*e_kx + delta^2*e_ky (kx, ky = the two axes other than the dominant
//    axis of d), lies strictly inside the triangle's projection along d.  The
//    three edge signs are exact: an FP32 evaluation with a static forward-error
//    bound decides almost every case, and the rest are re-evaluated exactly as a
//    sum of 36 FP64 triple products (each product of three floats is exactly a
//    two-term FP64 expansion) accumulated into a non-overlapping expansion;
//  * the hit distance is a fixed sequence of individually rounded float
//    operations (no contraction), clamped to the slab interval of the
//    triangle's own box, and accepted when it lies in [tmin, tmax];
//  * box tests use the same slab formula, which is monotone in the box bounds,
//    so BVH culling never changes the hit set.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace rs {

// ---------------------------------------------------------------------------
// Status bits raised by kernels (OR-ed into a device word).
// ---------------------------------------------------------------------------
enum : uint32_t {
    ST_TABLE_FULL = 1u << 0,     // a pair key found no free slot within the probe limit
    ST_HIT_OVERFLOW = 1u << 1,   // a per-ray hit list overflowed (handled by a fallback pass)
    ST_STACK_OVERFLOW = 1u << 2, // a traversal stack overflowed (result invalid)
    ST_ITER_LIMIT = 1u << 3,     // an iteration budget ran out (result invalid)
    ST_TARGET_OVERFLOW = 1u << 4, // reserved (containment handles any number of targets in passes)
    ST_SPILLED = 1u << 5         // the table passed 3/4 load or a key found no slot within the
                                 // probe limit; later keys may sit in the overflow table (none
                                 // lost): the table must be regrown from both
};

// ---------------------------------------------------------------------------
// Recheck statistics, one copy per translation unit: [0] edge signs that the FP32
// filter could not decide (always counted: the exact path is rare), [1] triangle
// tests (counted while g_recheck_on is set, one warp-aggregated atomic per thread).
// ---------------------------------------------------------------------------
static __device__ unsigned long long g_recheck[2];
static __device__ int g_recheck_on;

__device__ __forceinline__ void note_exact() { atomicAdd(&g_recheck[0], 1ull); }

__device__ __forceinline__ void add_tests(unsigned int n) {
    if (!__ldcg(&g_recheck_on)) return;
    const unsigned int mask = __activemask();
    const unsigned int sum = __reduce_add_sync(mask, n);
    if ((int)(threadIdx.x & 31) == __ffs(mask) - 1) atomicAdd(&g_recheck[1], (unsigned long long)sum);
}

// Host side: op 0 = disable, 1 = enable, 2 = reset, 3 = read into out[2] (adds).
static inline int recheck_op(int op, unsigned long long* out) {
    if (op == 0 || op == 1) {
        const int v = op;
        return (int)cudaMemcpyToSymbol(g_recheck_on, &v, sizeof(v));
    }
    if (op == 2) {
        const unsigned long long z[2] = {0, 0};
        return (int)cudaMemcpyToSymbol(g_recheck, z, sizeof(z));
    }
    unsigned long long v[2] = {0, 0};
    const cudaError_t e = cudaMemcpyFromSymbol(v, g_recheck, sizeof(v));
    if (e == cudaSuccess && out) {
        out[0] += v[0];
        out[1] += v[1];
    }
    return (int)e;
}

// ---------------------------------------------------------------------------
// Exact FP64 building blocks (Knuth two-sum, FMA two-product, Shewchuk
// grow-expansion).  Intrinsics keep the compiler from re-associating them.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double two_sum(double a, double b, double& err) {
    double s = __dadd_rn(a, b);
    double bb = __dsub_rn(s, a);
    double aa = __dsub_rn(s, bb);
    err = __dadd_rn(__dsub_rn(a, aa), __dsub_rn(b, bb));
    return s;
}

__device__ __forceinline__ double two_prod(double a, double b, double& err) {
    double p = __dmul_rn(a, b);
    err = __fma_rn(a, b, -p);
    return p;
}

// Adds b into the non-overlapping expansion e[0..m) (increasing magnitude),
// dropping zero components.  Returns the new length (<= m+1).
__device__ __forceinline__ int grow_expansion(double* e, int m, double b) {
    double q = b;
    int k = 0;
    for (int i = 0; i < m; ++i) {
        double h;
        q = two_sum(q, e[i], h);
        if (h != 0.0) e[k++] = h;
    }
    if (q != 0.0) e[k++] = q;
    return k;
}

__device__ __forceinline__ int expansion_sign(const double* e, int m) {
    if (m == 0) return 0;
    double top = e[m - 1];
    return top > 0.0 ? 1 : (top < 0.0 ? -1 : 0);
}

// Exact sign of det[d, a-o, b-o] = d . (a x b + b x o + o x a).  Operands are passed
// by value so callers never have to keep them addressable in local memory.
static __device__ __noinline__ int orient_exact(float d0, float d1, float d2, float o0, float o1, float o2,
                                                float a0, float a1, float a2, float b0, float b1, float b2) {
    note_exact();
    // a == o, b == o or a == b makes a-o, b-o dependent: the determinant is exactly zero
    // (points snapped onto mesh vertices hit this for every incident edge).
    if ((a0 == o0 && a1 == o1 && a2 == o2) || (b0 == o0 && b1 == o1 && b2 == o2) ||
        (a0 == b0 && a1 == b1 && a2 == b2))
        return 0;
    const float d[3] = {d0, d1, d2}, o[3] = {o0, o1, o2}, a[3] = {a0, a1, a2}, b[3] = {b0, b1, b2};
    const float* X[3] = {a, b, o};
    const float* Y[3] = {b, o, a};
    // FP64 filter: each of the 36 terms d_k * (X_i Y_j) has an exact float-by-float product
    // and one rounding (relative 2^-53), the sum of 36 terms 35 more, so
    // |sum - det| <= 36 * 2^-53 * sum|terms| (1 + 2^-50); 40 * 2^-53 is used.
    {
        double sum = 0.0, mag = 0.0;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const int i = (k + 1) % 3, j = (k + 2) % 3;
            const double dk = (double)d[k];
#pragma unroll
            for (int s = 0; s < 3; ++s) {
                const double p = __dmul_rn(dk, __dmul_rn((double)X[s][i], (double)Y[s][j]));
                const double q = __dmul_rn(dk, __dmul_rn((double)X[s][j], (double)Y[s][i]));
                sum = __dadd_rn(sum, __dsub_rn(p, q));
                mag = __dadd_rn(mag, __dadd_rn(fabs(p), fabs(q)));
            }
        }
        // Products of floats neither underflow nor overflow in FP64; mag == 0 means every
        // term, hence the determinant, is exactly zero.
        if (mag == 0.0) return 0;
        const double bound = __dmul_rn(mag, 40.0 * 1.1102230246251565e-16);
        if (sum > bound) return 1;
        if (sum < -bound) return -1;
    }
    double e[40];
    int m = 0;
#pragma unroll 1
    for (int k = 0; k < 3; ++k) {
        if (d[k] == 0.0f) continue;
        const int i = (k + 1) % 3, j = (k + 2) % 3;
        const double dk = (double)d[k];
#pragma unroll 1
        for (int s = 0; s < 3; ++s) {
            double p = __dmul_rn((double)X[s][i], (double)Y[s][j]);  // exact: 48-bit product
            double q = __dmul_rn((double)X[s][j], (double)Y[s][i]);
            double lo;
            double hi = two_prod(dk, p, lo);
            m = grow_expansion(e, m, hi);
            m = grow_expansion(e, m, lo);
            hi = two_prod(dk, -q, lo);
            m = grow_expansion(e, m, hi);
            m = grow_expansion(e, m, lo);
        }
    }
    return expansion_sign(e, m);
}

// Exact sign of det[d, e_k, b-a] = d_j (b_i - a_i) - d_i (b_j - a_j), i = k+1, j = k+2 (mod 3).
// Components are picked with selects so no operand array is indexed by a variable.
static __device__ __noinline__ int axis_det_exact(int k, float d0, float d1, float d2, float a0, float a1, float a2,
                                                  float b0, float b1, float b2) {
    note_exact();
    const float di = k == 0 ? d1 : (k == 1 ? d2 : d0), dj = k == 0 ? d2 : (k == 1 ? d0 : d1);
    const float ai = k == 0 ? a1 : (k == 1 ? a2 : a0), aj = k == 0 ? a2 : (k == 1 ? a0 : a1);
    const float bi = k == 0 ? b1 : (k == 1 ? b2 : b0), bj = k == 0 ? b2 : (k == 1 ? b0 : b1);
    double e[5];
    int m = 0;
    m = grow_expansion(e, m, __dmul_rn((double)dj, (double)bi));
    m = grow_expansion(e, m, -__dmul_rn((double)dj, (double)ai));
    m = grow_expansion(e, m, -__dmul_rn((double)di, (double)bj));
    m = grow_expansion(e, m, __dmul_rn((double)di, (double)aj));
    return expansion_sign(e, m);
}

// Adds b into the expansion e[0..M) of exactly M components (zeros kept), giving M+1
// components; with compile-time M every index is static, so e stays in registers.
template <int M>
__device__ __forceinline__ void grow_fixed(double* e, double b) {
    double q = b;
#pragma unroll
    for (int i = 0; i < M; ++i) {
        double h;
        q = two_sum(q, e[i], h);
        e[i] = h;
    }
    e[M] = q;
}

// The same in FP32 (Knuth two-sum in float), for the float expansion below.
__device__ __forceinline__ float two_sum_f(float a, float b, float& err) {
    float s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    float aa = __fsub_rn(s, bb);
    err = __fadd_rn(__fsub_rn(a, aa), __fsub_rn(b, bb));
    return s;
}

template <int M>
__device__ __forceinline__ void grow_fixed_f(float* e, float b) {
    float q = b;
#pragma unroll
    for (int i = 0; i < M; ++i) {
        float h;
        q = two_sum_f(q, e[i], h);
        e[i] = h;
    }
    e[M] = q;
}

// Exact sign of A_i B_j - A_j B_i with A = a - o, B = b - o (the determinant for a ray
// along +e_AXIS), expanded into six products of input coordinates:
//   a_i b_j - a_j b_i - a_i o_j + a_j o_i - o_i b_j + o_j b_i.
// Coincident or axis-parallel collinear inputs are exact zeros without arithmetic.
// When every nonzero coordinate lies in [2^-50, 2^50], each product is exactly the sum
// of two floats (FMA two-product: no overflow, and the error term is a multiple of
// 2^-146, above the subnormal spacing), and the twelve parts are summed exactly as a
// float expansion (Shewchuk grow-expansion, zeros kept, registers only): FP32 throughput
// on this part is many times its FP64 throughput.  Otherwise each product is exact in
// FP64 and the six are summed as an FP64 expansion.
__device__ __forceinline__ bool in_f32_range(float x) {
    const float ax = fabsf(x);
    return ax == 0.0f || (ax >= 8.881784197001252e-16f && ax <= 1.125899906842624e15f);
}

static __device__ __noinline__ int orient2_exact(float ai, float aj, float bi, float bj, float oi, float oj) {
    note_exact();
    if ((ai == oi && aj == oj) || (bi == oi && bj == oj) || (ai == bi && aj == bj) || (ai == oi && bi == oi) ||
        (aj == oj && bj == oj))
        return 0;
    if (in_f32_range(ai) && in_f32_range(aj) && in_f32_range(bi) && in_f32_range(bj) && in_f32_range(oi) &&
        in_f32_range(oj)) {
        const float x[6] = {ai, -aj, -ai, aj, -oi, oj};
        const float y[6] = {bj, bi, oj, oi, bj, bi};
        float e[12];
        e[0] = __fmul_rn(x[0], y[0]);
        grow_fixed_f<1>(e, __fmaf_rn(x[0], y[0], -e[0]));
#define RS_TWO_PROD_GROW(K, M)                                   \
    {                                                            \
        const float p = __fmul_rn(x[K], y[K]);                   \
        grow_fixed_f<M>(e, p);                                   \
        grow_fixed_f<M + 1>(e, __fmaf_rn(x[K], y[K], -p));       \
    }
        RS_TWO_PROD_GROW(1, 2)
        RS_TWO_PROD_GROW(2, 4)
        RS_TWO_PROD_GROW(3, 6)
        RS_TWO_PROD_GROW(4, 8)
        RS_TWO_PROD_GROW(5, 10)
#undef RS_TWO_PROD_GROW
#pragma unroll
        for (int i = 11; i >= 0; --i)
            if (e[i] != 0.0f) return e[i] > 0.0f ? 1 : -1;
        return 0;
    }
    double e[6];
    e[0] = __dmul_rn((double)ai, (double)bj);
    grow_fixed<1>(e, -__dmul_rn((double)aj, (double)bi));
    grow_fixed<2>(e, -__dmul_rn((double)ai, (double)oj));
    grow_fixed<3>(e, __dmul_rn((double)aj, (double)oi));
    grow_fixed<4>(e, -__dmul_rn((double)oi, (double)bj));
    grow_fixed<5>(e, __dmul_rn((double)oj, (double)bi));
#pragma unroll
    for (int i = 5; i >= 0; --i)
        if (e[i] != 0.0) return e[i] > 0.0 ? 1 : -1;
    return 0;
}

// FP32 filter for det[d, a-o, b-o].  Roundings on any elementary product are at
// most 7 (two input differences, product, difference, scale by d, two sums), so
// |computed - exact| <= 7.01u * M with u = 2^-24 and M the float magnitude sum;
// 12u is used.  Tiny or non-finite magnitudes go to the exact path.
template <int AXIS>
__device__ __forceinline__ int orient_sign(const float* d, const float* o, const float* a, const float* b) {
    float A[3], B[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        A[k] = __fsub_rn(a[k], o[k]);
        B[k] = __fsub_rn(b[k], o[k]);
    }
    float det, mag;
    if (AXIS >= 0) {
        // d = +e_AXIS: det = A_i B_j - A_j B_i with i = AXIS+1, j = AXIS+2 (mod 3).
        const int i = (AXIS + 1) % 3, j = (AXIS + 2) % 3;
        float p = __fmul_rn(A[i], B[j]), q = __fmul_rn(A[j], B[i]);
        det = __fsub_rn(p, q);
        mag = __fadd_rn(fabsf(p), fabsf(q));
    } else {
        det = 0.0f;
        mag = 0.0f;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const int i = (k + 1) % 3, j = (k + 2) % 3;
            float p = __fmul_rn(A[i], B[j]), q = __fmul_rn(A[j], B[i]);
            float c = __fsub_rn(p, q);
            det = __fadd_rn(det, __fmul_rn(d[k], c));
            mag = __fadd_rn(mag, __fmul_rn(fabsf(d[k]), __fadd_rn(fabsf(p), fabsf(q))));
        }
    }
    const float bound = __fmul_rn(mag, 12.0f * 5.9604644775390625e-08f);
    if (mag > 7.888609052210118e-31f && mag < 3.0e38f) {  // 2^-100 < M < overflow
        if (det > bound) return 1;
        if (det < -bound) return -1;
    }
    if (AXIS >= 0) {
        const int i = (AXIS + 1) % 3, j = (AXIS + 2) % 3;
        return orient2_exact(a[i], a[j], b[i], b[j], o[i], o[j]);
    }
    return orient_exact(d[0], d[1], d[2], o[0], o[1], o[2], a[0], a[1], a[2], b[0], b[1], b[2]);
}

// Perturbation axes of a direction: kz = the dominant axis of d (ties keep z, then x),
// kx = kz+1, ky = kz+2 (mod 3).  Written without indexing d by a variable.
__device__ __forceinline__ void perturb_axes(const float* d, int& kx, int& ky) {
    const float ax = fabsf(d[0]), ay = fabsf(d[1]), az = fabsf(d[2]);
    int kz = 2;
    float best = az;
    if (ax > best) { kz = 0; best = ax; }
    if (ay > best) kz = 1;
    kx = kz == 2 ? 0 : kz + 1;
    ky = kz == 0 ? 2 : (kz == 1 ? 0 : 1);
}

// Edge sign of (a,b) for the perturbed origin (see file header).
template <int AXIS>
__device__ __forceinline__ int perturbed_sign(const float* d, const float* o, const float* a, const float* b) {
    int s = orient_sign<AXIS>(d, o, a, b);
    if (s) return s;
    if (AXIS >= 0) {
        // d = +e_AXIS, kx = AXIS+1, ky = AXIS+2 (mod 3):
        // det[d,e_kx,b-a] = b_ky - a_ky and det[d,e_ky,b-a] = -(b_kx - a_kx), so the
        // perturbation terms are -(b_ky - a_ky) and then +(b_kx - a_kx).
        const int kxa = (AXIS + 1) % 3, kya = (AXIS + 2) % 3;
        if (b[kya] != a[kya]) return b[kya] > a[kya] ? -1 : 1;
        if (b[kxa] != a[kxa]) return b[kxa] > a[kxa] ? 1 : -1;
        return 0;
    }
    int kx, ky;
    perturb_axes(d, kx, ky);
    s = -axis_det_exact(kx, d[0], d[1], d[2], a[0], a[1], a[2], b[0], b[1], b[2]);
    if (s) return s;
    return -axis_det_exact(ky, d[0], d[1], d[2], a[0], a[1], a[2], b[0], b[1], b[2]);
}

// ---------------------------------------------------------------------------
// Rays and the slab rule.
// ---------------------------------------------------------------------------
// A ray: origin, direction, 1/direction per axis (0 for an axis the direction does not
// move along: d == 0, or 1/d overflows), and the accepted t range.
struct Ray {
    float o[3], d[3], inv[3];
    float tmin, tmax;
};

__device__ __forceinline__ Ray make_ray(float ox, float oy, float oz, float dx, float dy, float dz,
                                        float tmin, float tmax) {
    Ray r;
    r.o[0] = ox; r.o[1] = oy; r.o[2] = oz;
    r.d[0] = dx; r.d[1] = dy; r.d[2] = dz;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        r.inv[k] = 0.0f;
        if (r.d[k] != 0.0f) {
            const float inv = __fdiv_rn(1.0f, r.d[k]);
            if (!isinf(inv)) r.inv[k] = inv;
        }
    }
    r.tmin = tmin;
    r.tmax = tmax;
    return r;
}

// Slab interval of [lo,hi] intersected with [en,ex].  For AXIS >= 0 the ray is
// +e_AXIS and the two other axes reduce to exact containment tests.
template <int AXIS>
__device__ __forceinline__ bool slab(const Ray& r, const float* lo, const float* hi, float en, float ex,
                                     float& enter, float& exit) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const bool zero = (AXIS >= 0) ? (k != AXIS) : (r.inv[k] == 0.0f);
        if (zero) {
            if (r.o[k] < lo[k] || r.o[k] > hi[k]) return false;
            continue;
        }
        float inv = (AXIS >= 0) ? 1.0f : r.inv[k];
        float t1 = (AXIS >= 0) ? __fsub_rn(lo[k], r.o[k]) : __fmul_rn(__fsub_rn(lo[k], r.o[k]), inv);
        float t2 = (AXIS >= 0) ? __fsub_rn(hi[k], r.o[k]) : __fmul_rn(__fsub_rn(hi[k], r.o[k]), inv);
        float tn = inv > 0.0f ? t1 : t2;
        float tf = inv > 0.0f ? t2 : t1;
        en = tn > en ? tn : en;
        ex = tf < ex ? tf : ex;
    }
    enter = en;
    exit = ex;
    return en <= ex;
}

// The triangle hit contract.  Returns true and the hit distance t when the
// triangle (a,b,c) is crossed with t in [tmin, tmax].
template <int AXIS>
__device__ __forceinline__ bool hit_triangle(const Ray& r, const float* a, const float* b, const float* c, float& t) {
    float lo[3], hi[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float mn = a[k] < b[k] ? a[k] : b[k];
        mn = c[k] < mn ? c[k] : mn;
        float mx = a[k] > b[k] ? a[k] : b[k];
        mx = c[k] > mx ? c[k] : mx;
        lo[k] = mn;
        hi[k] = mx;
    }
    float en, ex;
    if (!slab<AXIS>(r, lo, hi, -INFINITY, INFINITY, en, ex)) return false;
    // Cheap reject before the sign tests: the clamped t lies in [en, ex].
    if (ex < r.tmin || en > r.tmax) return false;
    const int s0 = perturbed_sign<AXIS>(r.d, r.o, a, b);
    if (s0 == 0) return false;
    if (perturbed_sign<AXIS>(r.d, r.o, b, c) != s0) return false;
    if (perturbed_sign<AXIS>(r.d, r.o, c, a) != s0) return false;
    const float e1x = __fsub_rn(b[0], a[0]), e1y = __fsub_rn(b[1], a[1]), e1z = __fsub_rn(b[2], a[2]);
    const float e2x = __fsub_rn(c[0], a[0]), e2y = __fsub_rn(c[1], a[1]), e2z = __fsub_rn(c[2], a[2]);
    const float nx = __fsub_rn(__fmul_rn(e1y, e2z), __fmul_rn(e1z, e2y));
    const float ny = __fsub_rn(__fmul_rn(e1z, e2x), __fmul_rn(e1x, e2z));
    const float nz = __fsub_rn(__fmul_rn(e1x, e2y), __fmul_rn(e1y, e2x));
    const float wx = __fsub_rn(a[0], r.o[0]), wy = __fsub_rn(a[1], r.o[1]), wz = __fsub_rn(a[2], r.o[2]);
    const float num = __fadd_rn(__fadd_rn(__fmul_rn(wx, nx), __fmul_rn(wy, ny)), __fmul_rn(wz, nz));
    const float den = __fadd_rn(__fadd_rn(__fmul_rn(r.d[0], nx), __fmul_rn(r.d[1], ny)), __fmul_rn(r.d[2], nz));
    const float traw = __fdiv_rn(num, den);
    t = (traw >= en) ? ((traw <= ex) ? traw : ex) : en;
    return t >= r.tmin && t <= r.tmax;
}

// ---------------------------------------------------------------------------
// BVH layout in HBM.  One 64-byte node holds both child boxes; a child with
// count > 0 is a leaf of `count` consecutive triangles starting at `idx`,
// count == 0 is the internal node `idx`.  Triangles are three float4 each in
// leaf order: (v0, original triangle id), (v1, object id), (v2, 0).
// ---------------------------------------------------------------------------
struct __align__(16) BNode {
    float4 a;  // lo0.x lo0.y lo0.z hi0.x
    float4 b;  // hi0.y hi0.z lo1.x lo1.y
    float4 c;  // lo1.z hi1.x hi1.y hi1.z
    int4 d;    // idx0 count0 idx1 count1
};

constexpr int kStack = 64;

// Visits every leaf whose box passes the slab test and calls on_leaf(first, count)
// for it.  The stack lives at stack[sp * stride] (a thread-private array, or a column
// of a shared-memory array).  A valid tree visits each node at most once, so
// `max_steps` (the node count) bounds the loop even if the node array were corrupt.
// Returns false on stack overflow or an exhausted step budget.  ORDERED visits first the
// child the ray enters first, for callers that shrink r.tmax as hits come in: the far
// child's subtree is then mostly rejected by the shrunken range when it is popped.
template <int AXIS, int STACK = kStack, bool ORDERED = false, class F>
__device__ __forceinline__ bool traverse_with(int* stack, int stride, const BNode* __restrict__ nodes,
                                              uint32_t max_steps, const Ray& r, F&& on_leaf, int start = 0) {
    int sp = 0;
    int node = start;  // the root, or a node known to hold every triangle the ray can hit
    for (uint32_t step = 0;; ++step) {
        if (step > max_steps) return false;
        const float4 na = __ldg(&nodes[node].a);
        const float4 nb = __ldg(&nodes[node].b);
        const float4 nc = __ldg(&nodes[node].c);
        const int4 nd = __ldg(&nodes[node].d);
        const float lo0[3] = {na.x, na.y, na.z}, hi0[3] = {na.w, nb.x, nb.y};
        const float lo1[3] = {nb.z, nb.w, nc.x}, hi1[3] = {nc.y, nc.z, nc.w};
        float e0, x0, e1, x1;
        bool h0 = slab<AXIS>(r, lo0, hi0, r.tmin, r.tmax, e0, x0);
        bool h1 = slab<AXIS>(r, lo1, hi1, r.tmin, r.tmax, e1, x1);
        if (h0 && nd.y > 0) { on_leaf(nd.x, nd.y); h0 = false; }
        if (h1 && nd.w > 0) { on_leaf(nd.z, nd.w); h1 = false; }
        if (h0 && h1) {
            if (sp == STACK) return false;
            const bool first1 = ORDERED && e1 < e0;
            stack[sp * stride] = first1 ? nd.x : nd.z;
            ++sp;
            node = first1 ? nd.z : nd.x;
        } else if (h0) {
            node = nd.x;
        } else if (h1) {
            node = nd.z;
        } else {
            if (sp == 0) break;
            --sp;
            node = stack[sp * stride];
        }
    }
    return true;
}

template <int AXIS, int STACK = kStack, bool ORDERED = false, class F>
__device__ __forceinline__ bool traverse(const BNode* __restrict__ nodes, uint32_t max_steps, const Ray& r,
                                         F&& on_leaf) {
    int stack[STACK];
    return traverse_with<AXIS, STACK, ORDERED>(stack, 1, nodes, max_steps, r, on_leaf);
}

__device__ __forceinline__ void load_tri(const float4* __restrict__ tris, int k, float* a, float* b, float* c,
                                         uint32_t& tri_id, int32_t& obj) {
    const float4 p = __ldg(&tris[3 * (size_t)k]);
    const float4 q = __ldg(&tris[3 * (size_t)k + 1]);
    const float4 s = __ldg(&tris[3 * (size_t)k + 2]);
    a[0] = p.x; a[1] = p.y; a[2] = p.z;
    b[0] = q.x; b[1] = q.y; b[2] = q.z;
    c[0] = s.x; c[1] = s.y; c[2] = s.z;
    tri_id = __float_as_uint(p.w);
    obj = __float_as_int(q.w);
}

// ---------------------------------------------------------------------------
// Pair hash table: open addressing, linear probing, MurmurHash3 fmix64 of the
// key (id1<<32 | id2), empty slot = all ones (mesh_overlap_edges.cu:62-104).
// ---------------------------------------------------------------------------
constexpr unsigned long long kEmptyKey = 0xFFFFFFFFFFFFFFFFull;

__device__ __forceinline__ unsigned long long fmix64(unsigned long long k) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ull;
    k ^= k >> 33;
    return k;
}

struct PairTable {
    unsigned long long* slots;
    unsigned long long capacity;  // power of two when pow2 != 0
    int pow2;
    unsigned int max_probes;
    unsigned int* status;         // OR of ST_* bits
    unsigned long long* count;    // number of distinct keys inserted
    unsigned long long* stats;    // nullable: [0] slot accesses, [1] contended probes (--track-hash-contention)
    // Hit rule of the edge rays that insert into the table: at most max_hits hits per
    // edge, the next hit searched from t + 1e-6 (next_float == 0) or from the next float
    // after t (next_float != 0).
    int max_hits;
    int next_float;
    // Overflow table (nullable): a second open-addressing table of over_mask + 1 slots,
    // kept empty between joins.  Once the main table passes 3/4 of its slots, or a key
    // finds no slot within max_probes, ST_SPILLED is raised; from then on an insert that
    // does not settle at its first slot of the main table goes to the overflow table (a
    // full main table would otherwise make every insert walk its whole probe limit, each
    // step a dependent load).  A key may then sit in both tables; the regrowth merges
    // them.  A key that finds no slot in either raises ST_TABLE_FULL.
    unsigned long long* over;
    unsigned long long over_mask;
    unsigned long long* over_count;
    unsigned long long spill_at;  // main-table count that raises ST_SPILLED
};

constexpr unsigned int kOverProbes = 256;

// Open-addressing insert into slots[0..mask] (a power of two) from hash h; false when no
// slot was found within `probes`.
__device__ __forceinline__ bool probe_insert(unsigned long long* slots, unsigned long long mask, unsigned long long h,
                                             unsigned long long key, unsigned int probes, unsigned long long* count) {
    unsigned long long slot = h & mask;
    for (unsigned int i = 0; i < probes; ++i) {
        const unsigned long long cur = slots[slot];
        if (cur == key) return true;
        if (cur == kEmptyKey) {
            const unsigned long long old = atomicCAS(&slots[slot], kEmptyKey, key);
            if (old == kEmptyKey) {
                atomicAdd(count, 1ull);
                return true;
            }
            if (old == key) return true;
        }
        slot = (slot + 1) & mask;
    }
    return false;
}

__device__ __forceinline__ void table_insert(const PairTable& t, unsigned long long key) {
    const unsigned long long h = fmix64(key);
    unsigned long long slot = t.pow2 ? (h & (t.capacity - 1)) : (h % t.capacity);
    // The status word is read with the first probe (the two loads overlap) and again every
    // 32 probes: once the table has spilled, an insert that does not settle at its first
    // slot goes to the overflow table.
    unsigned int st = t.over ? *(volatile unsigned int*)t.status : 0u;
    unsigned int i = 0;
    for (; i < t.max_probes; ++i) {
        if (i > 0 && t.over) {
            if ((i & 31u) == 0) st = *(volatile unsigned int*)t.status;
            if (st & ST_SPILLED) break;
        }
        if (t.stats) atomicAdd(&t.stats[0], 1ull);
        unsigned long long cur = t.slots[slot];
        if (cur == key) return;
        if (cur == kEmptyKey) {
            unsigned long long old = atomicCAS(&t.slots[slot], kEmptyKey, key);
            if (old == kEmptyKey) {
                const unsigned long long c = atomicAdd(t.count, 1ull);
                if (t.over && c + 1 == t.spill_at) atomicOr(t.status, ST_SPILLED);
                return;
            }
            if (old == key) return;
        }
        if (t.stats) atomicAdd(&t.stats[1], 1ull);
        slot = slot + 1;
        if (slot == t.capacity) slot = 0;
    }
    if (t.over) {
        if (i == t.max_probes) atomicOr(t.status, ST_SPILLED);
        // The overflow table hashes the other half of the key's hash.
        if (probe_insert(t.over, t.over_mask, h >> 32 | h << 32, key, kOverProbes, t.over_count)) return;
    }
    atomicOr(t.status, ST_TABLE_FULL);
}

}  // namespace rs
