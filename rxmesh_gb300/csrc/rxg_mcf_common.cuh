// Device pieces shared by the MCF, adjoint and batched-MCF kernels:
// cotangent weights and Voronoi areas, 4-wide row vectors and packed
// entries, block reductions and the packed row SpMV.
#pragma once

#include <cfloat>

#include "rxg_device.cuh"

namespace rxg {

// ---------------------------------------------------------------------
// cotangent weights and Voronoi areas (include/rxmesh/geometry_util.cuh)
// ---------------------------------------------------------------------

template <typename T>
struct V3
{
    T x, y, z;
};
template <typename T>
__device__ __forceinline__ V3<T> sub(V3<T> a, V3<T> b)
{
    return {a.x - b.x, a.y - b.y, a.z - b.z};
}
template <typename T>
__device__ __forceinline__ T dot(V3<T> a, V3<T> b)
{
    return a.x * b.x + a.y * b.y + a.z * b.z;
}
template <typename T>
__device__ __forceinline__ V3<T> cross(V3<T> a, V3<T> b)
{
    // glm::cross component order
    return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}
template <typename T>
__device__ __forceinline__ T tri_area(V3<T> p0, V3<T> p1, V3<T> p2)
{
    V3<T> c = cross(sub(p1, p0), sub(p2, p0));
    return T(0.5) * sqrt(dot(c, c));
}
template <typename T>
__device__ __forceinline__ T clamp_cot(T v)
{
    const T bound = T(19.1);
    return v < -bound ? -bound : (v > bound ? bound : v);
}
template <typename T>
__device__ __forceinline__ T tmin();
template <>
__device__ __forceinline__ float tmin<float>()
{
    return FLT_MIN;
}
template <>
__device__ __forceinline__ double tmin<double>()
{
    return DBL_MIN;
}

// partial_weight of edge_cotan_weight (geometry_util.cuh:173-206)
template <typename T>
__device__ __forceinline__ T half_cot(V3<T> p, V3<T> r, V3<T> v)
{
    const T A = tri_area(p, r, v);
    if (A > tmin<T>()) return clamp_cot(dot(sub(p, v), sub(r, v)) / A);
    return T(0);
}

// partial_voronoi_area (geometry_util.cuh:117-167)
template <typename T>
__device__ __forceinline__ T voronoi(V3<T> p, V3<T> q, V3<T> r)
{
    const V3<T> pq = sub(q, p), qr = sub(r, q), pr = sub(r, p);
    const T     A  = tri_area(p, q, r);
    if (A <= tmin<T>()) return T(-1);
    const T dp = dot(pq, pr), dq = -dot(qr, pq), dr = dot(qr, pr);
    if (dp < T(0)) return T(0.25) * A;
    if (dq < T(0) || dr < T(0)) return T(0.125) * A;
    return T(0.125) * (dot(pr, pr) * clamp_cot(dq / A) + dot(pq, pq) * clamp_cot(dr / A));
}

// 1 / sqrt(x) in one call (FP64 and FP32 reciprocal square roots)
__device__ __forceinline__ double inv_sqrt(double x) { return ::rsqrt(x); }
__device__ __forceinline__ float  inv_sqrt(float x) { return ::rsqrtf(x); }

// The three geometry terms of fan triangle (p, a, b) (a before b around p)
// that a row of the MCF system uses, sharing the triangle's area:
//   ha = half_cot(p, a, b)   (edge p-a, seen from b)
//   hb = half_cot(p, b, a)   (edge p-b, seen from a)
//   va = voronoi(p, a, b)
// The same formulas as the three separate calls with the area's square root
// and the two cotangent divisions replaced by one reciprocal square root of
// |cross|^2: with il = 1 / |cross|, A = |cross|^2 il / 2 and dot / A =
// 2 dot il (within a unit or two in the last place of the separate calls'
// values; on GB300 each FP64 square root or division is a long sequence on
// the FP64 pipe).  The three areas are one |cross| (a swapped cross product
// is its exact negation) and the half-cotangents' dot products are the
// Voronoi corner products dr and dq.  A > DBL_MIN (FLT_MIN) of the
// separate calls holds exactly when |cross|^2 > 0.
template <typename T>
struct TriTerms
{
    T ha, hb, va;
};
template <typename T>
__device__ __forceinline__ TriTerms<T> tri_terms(V3<T> p, V3<T> a, V3<T> b)
{
    const V3<T> pq = sub(a, p), qr = sub(b, a), pr = sub(b, p);
    const V3<T> c  = cross(pq, pr);
    const T     cc = dot(c, c);
    if (!(cc > T(0))) return {T(0), T(0), T(-1)};
    const T il = inv_sqrt(cc);
    const T A  = T(0.5) * (cc * il);
    const T dp = dot(pq, pr), dq = -dot(qr, pq), dr = dot(qr, pr);
    const T ha = clamp_cot(T(2) * (dr * il)), hb = clamp_cot(T(2) * (dq * il));
    T       va;
    if (dp < T(0)) va = T(0.25) * A;
    else if (dq < T(0) || dr < T(0)) va = T(0.125) * A;
    else va = T(0.125) * (dot(pr, pr) * hb + dot(pq, pq) * ha);
    return {ha, hb, va};
}

template <typename T, typename S>
__device__ __forceinline__ V3<T> to_t(V3<S> a)
{
    return {(T)a.x, (T)a.y, (T)a.z};
}

// Row geometry of vertex p's fan with each triangle evaluated once
// (tri_terms): calls on_w(i, w_i) for ring entries i = 0..k-1 in order, w_i
// = max(0, cot-halves) * dt as the per-call loop forms it (Q half first,
// then S half), and returns the sum of the clamped Voronoi terms in the same
// order.  pos(i): the position (V3<double>, or V3<float> already rounded
// when T is float) of ring entry i.  wrap: a closed fan (interior vertex);
// an open fan has no triangle (p, r_{k-1}, r_0).
template <typename T, typename TB, typename PP, typename Pos, typename OnW>
__device__ __forceinline__ TB fan_row(V3<PP> Pd, int32_t k, bool wrap, T dt, Pos pos, OnW on_w)
{
    TB area = TB(0);
    if (k <= 0) return area;
    const V3<T> P     = to_t<T>(Pd);
    const V3<T> first = to_t<T>(pos(0));
    V3<T>       R     = first;
    TriTerms<T> prev{T(0), T(0), T(-1)}, last{T(0), T(0), T(-1)};
    if (wrap) {
        last = tri_terms<T>(P, to_t<T>(pos(k - 1)), first);  // (p, r_{k-1}, r_0)
        prev = last;
    }
    for (int32_t i = 0; i < k; ++i) {
        const bool  has_q = wrap || i > 0, has_s = wrap || i < k - 1;
        TriTerms<T> cur{T(0), T(0), T(-1)};
        V3<T>       S = R;
        if (has_s) {
            if (i + 1 < k) {
                S   = to_t<T>(pos(i + 1));
                cur = tri_terms<T>(P, R, S);
            } else {
                cur = last;  // the closing triangle, evaluated above
            }
        }
        T w = T(0);
        if (has_q) w += prev.hb;
        if (has_s) w += cur.ha;
        w = (w >= T(0) ? w : T(0)) * dt;
        on_w(i, w);
        if (has_q) area += prev.va > T(0) ? (TB)prev.va : TB(0);
        prev = cur;
        R    = S;
    }
    return area;
}

// fan_row for rings of at most eight neighbours whose positions are already
// in registers (X[0..k)): the same triangles, arithmetic and order, with the
// ring loop unrolled over the eight slots so that every X[i] and every
// on_w(i, .) index is a compile-time constant (no run-time selection among
// registers); only the closing triangle's r_{k-1} is selected at run time.
template <typename T, typename TB, typename PP, typename OnW>
__device__ __forceinline__ TB fan_row8(V3<PP> Pd, int32_t k, bool wrap, T dt, const V3<PP> (&X)[8], OnW on_w)
{
    TB area = TB(0);
    if (k <= 0) return area;
    const V3<T> P = to_t<T>(Pd);
    V3<T>       Xt[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) Xt[i] = to_t<T>(X[i]);
    TriTerms<T> prev{T(0), T(0), T(-1)}, last{T(0), T(0), T(-1)};
    if (wrap) {
        V3<T> rl = Xt[0];
#pragma unroll
        for (int j = 1; j < 8; ++j)
            if (j == k - 1) rl = Xt[j];
        last = tri_terms<T>(P, rl, Xt[0]);  // (p, r_{k-1}, r_0)
        prev = last;
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        if (i < k) {
            const bool  has_q = wrap || i > 0, has_s = wrap || i < k - 1;
            TriTerms<T> cur{T(0), T(0), T(-1)};
            if (has_s) {
                if (i + 1 < k) cur = tri_terms<T>(P, Xt[i], Xt[i < 7 ? i + 1 : 7]);
                else cur = last;  // the closing triangle, evaluated above
            }
            T w = T(0);
            if (has_q) w += prev.hb;
            if (has_s) w += cur.ha;
            w = (w >= T(0) ? w : T(0)) * dt;
            on_w(i, w);
            if (has_q) area += prev.va > T(0) ? (TB)prev.va : TB(0);
            prev = cur;
        }
    }
    return area;
}

__device__ __forceinline__ V3<float> tof(V3<double> a)
{
    return {(float)a.x, (float)a.y, (float)a.z};
}

// true when a triangle has an angle below 1e-3 rad: sin^2 of its smallest
// angle, |cross|^2 / (product of the two largest squared edge lengths)
__device__ __forceinline__ bool near_degenerate(V3<float> a, V3<float> b, V3<float> c)
{
    const V3<float> ab = sub(b, a), ac = sub(c, a), bc = sub(c, b);
    const V3<float> cr = cross(ab, ac);
    const float     l0 = dot(ab, ab), l1 = dot(ac, ac), l2 = dot(bc, bc);
    const float     mn = fminf(l0, fminf(l1, l2));
    const float     big = (l0 * l1 * l2) / fmaxf(mn, FLT_MIN);
    return dot(cr, cr) < 1e-6f * big;
}

// weight and area evaluators: exact type T, or FP32 with an FP64 redo of
// near-degenerate triangles (the mixed path).  Each takes points of its own
// type (G::Pt, made once per loaded position by G::make), so that a position
// is converted once however many triangles it belongs to.
template <typename T>
struct Geo
{
    using Pt = V3<double>;
    __device__ static Pt make(V3<double> a) { return a; }
    __device__ static T  hc(V3<double> p, V3<double> r, V3<double> v)
    {
        return half_cot<T>({(T)p.x, (T)p.y, (T)p.z}, {(T)r.x, (T)r.y, (T)r.z}, {(T)v.x, (T)v.y, (T)v.z});
    }
    __device__ static T va(V3<double> p, V3<double> q, V3<double> r)
    {
        return voronoi<T>({(T)p.x, (T)p.y, (T)p.z}, {(T)q.x, (T)q.y, (T)q.z}, {(T)r.x, (T)r.y, (T)r.z});
    }
};
// true when a corner angle of the triangle is within ~1e-5 rad of 90 degrees:
// partial_voronoi_area switches branch there and its value jumps (A to A/4
// at p, A/2 to A/8 at q or r), so FP32 rounding must not pick the branch
__device__ __forceinline__ bool near_right_angle(V3<float> p, V3<float> q, V3<float> r)
{
    const V3<float> pq = sub(q, p), pr = sub(r, p), qr = sub(r, q);
    const float     lpq = dot(pq, pq), lpr = dot(pr, pr), lqr = dot(qr, qr);
    const float     dp = dot(pq, pr), dq = dot(qr, pq), dr = dot(qr, pr);
    const float     t  = 1e-10f;  // (1e-5)^2
    return dp * dp < t * lpq * lpr || dq * dq < t * lqr * lpq || dr * dr < t * lqr * lpr;
}

// a position in FP64 and its FP32 rounding
struct MixedPt
{
    V3<double> d;
    V3<float>  f;
};

struct GeoMixed
{
    using Pt = MixedPt;
    __device__ static Pt    make(V3<double> a) { return {a, tof(a)}; }
    __device__ static float hc(const Pt& p, const Pt& r, const Pt& v)
    {
        if (near_degenerate(p.f, r.f, v.f)) return (float)half_cot<double>(p.d, r.d, v.d);
        return half_cot<float>(p.f, r.f, v.f);
    }
    __device__ static float va(const Pt& p, const Pt& q, const Pt& r)
    {
        if (near_degenerate(p.f, q.f, r.f) || near_right_angle(p.f, q.f, r.f))
            return (float)voronoi<double>(p.d, q.d, r.d);
        return voronoi<float>(p.f, q.f, r.f);
    }
};

__device__ __forceinline__ V3<double> ld3(const double* __restrict__ x, int32_t i)
{
    return {__ldg(x + 3 * (int64_t)i), __ldg(x + 3 * (int64_t)i + 1), __ldg(x + 3 * (int64_t)i + 2)};
}
__device__ __forceinline__ V3<float> ld3(const float* __restrict__ x, int32_t i)
{
    return {__ldg(x + 3 * (int64_t)i), __ldg(x + 3 * (int64_t)i + 1), __ldg(x + 3 * (int64_t)i + 2)};
}

// 4-wide row vectors (x, y, z, pad) and packed (column, value) entries of the
// MCF solver: one 16- or 32-byte access per row and one per non-zero.
template <typename T>
struct alignas(4 * sizeof(T)) R4
{
    T x, y, z, w;
};
template <typename T>
struct alignas(sizeof(T) == 8 ? 16 : 8) Ent
{
    int32_t col;
    T       val;
};

// block sum of a double, result valid in every thread
template <int BT>
__device__ __forceinline__ double block_sum(double v, double* s_red)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) s_red[warp] = v;
    __syncthreads();
    double t = 0;
    if (warp == 0) {
        t = lane < BT / 32 ? s_red[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (lane == 0) s_red[BT / 32] = t;
    }
    __syncthreads();
    return s_red[BT / 32];
}

// acc += sum_j A_ij x_j over row i, eight entries per round (all entry
// loads, then all gathers, in flight together); diag receives A_ii if asked
template <typename T>
__device__ __forceinline__ void row_spmv4(const int32_t* __restrict__ rp, const Ent<T>* __restrict__ ent,
                                          int64_t i, const R4<T>* x, T& ax, T& ay, T& az, T* diag)
{
    const int32_t b = __ldg(rp + i), e = __ldg(rp + i + 1);
    // seven entries per round: a valence-6 vertex's row in one round with no
    // padded entry (no FP64 multiply-add spent on padding)
    constexpr int RW = 7;
    for (int32_t j0 = b; j0 < e; j0 += RW) {
        Ent<T> q[RW];
#pragma unroll
        for (int u = 0; u < RW; ++u) {
            if (j0 + u < e) {
                q[u] = ent[j0 + u];
            } else {
                q[u].col = (int32_t)i;
                q[u].val = T(0);
            }
        }
#pragma unroll
        for (int u = 0; u < RW; ++u) {
            if (diag && j0 + u < e && q[u].col == i) *diag = q[u].val;
            const R4<T> xv = x[q[u].col];
            ax += q[u].val * xv.x;
            ay += q[u].val * xv.y;
            az += q[u].val * xv.z;
        }
    }
}

}  // namespace rxg
