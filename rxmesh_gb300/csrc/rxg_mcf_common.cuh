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
// near-degenerate triangles (the mixed path)
template <typename T>
struct Geo
{
    __device__ static T hc(V3<double> p, V3<double> r, V3<double> v)
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

struct GeoMixed
{
    __device__ static float hc(V3<double> p, V3<double> r, V3<double> v)
    {
        const V3<float> pf = tof(p), rf = tof(r), vf = tof(v);
        if (near_degenerate(pf, rf, vf)) return (float)half_cot<double>(p, r, v);
        return half_cot<float>(pf, rf, vf);
    }
    __device__ static float va(V3<double> p, V3<double> q, V3<double> r)
    {
        const V3<float> pf = tof(p), qf = tof(q), rf = tof(r);
        if (near_degenerate(pf, qf, rf) || near_right_angle(pf, qf, rf))
            return (float)voronoi<double>(p, q, r);
        return voronoi<float>(pf, qf, rf);
    }
};

__device__ __forceinline__ V3<double> ld3(const double* __restrict__ x, int32_t i)
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
    for (int32_t j0 = b; j0 < e; j0 += 8) {
        Ent<T> q[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            if (j0 + u < e) {
                q[u] = ent[j0 + u];
            } else {
                q[u].col = (int32_t)i;
                q[u].val = T(0);
            }
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            if (diag && j0 + u < e && q[u].col == i) *diag = q[u].val;
            const R4<T> xv = x[q[u].col];
            ax += q[u].val * xv.x;
            ay += q[u].val * xv.y;
            az += q[u].val * xv.z;
        }
    }
}

}  // namespace rxg
