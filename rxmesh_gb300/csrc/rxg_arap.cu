// Per-face ARAP energy, gradient and 3x3-block Hessian (the DiffScalarProblem
// path: diff/diff_scalar_problem.h:310-321, diff/diff_query_kernel.cuh:199-322,
// diff/hessian_sparse_matrix.h:16-137), written analytically instead of with
// forward-mode AD.
//
// Energy of face f with rest frame Mr (param.cu:113-141) and deformed edge
// matrix M = [b-a, c-a] (3x2): J = M Mr^{-1} = [j1 j2],
//   E_f = A_f * ||J - R(J)||_F^2 = A_f * (s - 2 sqrt(s + 2d) + 2),
//   s = |j1|^2 + |j2|^2 = s1^2 + s2^2,  d = |j1 x j2| = s1 s2,
// with R(J) the polar factor and s1, s2 the singular values of J.
//
// Assembly is a vertex-centred gather: each vertex walks the faces of its
// oriented fan and writes its own block row [diag, ring...] once, so no
// atomics are needed and the result is deterministic.  In FP32 each vertex
// evaluates its fan's faces itself (k_arap_vertex); in FP64, which runs at a
// small fraction of the FP32 rate, each face is evaluated once into a global
// record (k_arap_face) that its three vertices then read (k_arap_gather).
#include <algorithm>
#include <cfloat>
#include <climits>
#include <cstdlib>
#include <type_traits>

#include "rxg_device.cuh"
#include "rxg_gridsum.cuh"
#include "rxg_lazy.h"

namespace rxg {

template <typename T>
struct FaceDeriv
{
    T E;
    T gE[6];     // dE/du, u = [j1; j2]
    T Hu[6][6];  // d2E/du2
    T d[3][2];   // u_k = sum_v d[v][k] x_v
};

template <typename T>
__device__ __forceinline__ void cross3(const T* a, const T* b, T* c)
{
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

// 1 / sqrt(x), FP64 and FP32
__device__ __forceinline__ double arap_rsqrt(double x) { return ::rsqrt(x); }
__device__ __forceinline__ float  arap_rsqrt(float x) { return ::rsqrtf(x); }

template <typename T, bool HESS>
__device__ __forceinline__ void arap_face(const T* x9, const T* mi, T A, FaceDeriv<T>& o)
{
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        o.d[1][k] = mi[k];
        o.d[2][k] = mi[2 + k];
        o.d[0][k] = -(o.d[1][k] + o.d[2][k]);
    }
    T u[6];
#pragma unroll
    for (int k = 0; k < 2; ++k)
#pragma unroll
        for (int c = 0; c < 3; ++c)
            u[3 * k + c] = o.d[0][k] * x9[c] + o.d[1][k] * x9[3 + c] + o.d[2][k] * x9[6 + c];
    const T* j1 = u;
    const T* j2 = u + 3;
    const T  s  = j1[0] * j1[0] + j1[1] * j1[1] + j1[2] * j1[2] + j2[0] * j2[0] + j2[1] * j2[1] +
               j2[2] * j2[2];
    T w[3];
    cross3(j1, j2, w);
    // |w| and |q|^(1/2) with their reciprocals from one reciprocal square
    // root each (FP64 square roots and divisions are long sequences on
    // GB300's FP64 pipe): d = ww / sqrt(ww), sq = q / sqrt(q)
    const T ww  = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
    const T id  = ww > T(0) ? arap_rsqrt(ww) : T(0);  // 1 / d (0 for a degenerate J)
    const T d   = ww * id;
    const T q   = s + T(2) * d;
    const T isq = arap_rsqrt(q);
    const T sq  = q * isq;
    {
        // Energy without cancellation near the rest state: with M = J^T J - I
        // and mu its eigenvalues (sigma^2 - 1), (sigma - 1)^2 equals
        // mu^2 / (sqrt(1 + mu) + 1)^2.  (s - 2 sqrt(q) + 2 loses every digit
        // of a small strain in FP32.)
        const T m00 = fma(j1[0], j1[0], fma(j1[1], j1[1], fma(j1[2], j1[2], T(-1))));
        const T m11 = fma(j2[0], j2[0], fma(j2[1], j2[1], fma(j2[2], j2[2], T(-1))));
        const T m01 = j1[0] * j2[0] + j1[1] * j2[1] + j1[2] * j2[2];
        const T hm  = T(0.5) * (m00 + m11);
        const T dm  = T(0.5) * (m00 - m11);
        const T r   = sqrt(dm * dm + m01 * m01);
        const T det = m00 * m11 - m01 * m01;
        T       mu1, mu2;
        if (hm >= T(0)) {
            mu1 = hm + r;
            mu2 = mu1 != T(0) ? det / mu1 : T(0);
        } else {
            mu2 = hm - r;
            mu1 = det / mu2;
        }
        auto f = [](T mu) {
            const T den = sqrt(max(T(0), T(1) + mu)) + T(1);
            return (mu / den) * (mu / den);
        };
        o.E = A * (f(mu1) + f(mu2));
    }
    // W = dw/du = [ -[j2]x , [j1]x ]
    T W[3][6];
    {
        const T cj2[3][3] = {{0, -j2[2], j2[1]}, {j2[2], 0, -j2[0]}, {-j2[1], j2[0], 0}};
        const T cj1[3][3] = {{0, -j1[2], j1[1]}, {j1[2], 0, -j1[0]}, {-j1[1], j1[0], 0}};
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                W[i][j]     = -cj2[i][j];
                W[i][j + 3] = cj1[i][j];
            }
    }
    const T wh[3] = {w[0] * id, w[1] * id, w[2] * id};  // 0 when d = 0
    T       gq[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        const T gd = W[0][i] * wh[0] + W[1][i] * wh[1] + W[2][i] * wh[2];
        gq[i]      = T(2) * u[i] + T(2) * gd;
        o.gE[i]    = A * (T(2) * u[i] - gq[i] * isq);
    }
    if (!HESS) return;
    // Hd = W^T P W + [[0, -[wh]x], [[wh]x, 0]],  P = (I - wh wh^T) / d
    T PW[3][6];
    if (d > T(0)) {
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int b = 0; b < 6; ++b) {
                const T ww = wh[0] * W[0][b] + wh[1] * W[1][b] + wh[2] * W[2][b];
                PW[i][b]   = (W[i][b] - wh[i] * ww) * id;
            }
    } else {
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int b = 0; b < 6; ++b) PW[i][b] = T(0);
    }
    const T cw[3][3] = {{0, -wh[2], wh[1]}, {wh[2], 0, -wh[0]}, {-wh[1], wh[0], 0}};
    const T c3 = T(0.5) * isq * isq * isq;  // 1 / (2 q sq)
#pragma unroll
    for (int a = 0; a < 6; ++a)
#pragma unroll
        for (int b = a; b < 6; ++b) {
            T hd = W[0][a] * PW[0][b] + W[1][a] * PW[1][b] + W[2][a] * PW[2][b];
            if (a < 3 && b >= 3) hd += -cw[a][b - 3];
            const T hs = a == b ? T(2) : T(0);
            const T h  = A * (hs - (hs + T(2) * hd) * isq + gq[a] * gq[b] * c3);
            o.Hu[a][b] = h;
            o.Hu[b][a] = h;
        }
}

// d[l][k] with a run-time l, by selects (keeps d in registers)
template <typename T>
__device__ __forceinline__ T dsel(const FaceDeriv<T>& o, int l, int k)
{
    return l == 0 ? o.d[0][k] : (l == 1 ? o.d[1][k] : o.d[2][k]);
}

// out (3x3 row-major) += d[vi] x d[vj] contraction of Hu
template <typename T>
__device__ __forceinline__ void block_of(const FaceDeriv<T>& o, int vi, int vj, T* out)
{
    const T a0 = dsel(o, vi, 0), a1 = dsel(o, vi, 1), b0 = dsel(o, vj, 0), b1 = dsel(o, vj, 1);
#pragma unroll
    for (int ci = 0; ci < 3; ++ci)
#pragma unroll
        for (int cj = 0; cj < 3; ++cj)
            out[3 * ci + cj] += a0 * (b0 * o.Hu[ci][cj] + b1 * o.Hu[ci][3 + cj]) +
                                a1 * (b0 * o.Hu[3 + ci][cj] + b1 * o.Hu[3 + ci][3 + cj]);
}

// rest frame of param.cu:113-141 -> Mr^{-1} (row-major 2x2) per face
template <typename T>
__global__ void k_arap_rest(int64_t nf, const int32_t* __restrict__ fv, const double* __restrict__ xr,
                            T* __restrict__ minv)
{
    for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < nf;
         f += (int64_t)gridDim.x * blockDim.x) {
        const double* a = xr + 3 * (int64_t)fv[3 * f];
        const double* b = xr + 3 * (int64_t)fv[3 * f + 1];
        const double* c = xr + 3 * (int64_t)fv[3 * f + 2];
        const double  e1[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
        const double  e2[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
        double        n[3], t[3];
        cross3(e1, e2, n);
        const double l1    = sqrt(e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2]);
        const double b1[3] = {e1[0] / l1, e1[1] / l1, e1[2] / l1};
        cross3(n, b1, t);
        const double lt    = sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
        const double b2[3] = {t[0] / lt, t[1] / lt, t[2] / lt};
        const double m00 = e1[0] * b1[0] + e1[1] * b1[1] + e1[2] * b1[2];
        const double m01 = e2[0] * b1[0] + e2[1] * b1[1] + e2[2] * b1[2];
        const double m11 = e2[0] * b2[0] + e2[1] * b2[1] + e2[2] * b2[2];
        const double det = m00 * m11;
        minv[4 * f + 0]  = (T)(m11 / det);
        minv[4 * f + 1]  = (T)(-m01 / det);
        minv[4 * f + 2]  = (T)0;
        minv[4 * f + 3]  = (T)(m00 / det);
    }
}

template <typename T>
__device__ __forceinline__ void load_face(const int32_t* __restrict__ fv, const T* __restrict__ x,
                                          const T* __restrict__ minv, int32_t f, int32_t v[3],
                                          T x9[9], T mi[4], T& area)
{
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        v[k] = __ldg(fv + 3 * (int64_t)f + k);
#pragma unroll
        for (int c = 0; c < 3; ++c) x9[3 * k + c] = x[3 * (int64_t)v[k] + c];
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) mi[k] = __ldg(minv + 4 * (int64_t)f + k);
    area = T(0.5) / (mi[0] * mi[3] - mi[1] * mi[2]);
}

__device__ __forceinline__ int local_index(const int32_t v[3], int32_t p)
{
    return v[0] == p ? 0 : (v[1] == p ? 1 : 2);
}

template <int BT>
__device__ __forceinline__ double block_sum_d(double v, double* s_red)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) s_red[warp] = v;
    __syncthreads();
    double t = 0;
    if (warp == 0) {
        t = lane < BT / 32 ? s_red[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    }
    return t;  // valid in thread 0
}

// One thread per vertex p: gradient row, Hessian block row [diag, ring...],
// and (for faces whose first vertex is p) the face energy.
template <typename T, bool HESS>
// FP32: registers capped for 5 CTAs per SM (96, with a 32-byte spill): 0.155
// against 0.164 ms uncapped (120 registers, 4 CTAs) on the 512^2 cloth; FP64
// keeps its registers
__global__ void __launch_bounds__(128, sizeof(T) == 4 ? 5 : 1) k_arap_vertex(
    int64_t nv, const int32_t* __restrict__ row_ptr, const int32_t* __restrict__ ring_off,
    const int32_t* __restrict__ ring, const int32_t* __restrict__ ring_face,
    const int8_t* __restrict__ bnd, const int32_t* __restrict__ fv, const T* __restrict__ x,
    const T* __restrict__ minv, T* __restrict__ face_E, T* __restrict__ grad, T* __restrict__ hval,
    double* __restrict__ part)
{
    __shared__ double s_red[128 / 32];
    double            esum = 0;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nv;
         p += (int64_t)gridDim.x * blockDim.x) {
        const int32_t  ro = ring_off[p];
        const int32_t  k  = ring_off[p + 1] - ro;
        const int32_t  nf = bnd[p] ? k - 1 : k;
        const int32_t  rp = row_ptr[p];
        T              g[3] = {0, 0, 0}, D[9], carry[9];
#pragma unroll
        for (int i = 0; i < 9; ++i) D[i] = carry[i] = T(0);
        for (int32_t i = 0; i < nf; ++i) {
            const int32_t f = ring_face[ro + i];
            int32_t       v[3];
            T             x9[9], mi[4], area;
            load_face(fv, x, minv, f, v, x9, mi, area);
            FaceDeriv<T> o;
            arap_face<T, HESS>(x9, mi, area, o);
            const int lp = local_index(v, (int32_t)p);
#pragma unroll
            for (int c = 0; c < 3; ++c) g[c] += dsel(o, lp, 0) * o.gE[c] + dsel(o, lp, 1) * o.gE[3 + c];
            if (lp == 0) {
                if (face_E) face_E[f] = o.E;
                esum += (double)o.E;
            }
            if (HESS) {
                const int li = local_index(v, ring[ro + i]);
                const int lj = local_index(v, ring[ro + (i + 1 < k ? i + 1 : 0)]);
                block_of(o, lp, lp, D);
                T bi[9];
#pragma unroll
                for (int t = 0; t < 9; ++t) bi[t] = carry[t];
                block_of(o, lp, li, bi);
                T* slot = hval + 9 * (int64_t)(rp + 1 + i);
#pragma unroll
                for (int t = 0; t < 9; ++t) {
                    slot[t]  = bi[t];
                    carry[t] = T(0);
                }
                block_of(o, lp, lj, carry);
            }
        }
        if (HESS) {
            if (k > 0) {
                // interior: the last face also touches ring[0]; boundary: the
                // last neighbour has only the face before it
                T* slot = hval + 9 * (int64_t)(rp + 1 + (bnd[p] ? k - 1 : 0));
                if (bnd[p]) {
#pragma unroll
                    for (int t = 0; t < 9; ++t) slot[t] = carry[t];
                } else {
#pragma unroll
                    for (int t = 0; t < 9; ++t) slot[t] += carry[t];
                }
            }
            T* dslot = hval + 9 * (int64_t)rp;
#pragma unroll
            for (int t = 0; t < 9; ++t) dslot[t] = D[t];
        }
        if (grad) {
#pragma unroll
            for (int c = 0; c < 3; ++c) grad[3 * p + c] = g[c];
        }
    }
    const double t = block_sum_d<128>(esum, s_red);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// Words of one face record: E, dE/du (6), and with the Hessian its 21
// upper-triangle entries (row-major, a <= b), then the rest-frame inverse
// (4); padded to whole 16-byte vectors.
template <bool HESS>
__host__ __device__ constexpr int rec_words() { return HESS ? 32 : 12; }

// One thread per face: each face's energy, gradient and J-space Hessian are
// evaluated once into its record (face_E and the energy partials as well).
template <typename T, bool HESS>
__global__ void __launch_bounds__(128, sizeof(T) == 4 ? 5 : 1) k_arap_face(
    int64_t nf, const int32_t* __restrict__ fv, const T* __restrict__ x,
    const T* __restrict__ minv, T* __restrict__ rec, T* __restrict__ face_E,
    double* __restrict__ part)
{
    __shared__ double s_red[128 / 32];
    double            esum = 0;
    for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < nf;
         f += (int64_t)gridDim.x * blockDim.x) {
        int32_t v[3];
        T       x9[9], mi[4], area;
        load_face(fv, x, minv, (int32_t)f, v, x9, mi, area);
        FaceDeriv<T> o;
        arap_face<T, HESS>(x9, mi, area, o);
        T r[rec_words<HESS>()];
        r[0] = o.E;
#pragma unroll
        for (int i = 0; i < 6; ++i) r[1 + i] = o.gE[i];
        int t = 7;
        if (HESS) {
#pragma unroll
            for (int a = 0; a < 6; ++a)
#pragma unroll
                for (int c = a; c < 6; ++c) r[t++] = o.Hu[a][c];
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) r[t + i] = mi[i];
#pragma unroll
        for (int i = t + 4; i < rec_words<HESS>(); ++i) r[i] = T(0);
        // 16-byte stores of the whole record
        using V = typename std::conditional<sizeof(T) == 4, float4, double2>::type;
        constexpr int per = 16 / sizeof(T);
        V*       dst = reinterpret_cast<V*>(rec + (int64_t)rec_words<HESS>() * f);
        const V* src = reinterpret_cast<const V*>(r);
#pragma unroll
        for (int i = 0; i < rec_words<HESS>() / per; ++i) dst[i] = src[i];
        if (face_E) face_E[f] = o.E;
        esum += (double)o.E;
    }
    const double t = block_sum_d<128>(esum, s_red);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// the fields of face f's record that the vertex gather needs
template <typename T, bool HESS>
__device__ __forceinline__ void load_record(const T* __restrict__ rec, int32_t f, FaceDeriv<T>& o)
{
    using V = typename std::conditional<sizeof(T) == 4, float4, double2>::type;
    constexpr int per = 16 / sizeof(T);
    T             r[rec_words<HESS>()];
    const V*      src = reinterpret_cast<const V*>(rec + (int64_t)rec_words<HESS>() * f);
    V*            dst = reinterpret_cast<V*>(r);
#pragma unroll
    for (int i = 0; i < rec_words<HESS>() / per; ++i) dst[i] = __ldg(src + i);
    o.E = r[0];
#pragma unroll
    for (int i = 0; i < 6; ++i) o.gE[i] = r[1 + i];
    int t = 7;
    if (HESS) {
#pragma unroll
        for (int a = 0; a < 6; ++a)
#pragma unroll
            for (int c = a; c < 6; ++c) {
                o.Hu[a][c] = r[t];
                o.Hu[c][a] = r[t];
                ++t;
            }
    }
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        o.d[1][k] = r[t + k];
        o.d[2][k] = r[t + 2 + k];
        o.d[0][k] = -(o.d[1][k] + o.d[2][k]);
    }
}

// One thread per vertex p: gradient row and Hessian block row [diag,
// ring...] from the records of its fan's faces (the same contractions, in
// the same order, as k_arap_vertex).
template <typename T, bool HESS>
__global__ void __launch_bounds__(128) k_arap_gather(
    int64_t nv, const int32_t* __restrict__ row_ptr, const int32_t* __restrict__ ring_off,
    const int32_t* __restrict__ ring, const int32_t* __restrict__ ring_face,
    const int8_t* __restrict__ bnd, const int32_t* __restrict__ fv, const T* __restrict__ rec,
    T* __restrict__ grad, T* __restrict__ hval)
{
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nv;
         p += (int64_t)gridDim.x * blockDim.x) {
        const int32_t ro = ring_off[p];
        const int32_t k  = ring_off[p + 1] - ro;
        const int32_t nf = bnd[p] ? k - 1 : k;
        const int32_t rp = row_ptr[p];
        T             g[3] = {0, 0, 0}, D[9], carry[9];
#pragma unroll
        for (int i = 0; i < 9; ++i) D[i] = carry[i] = T(0);
        for (int32_t i = 0; i < nf; ++i) {
            const int32_t f    = ring_face[ro + i];
            const int32_t v[3] = {__ldg(fv + 3 * (int64_t)f), __ldg(fv + 3 * (int64_t)f + 1),
                                  __ldg(fv + 3 * (int64_t)f + 2)};
            FaceDeriv<T>  o;
            load_record<T, HESS>(rec, f, o);
            const int lp = local_index(v, (int32_t)p);
#pragma unroll
            for (int c = 0; c < 3; ++c) g[c] += dsel(o, lp, 0) * o.gE[c] + dsel(o, lp, 1) * o.gE[3 + c];
            if (HESS) {
                const int li = local_index(v, ring[ro + i]);
                const int lj = local_index(v, ring[ro + (i + 1 < k ? i + 1 : 0)]);
                block_of(o, lp, lp, D);
                T bi[9];
#pragma unroll
                for (int t = 0; t < 9; ++t) bi[t] = carry[t];
                block_of(o, lp, li, bi);
                T* slot = hval + 9 * (int64_t)(rp + 1 + i);
#pragma unroll
                for (int t = 0; t < 9; ++t) {
                    slot[t]  = bi[t];
                    carry[t] = T(0);
                }
                block_of(o, lp, lj, carry);
            }
        }
        if (HESS) {
            if (k > 0) {
                T* slot = hval + 9 * (int64_t)(rp + 1 + (bnd[p] ? k - 1 : 0));
                if (bnd[p]) {
#pragma unroll
                    for (int t = 0; t < 9; ++t) slot[t] = carry[t];
                } else {
#pragma unroll
                    for (int t = 0; t < 9; ++t) slot[t] += carry[t];
                }
            }
            T* dslot = hval + 9 * (int64_t)rp;
#pragma unroll
            for (int t = 0; t < 9; ++t) dslot[t] = D[t];
        }
        if (grad) {
#pragma unroll
            for (int c = 0; c < 3; ++c) grad[3 * p + c] = g[c];
        }
    }
}

// ---------------------------------------------------------------------
// Hessian projection (the reference's add_term<Op::FV, ProjectHess = true>,
// include/rxmesh/diff/hessian_projection.h:21-95): each face's 9x9 Hessian
// in vertex space is made positive definite before assembly.
// ---------------------------------------------------------------------

// Cyclic Jacobi eigen-decomposition of a symmetric K x K matrix (Golub and
// Van Loan, Matrix Computations, sec. 8.5): A (row-major) is rotated until
// its off-diagonal part vanishes, leaving the eigenvalues on its diagonal;
// V receives the eigenvectors as columns.  Each rotation zeroes A[p][q] with
// t = sgn(th) / (|th| + sqrt(th^2 + 1)), th = (A[q][q] - A[p][p]) / (2 A[p][q]),
// formed as sgn(th) |2 A[p][q]| / (|A[q][q] - A[p][p]| + hypot) (the same t
// with one division) and c = 1 / sqrt(t^2 + 1) as one reciprocal square root.
template <typename T, int K>
__device__ void jacobi_eigen(T* A, T* V)
{
    for (int i = 0; i < K * K; ++i) V[i] = (i % (K + 1)) == 0 ? T(1) : T(0);
    const T rel = sizeof(T) == 4 ? T(1e-14) : T(1e-30);
    for (int sweep = 0; sweep < 40; ++sweep) {
        T off = 0, all = 0;
        for (int i = 0; i < K; ++i)
            for (int j = 0; j < K; ++j) {
                const T a = A[i * K + j];
                all += a * a;
                if (i != j) off += a * a;
            }
        if (off <= rel * all) break;
        for (int p = 0; p < K - 1; ++p)
            for (int q = p + 1; q < K; ++q) {
                const T apq = A[p * K + q];
                if (apq == T(0)) continue;
                const T    dl  = A[q * K + q] - A[p * K + p], tw = T(2) * apq;
                const bool pos = dl == T(0) || ((dl > T(0)) == (tw > T(0)));  // th >= 0
                const T    t   = (pos ? fabs(tw) : -fabs(tw)) / (fabs(dl) + sqrt(dl * dl + tw * tw));
                const T    c = arap_rsqrt(t * t + T(1)), sn = t * c;
                for (int r = 0; r < K; ++r) {
                    const T arp = A[r * K + p], arq = A[r * K + q];
                    A[r * K + p] = c * arp - sn * arq;
                    A[r * K + q] = sn * arp + c * arq;
                }
                for (int r = 0; r < K; ++r) {
                    const T apr = A[p * K + r], aqr = A[q * K + r];
                    A[p * K + r] = c * apr - sn * aqr;
                    A[q * K + r] = sn * apr + c * aqr;
                }
                for (int r = 0; r < K; ++r) {
                    const T vrp = V[r * K + p], vrq = V[r * K + q];
                    V[r * K + p] = c * vrp - sn * vrq;
                    V[r * K + q] = sn * vrp + c * vrq;
                }
            }
    }
}

// The rule of project_positive_definite on a face's 9x9 vertex-space
// Hessian H9 = D^T Hu D, with D = d^T (x) I3 (u_k = sum_v d[v][k] x_v): left
// alone when positive diagonally dominant with margin eps; otherwise
// eigenvalues below eps raised to eps and H9 rebuilt.  d's two columns sum
// to zero, so with d = q R2 (Gram-Schmidt, q orthonormal 3x2) H9 = Q M Q^T,
// Q = q (x) I3, M = (R2 (x) I3) Hu (R2^T (x) I3) (6x6); H9's other three
// eigenvalues are 0 (the translations t (x) I3, t = (1,1,1)/sqrt 3).  So the
// 9x9 eigenproblem is M's 6x6 one, and the translations (eigenvalue 0 < eps)
// are always raised to eps: H9' = (QW) diag(max(lambda, eps)) (QW)^T +
// eps (t t^T (x) I3) -- the same matrix as projecting H9 directly.
template <typename T>
__device__ void project_face_hessian(const FaceDeriv<T>& o, T eps, T* H)
{
    bool dd = true;
    for (int i = 0; i < 9 && dd; ++i) {
        T off = 0;
        for (int j = 0; j < 9; ++j)
            if (j != i) off += fabs(H[i * 9 + j]);
        dd = H[i * 9 + i] >= off + eps;
    }
    if (dd) return;
    // d = q R2
    T a[3], b[3], q[3][2];
    for (int v = 0; v < 3; ++v) {
        a[v] = o.d[v][0];
        b[v] = o.d[v][1];
    }
    const T a2 = a[0] * a[0] + a[1] * a[1] + a[2] * a[2], i11 = arap_rsqrt(a2), r11 = a2 * i11;
    for (int v = 0; v < 3; ++v) q[v][0] = a[v] * i11;
    const T r12 = q[0][0] * b[0] + q[1][0] * b[1] + q[2][0] * b[2];
    for (int v = 0; v < 3; ++v) b[v] -= r12 * q[v][0];
    const T b2 = b[0] * b[0] + b[1] * b[1] + b[2] * b[2], i22 = arap_rsqrt(b2), r22 = b2 * i22;
    for (int v = 0; v < 3; ++v) q[v][1] = b[v] * i22;
    const T R[2][2] = {{r11, r12}, {T(0), r22}};
    // M[(m,c),(n,e)] = sum_kl R[m][k] Hu[(k,c),(l,e)] R[n][l]
    T M[36], W[36];
    for (int m = 0; m < 2; ++m)
        for (int c = 0; c < 3; ++c)
            for (int n = 0; n < 2; ++n)
                for (int e = 0; e < 3; ++e) {
                    T acc = 0;
                    for (int k = 0; k < 2; ++k)
                        for (int l = 0; l < 2; ++l)
                            acc += R[m][k] * o.Hu[3 * k + c][3 * l + e] * R[n][l];
                    M[(3 * m + c) * 6 + 3 * n + e] = acc;
                }
    jacobi_eigen<T, 6>(M, W);
    T lam[6];
    for (int j = 0; j < 6; ++j) lam[j] = M[j * 6 + j] < eps ? eps : M[j * 6 + j];
    // QW[(v,c), j] = sum_m q[v][m] W[(m,c), j]
    T QW[54];
    for (int v = 0; v < 3; ++v)
        for (int c = 0; c < 3; ++c)
            for (int j = 0; j < 6; ++j)
                QW[(3 * v + c) * 6 + j] = q[v][0] * W[(0 + c) * 6 + j] + q[v][1] * W[(3 + c) * 6 + j];
    const T et = eps / T(3);
    for (int r = 0; r < 9; ++r)
        for (int cc = r; cc < 9; ++cc) {
            T acc = (r % 3 == cc % 3) ? et : T(0);
            for (int j = 0; j < 6; ++j) acc += QW[r * 6 + j] * lam[j] * QW[cc * 6 + j];
            H[r * 9 + cc] = acc;
            H[cc * 9 + r] = acc;
        }
}

// Projected records: E, dE/du (6), the rest-frame inverse (4), then the
// projected 9x9 vertex-space Hessian's upper triangle (45, row-major).
constexpr int kProjRec = 56;

__host__ __device__ constexpr int upper9(int i, int j) { return i * 9 - i * (i - 1) / 2 + (j - i); }

template <typename T>
__global__ void __launch_bounds__(128) k_arap_face_proj(
    int64_t nf, const int32_t* __restrict__ fv, const T* __restrict__ x,
    const T* __restrict__ minv, T* __restrict__ rec, T* __restrict__ face_E,
    double* __restrict__ part)
{
    __shared__ double s_red[128 / 32];
    double            esum = 0;
    const T           eps  = sizeof(T) == 4 ? T(1e-6) : T(1e-9);
    for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < nf;
         f += (int64_t)gridDim.x * blockDim.x) {
        int32_t v[3];
        T       x9[9], mi[4], area;
        load_face(fv, x, minv, (int32_t)f, v, x9, mi, area);
        FaceDeriv<T> o;
        arap_face<T, true>(x9, mi, area, o);
        T H[81];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                T b[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
                block_of(o, i, j, b);
                for (int a = 0; a < 3; ++a)
                    for (int c = 0; c < 3; ++c) H[(3 * i + a) * 9 + 3 * j + c] = b[3 * a + c];
            }
        project_face_hessian(o, eps, H);
        T* r = rec + (int64_t)kProjRec * f;
        r[0] = o.E;
        for (int i = 0; i < 6; ++i) r[1 + i] = o.gE[i];
        for (int i = 0; i < 4; ++i) r[7 + i] = mi[i];
        for (int i = 0; i < 9; ++i)
            for (int j = i; j < 9; ++j) r[11 + upper9(i, j)] = H[i * 9 + j];
        if (face_E) face_E[f] = o.E;
        esum += (double)o.E;
    }
    const double t = block_sum_d<128>(esum, s_red);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// block (li, lj) of a projected record, accumulated into out (3x3 row-major)
template <typename T>
__device__ __forceinline__ void proj_block(const T* __restrict__ r, int li, int lj, T* out)
{
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const int i = 3 * li + a, j = 3 * lj + c;
            out[3 * a + c] += __ldg(r + 11 + (i <= j ? upper9(i, j) : upper9(j, i)));
        }
}

// One thread per vertex: gradient row and projected Hessian block row, in
// the fan order of k_arap_gather.
template <typename T>
__global__ void __launch_bounds__(128) k_arap_gather_proj(
    int64_t nv, const int32_t* __restrict__ row_ptr, const int32_t* __restrict__ ring_off,
    const int32_t* __restrict__ ring, const int32_t* __restrict__ ring_face,
    const int8_t* __restrict__ bnd, const int32_t* __restrict__ fv, const T* __restrict__ rec,
    T* __restrict__ grad, T* __restrict__ hval)
{
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nv;
         p += (int64_t)gridDim.x * blockDim.x) {
        const int32_t ro = ring_off[p];
        const int32_t k  = ring_off[p + 1] - ro;
        const int32_t nf = bnd[p] ? k - 1 : k;
        const int32_t rp = row_ptr[p];
        T             g[3] = {0, 0, 0}, D[9], carry[9];
#pragma unroll
        for (int i = 0; i < 9; ++i) D[i] = carry[i] = T(0);
        for (int32_t i = 0; i < nf; ++i) {
            const int32_t f    = ring_face[ro + i];
            const int32_t v[3] = {__ldg(fv + 3 * (int64_t)f), __ldg(fv + 3 * (int64_t)f + 1),
                                  __ldg(fv + 3 * (int64_t)f + 2)};
            const T*      r    = rec + (int64_t)kProjRec * f;
            const int     lp   = local_index(v, (int32_t)p);
            // u_k = sum_v d[v][k] x_v: d[1] = mi[0..1], d[2] = mi[2..3], d[0] = -(d[1] + d[2])
            const T m0 = __ldg(r + 7), m1 = __ldg(r + 8), m2 = __ldg(r + 9), m3 = __ldg(r + 10);
            const T d0 = lp == 0 ? -(m0 + m2) : (lp == 1 ? m0 : m2);
            const T d1 = lp == 0 ? -(m1 + m3) : (lp == 1 ? m1 : m3);
#pragma unroll
            for (int c = 0; c < 3; ++c) g[c] += d0 * __ldg(r + 1 + c) + d1 * __ldg(r + 4 + c);
            if (hval) {
                const int li = local_index(v, ring[ro + i]);
                const int lj = local_index(v, ring[ro + (i + 1 < k ? i + 1 : 0)]);
                proj_block(r, lp, lp, D);
                T bi[9];
#pragma unroll
                for (int t = 0; t < 9; ++t) bi[t] = carry[t];
                proj_block(r, lp, li, bi);
                T* slot = hval + 9 * (int64_t)(rp + 1 + i);
#pragma unroll
                for (int t = 0; t < 9; ++t) {
                    slot[t]  = bi[t];
                    carry[t] = T(0);
                }
                proj_block(r, lp, lj, carry);
            }
        }
        if (hval) {
            if (k > 0) {
                T* slot = hval + 9 * (int64_t)(rp + 1 + (bnd[p] ? k - 1 : 0));
                if (bnd[p]) {
#pragma unroll
                    for (int t = 0; t < 9; ++t) slot[t] = carry[t];
                } else {
#pragma unroll
                    for (int t = 0; t < 9; ++t) slot[t] += carry[t];
                }
            }
            T* dslot = hval + 9 * (int64_t)rp;
#pragma unroll
            for (int t = 0; t < 9; ++t) dslot[t] = D[t];
        }
        if (grad) {
#pragma unroll
            for (int c = 0; c < 3; ++c) grad[3 * p + c] = g[c];
        }
    }
}

// ---------------------------------------------------------------------
// Hessian-free products and CG (the reference's eval_matvec and
// CGMatFreeSolver, diff/diff_query_kernel.cuh:26-148 and
// matrix/cg_mat_free_solver.h): y = H(x) v from the face records of x, no
// assembled Hessian.  bc (may be null): constrained vertices get identity
// rows and zero columns, as apply_bc does to an assembled Hessian.
// ---------------------------------------------------------------------

template <typename T>
struct MatFreeArgs
{
    int64_t        nv;
    const int32_t* ring_off;
    const int32_t* ring_face;
    const int8_t*  bnd;
    const int32_t* fv;
    const T*       rec;  // k_arap_face<T, true> records, or projected ones
    const int8_t*  bc;
    const T*       B;
    T*             X;
    T*             R;
    T*             P;
    T*             S;
    double*        part;   // 2 * gridDim
    unsigned*      bar;    // 4
    double*        dstat;  // start, final
    int*           istat;  // iters, converged
    int            max_iter;
    double         abs_tol, rel_tol;
    int*           err;
};

// y = row p of H src (3 values)
template <typename T, bool PROJ>
__device__ __forceinline__ void hvp_row(const MatFreeArgs<T>& a, int64_t p, const T* src, T y[3])
{
    y[0] = y[1] = y[2] = T(0);
    if (a.bc && a.bc[p]) {
#pragma unroll
        for (int c = 0; c < 3; ++c) y[c] = src[3 * p + c];
        return;
    }
    const int32_t ro = a.ring_off[p];
    const int32_t k  = a.ring_off[p + 1] - ro;
    const int32_t nf = a.bnd[p] ? k - 1 : k;
    for (int32_t i = 0; i < nf; ++i) {
        const int32_t f    = a.ring_face[ro + i];
        const int32_t v[3] = {__ldg(a.fv + 3 * (int64_t)f), __ldg(a.fv + 3 * (int64_t)f + 1),
                              __ldg(a.fv + 3 * (int64_t)f + 2)};
        const int     lp   = local_index(v, (int32_t)p);
        FaceDeriv<T>  o;
        if (!PROJ) load_record<T, true>(a.rec, f, o);
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            if (q != lp && a.bc && a.bc[v[q]]) continue;
            T b[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
            if (PROJ) proj_block(a.rec + (int64_t)kProjRec * f, lp, q, b);
            else block_of(o, lp, q, b);
            const T* sv = src + 3 * (int64_t)v[q];
            const T  s0 = sv[0], s1 = sv[1], s2 = sv[2];
#pragma unroll
            for (int r = 0; r < 3; ++r) y[r] += b[3 * r] * s0 + b[3 * r + 1] * s1 + b[3 * r + 2] * s2;
        }
    }
}

template <typename T, bool PROJ>
__global__ void __launch_bounds__(128) k_arap_hvp(MatFreeArgs<T> a, const T* __restrict__ v,
                                                  T* __restrict__ y)
{
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < a.nv;
         p += (int64_t)gridDim.x * blockDim.x) {
        T r[3];
        hvp_row<T, PROJ>(a, p, v, r);
#pragma unroll
        for (int c = 0; c < 3; ++c) y[3 * p + c] = r[c];
    }
}

template <int BT, typename Post>
__device__ __forceinline__ bool mf_sum(float v, double*, GridSum& g, RedSmem& r, Post post)
{
    return grid_sum<BT>(v, g, r, post);
}
template <int BT, typename Post>
__device__ __forceinline__ bool mf_sum(double v, double* s_part, GridSum& g, RedSmem& r, Post post)
{
    return grid_sum_staged<BT>(v, s_part, g, r, post);
}

// Plain CG on H(x) X = B (one cooperative launch, rows = vertices, three
// values per row): the recurrence of the generic solver, S = H r + beta S
// carrying H p, two grid sums per iteration; stops when r.r has fallen
// below abs_tol or by rel_tol from its start, or after max_iter iterations.
template <typename T, bool PROJ, int BT>
__global__ void __launch_bounds__(BT) k_cg_matfree(MatFreeArgs<T> a)
{
    __shared__ RedSmem red;
    __shared__ double  s_part[sizeof(T) == 8 ? BT : 1];
    __shared__ double  s_delta0, s_delta;
    __shared__ T       s_al, s_bt;
    __shared__ int     s_first, s_done, s_it, s_conv;
    const int64_t chunk = (a.nv + gridDim.x - 1) / gridDim.x;
    const int64_t r0    = blockIdx.x * chunk;
    const int64_t r1    = min(a.nv, r0 + chunk);
    GridSum       g{a.bar, a.part, a.err, gridDim.x, 0u, blockIdx.x};
    auto          conv = [&](double d) { return d < a.abs_tol || d / s_delta0 < a.rel_tol; };

    T tp = T(0);
    for (int64_t p = r0 + threadIdx.x; p < r1; p += BT) {
        T y[3];
        hvp_row<T, PROJ>(a, p, a.X, y);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const T r        = a.B[3 * p + c] - y[c];
            a.R[3 * p + c]   = r;
            tp += r * r;
        }
    }
    if (!mf_sum<BT>(tp, s_part, g, red, [&](double t) {
            s_delta0 = s_delta = t;
            s_it               = 0;
            s_conv             = conv(t);
            s_bt               = T(0);
            s_first            = 1;
            s_done             = s_conv || a.max_iter <= 0;
        }))
        return;
    while (!s_done) {
        const T    bt    = s_bt;
        const bool first = s_first != 0;
        tp               = T(0);
        for (int64_t p = r0 + threadIdx.x; p < r1; p += BT) {
            T y[3];
            hvp_row<T, PROJ>(a, p, a.R, y);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const T si     = first ? y[c] : y[c] + bt * a.S[3 * p + c];
                const T pi     = first ? a.R[3 * p + c] : a.R[3 * p + c] + bt * a.P[3 * p + c];
                a.P[3 * p + c] = pi;
                a.S[3 * p + c] = si;
                tp += si * pi;
            }
        }
        if (!mf_sum<BT>(tp, s_part, g, red, [&](double sp) { s_al = (T)(s_delta / sp); })) return;
        const T al = s_al;
        tp         = T(0);
        for (int64_t p = r0 + threadIdx.x; p < r1; p += BT) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                a.X[3 * p + c] += al * a.P[3 * p + c];
                const T r       = a.R[3 * p + c] - al * a.S[3 * p + c];
                a.R[3 * p + c]  = r;
                tp += r * r;
            }
        }
        if (!mf_sum<BT>(tp, s_part, g, red, [&](double dn) {
                if (conv(dn)) {
                    s_delta = dn;
                    s_conv  = 1;
                    s_done  = 1;
                    return;
                }
                const double beta = dn / s_delta;
                s_delta           = dn;
                ++s_it;
                s_bt    = (T)beta;
                s_first = 0;
                s_done  = s_it >= a.max_iter;
            }))
            return;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.dstat[0] = s_delta0;
        a.dstat[1] = s_delta;
        a.istat[0] = s_it;
        a.istat[1] = s_conv;
    }
}

// ---------------------------------------------------------------------
// Block-CSR helpers of the Newton step (diff/newton_solver.h)
// ---------------------------------------------------------------------

// scalar CSR of a DxD-block CSR: scalar row Di+a lists, block by block in
// the block row's order, the D entries (Dj+0..D-1) of each block (i,j).
// One warp per block row: the block row's D scalar rows are one contiguous
// run of D*D*nb output entries, written by consecutive lanes.
template <typename T, int D>
__global__ void k_bcsr_expand(int64_t n, const int32_t* __restrict__ brp,
                              const int32_t* __restrict__ bcol, const T* __restrict__ bval,
                              int32_t* __restrict__ rp, int32_t* __restrict__ col,
                              T* __restrict__ val)
{
    constexpr int DD     = D * D;
    const int     lane   = (int)(threadIdx.x & 31);
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; i < n; i += nwarps) {
        const int32_t b0 = __ldg(brp + i), nb = __ldg(brp + i + 1) - b0;
        const int64_t o0 = DD * (int64_t)b0;  // first entry of scalar row Di
        if (lane < D) rp[D * i + lane] = (int32_t)(o0 + (int64_t)D * lane * nb);
#pragma unroll
        for (int a = 0; a < D; ++a) {
            const int64_t oa = o0 + (int64_t)D * a * nb;
            for (int32_t r = lane; r < D * nb; r += 32) {
                const int32_t t = r / D, c = r - t * D;
                col[oa + r]     = D * __ldg(bcol + b0 + t) + c;
                val[oa + r]     = bval[DD * (int64_t)(b0 + t) + D * a + c];
            }
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) rp[D * n] = DD * __ldg(brp + n);
}

// apply_bc of diff/newton_solver.h on the block form: a constrained block
// row gets the identity as its diagonal block and zero off-diagonal blocks,
// every block (i, j) with j constrained is zeroed (the symmetric entries),
// and the constrained rows of the gradient are zeroed.
template <typename T, int D>
__global__ void k_bcsr_apply_bc(int64_t n, const int32_t* __restrict__ brp,
                                const int32_t* __restrict__ bcol, T* __restrict__ bval,
                                const int8_t* __restrict__ bc, T* __restrict__ grad)
{
    constexpr int DD = D * D;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const bool ci = bc[i] != 0;
        for (int32_t t = brp[i]; t < brp[i + 1]; ++t) {
            const int32_t j = bcol[t];
            T*            b = bval + DD * (int64_t)t;
            if (j == i) {
                if (ci)
#pragma unroll
                    for (int e = 0; e < DD; ++e) b[e] = (e % (D + 1) == 0) ? T(1) : T(0);
            } else if (ci || bc[j] != 0) {
#pragma unroll
                for (int e = 0; e < DD; ++e) b[e] = T(0);
            }
        }
        if (ci && grad)
#pragma unroll
            for (int c = 0; c < D; ++c) grad[D * i + c] = T(0);
    }
}

__global__ void k_sum_partials(const double* __restrict__ part, int n, double* __restrict__ out)
{
    double v = 0;
    for (int i = threadIdx.x; i < n; i += 32) v += part[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) out[0] = v;
}

}  // namespace rxg


using namespace rxg;

extern "C" {

rxg_status rxg_arap_rest(const rxg_mesh* h, const double* xyz_rest, int32_t dtype, void* rest,
                         void* stream)
{
    if (!h || !xyz_rest || !rest || (dtype != RXG_F32 && dtype != RXG_F64)) {
        set_error("rxg_arap_rest: bad argument");
        return RXG_ERR_INVALID;
    }
    if (!is_device_ptr(xyz_rest) || !is_device_ptr(rest)) {
        set_error("rxg_arap_rest: xyz_rest and rest must be device arrays");
        return RXG_ERR_INVALID;
    }
    const Mesh&  M = h->m;
    cudaStream_t s = (cudaStream_t)stream;
    const int    g = grid_for_items(M.nf);
    if (dtype == RXG_F64)
        k_arap_rest<double><<<g, 256, 0, s>>>(M.nf, M.d.fv_lin, xyz_rest, (double*)rest);
    else
        k_arap_rest<float><<<g, 256, 0, s>>>(M.nf, M.d.fv_lin, xyz_rest, (float*)rest);
    RXG_CUDA_TRY(cudaGetLastError());
    return RXG_OK;
}

rxg_status rxg_arap_eval(const rxg_mesh* h, int32_t dtype, const void* x, const void* rest,
                         double* energy, void* face_E, void* grad, rxg_bcsr* hess, void* stream)
{
    return rxg_arap_eval_ex(h, dtype, x, rest, 0, energy, face_E, grad, hess, stream);
}

rxg_status rxg_arap_eval_ex(const rxg_mesh* h, int32_t dtype, const void* x, const void* rest,
                            int32_t flags, double* energy, void* face_E, void* grad,
                            rxg_bcsr* hess, void* stream)
{
    if (!h || !x || !rest || (dtype != RXG_F32 && dtype != RXG_F64)) {
        set_error("rxg_arap_eval: bad argument");
        return RXG_ERR_INVALID;
    }
    if (hess && (!hess->row_ptr || !hess->col || !hess->val || hess->dtype != dtype ||
                 (hess->block_dim != 0 && hess->block_dim != 3))) {
        set_error("rxg_arap_eval: hess needs row_ptr, col, val of the same dtype and 3x3 blocks");
        return RXG_ERR_INVALID;
    }
    if (!is_device_ptr(x) || !is_device_ptr(rest) || (grad && !is_device_ptr(grad)) ||
        (face_E && !is_device_ptr(face_E)) || (hess && !is_device_ptr(hess->val))) {
        set_error("rxg_arap_eval: x, rest, grad, face_E and hess must be device arrays");
        return RXG_ERR_INVALID;
    }
    cudaStream_t s = (cudaStream_t)stream;
    Lazy*        z;
    rxg_status   st = ensure_pattern(&h->m, s, &z);
    if (st) return st;
    const int64_t nv = h->m.nv;
    if (hess) {
        hess->n   = nv;
        hess->nnzb = z->nnz;
        RXG_CUDA_TRY(cudaMemcpyAsync(hess->row_ptr, z->row_ptr, 4 * (nv + 1), cudaMemcpyDeviceToDevice, s));
        RXG_CUDA_TRY(cudaMemcpyAsync(hess->col, z->col, 4 * z->nnz, cudaMemcpyDeviceToDevice, s));
    }
    const Mesh&   M  = h->m;
    const int64_t nf = M.nf;
    const int     G  = std::min<int>(grid_for_items(nv) * 2, 152 * 16);
    const int     GF = std::min<int>(grid_for_items(nf) * 2, 152 * 16);
    // FP32: one thread per vertex evaluating its fan (cheap FP32 arithmetic,
    // no record traffic).  FP64 (bound by the FP64 pipe): each face evaluated
    // once into a global record, then the vertex gather.
    // Projected Hessians (flags & RXG_ARAP_PROJECT_HESSIAN, with a Hessian
    // requested): each face evaluated and projected once into a global
    // record, in either precision.
    const bool    f64  = dtype == RXG_F64;
    const bool    proj = hess && (flags & RXG_ARAP_PROJECT_HESSIAN);
    const int     NP   = (f64 || proj) ? GF : G;  // energy partials
    double*       part;
    void*         rec = nullptr;
    RXG_CUDA_TRY(scratch_alloc((void**)&part, sizeof(double) * (NP + 1), s));
    if (proj) {
        const size_t rb = (size_t)nf * kProjRec * (f64 ? 8 : 4);
        cudaError_t  ea = scratch_alloc(&rec, rb, s);
        if (ea != cudaSuccess) {
            cudaFreeAsync(part, s);
            return cuda_status(ea, "rxg_arap_eval: face records");
        }
    } else if (f64) {
        const size_t rb = (size_t)nf * (hess ? rec_words<true>() : rec_words<false>()) * 8;
        cudaError_t  ea = scratch_alloc(&rec, rb, s);
        if (ea != cudaSuccess) {
            cudaFreeAsync(part, s);
            return cuda_status(ea, "rxg_arap_eval: face records");
        }
    }
    cudaError_t e = cudaSuccess;
    auto launch = [&](auto tag, auto hs) {
        using T         = decltype(tag);
        constexpr bool H = decltype(hs)::value;
        T* hv            = hess ? (T*)hess->val : nullptr;
        if constexpr (std::is_same<T, float>::value) {
            k_arap_vertex<T, H><<<G, 128, 0, s>>>(nv, z->row_ptr, z->ring_off, z->ring,
                                                  z->ring_face, z->bnd, M.d.fv_lin, (const T*)x,
                                                  (const T*)rest, (T*)face_E, (T*)grad, hv, part);
        } else {
            k_arap_face<T, H><<<GF, 128, 0, s>>>(nf, M.d.fv_lin, (const T*)x, (const T*)rest,
                                                 (T*)rec, (T*)face_E, part);
            k_arap_gather<T, H><<<G, 128, 0, s>>>(nv, z->row_ptr, z->ring_off, z->ring,
                                                  z->ring_face, z->bnd, M.d.fv_lin, (const T*)rec,
                                                  (T*)grad, hv);
        }
    };
    auto launch_proj = [&](auto tag) {
        using T = decltype(tag);
        k_arap_face_proj<T><<<GF, 128, 0, s>>>(nf, M.d.fv_lin, (const T*)x, (const T*)rest,
                                              (T*)rec, (T*)face_E, part);
        k_arap_gather_proj<T><<<G, 128, 0, s>>>(nv, z->row_ptr, z->ring_off, z->ring,
                                               z->ring_face, z->bnd, M.d.fv_lin, (const T*)rec,
                                               (T*)grad, (T*)hess->val);
    };
    if (proj) {
        if (f64) launch_proj(double{});
        else launch_proj(float{});
    } else if (dtype == RXG_F64) {
        if (hess) launch(double{}, std::true_type{});
        else launch(double{}, std::false_type{});
    } else {
        if (hess) launch(float{}, std::true_type{});
        else launch(float{}, std::false_type{});
    }
    k_sum_partials<<<1, 32, 0, s>>>(part, NP, part + NP);
    if (rec) cudaFreeAsync(rec, s);
    e = cudaGetLastError();
    if (e == cudaSuccess && energy) {
        if (is_device_ptr(energy))
            e = cudaMemcpyAsync(energy, part + NP, sizeof(double), cudaMemcpyDeviceToDevice, s);
        else {
            e = cudaMemcpyAsync(energy, part + NP, sizeof(double), cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        }
    }
    cudaFreeAsync(part, s);
    if (e != cudaSuccess) return cuda_status(e, "rxg_arap_eval");
    return RXG_OK;
}

}  // extern "C"

namespace rxg {

// Shared set-up of the matrix-free entry points: checks, the ring, and the
// face records of x (projected ones with RXG_ARAP_PROJECT_HESSIAN).
struct MatFree
{
    Lazy*   z    = nullptr;
    void*   rec  = nullptr;
    double* part = nullptr;
    cudaStream_t s = nullptr;
    ~MatFree()
    {
        if (rec) cudaFreeAsync(rec, s);
        if (part) cudaFreeAsync(part, s);
    }
};

static rxg_status matfree_setup(const rxg_mesh* h, int32_t dtype, const void* x, const void* rest,
                                int32_t flags, cudaStream_t s, MatFree& mf, const char* who)
{
    if (!h || !x || !rest || (dtype != RXG_F32 && dtype != RXG_F64)) {
        set_error("%s: bad argument", who);
        return RXG_ERR_INVALID;
    }
    if (!is_device_ptr(x) || !is_device_ptr(rest)) {
        set_error("%s: x and rest must be device arrays", who);
        return RXG_ERR_INVALID;
    }
    mf.s          = s;
    rxg_status st = ensure_pattern(&h->m, s, &mf.z);
    if (st) return st;
    const Mesh&   M    = h->m;
    const int64_t nf   = M.nf;
    const bool    proj = (flags & RXG_ARAP_PROJECT_HESSIAN) != 0;
    const size_t  ts   = dtype == RXG_F64 ? 8 : 4;
    const int     GF   = std::min<int>(grid_for_items(nf) * 2, 152 * 16);
    RXG_CUDA_TRY(scratch_alloc((void**)&mf.part, sizeof(double) * (GF + 1), s));
    RXG_CUDA_TRY(scratch_alloc(&mf.rec, (size_t)nf * (proj ? kProjRec : rec_words<true>()) * ts, s));
    auto run = [&](auto tag) {
        using T = decltype(tag);
        if (proj)
            k_arap_face_proj<T><<<GF, 128, 0, s>>>(nf, M.d.fv_lin, (const T*)x, (const T*)rest,
                                                  (T*)mf.rec, nullptr, mf.part);
        else
            k_arap_face<T, true><<<GF, 128, 0, s>>>(nf, M.d.fv_lin, (const T*)x, (const T*)rest,
                                                    (T*)mf.rec, nullptr, mf.part);
    };
    if (dtype == RXG_F64) run(double{});
    else run(float{});
    RXG_CUDA_TRY(cudaGetLastError());
    return RXG_OK;
}

template <typename T>
static MatFreeArgs<T> matfree_args(const rxg_mesh* h, const MatFree& mf, const int8_t* bc)
{
    MatFreeArgs<T> a{};
    a.nv        = h->m.nv;
    a.ring_off  = mf.z->ring_off;
    a.ring_face = mf.z->ring_face;
    a.bnd       = mf.z->bnd;
    a.fv        = h->m.d.fv_lin;
    a.rec       = (const T*)mf.rec;
    a.bc        = bc;
    a.err       = device_error_word();
    return a;
}

template <typename T, bool PROJ>
static rxg_status cg_matfree_launch(MatFreeArgs<T> a, const rxg_solver_opts& o,
                                    rxg_solver_stats* st, cudaStream_t s)
{
    constexpr int BT   = 256;
    auto          kern = k_cg_matfree<T, PROJ, BT>;
    int           per  = 0;
    RXG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, BT, 0));
    int dev = 0, sms = 0;
    RXG_CUDA_TRY(cudaGetDevice(&dev));
    RXG_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int64_t G = std::max<int64_t>(
        1, std::min<int64_t>((int64_t)sms * std::max(1, std::min(per, 4)), (a.nv + 31) / 32));
    const size_t vb    = ((sizeof(T) * 3 * (size_t)a.nv) + 255) & ~size_t(255);
    const size_t bytes = 3 * vb + ((sizeof(double) * 2 * G + 255) & ~size_t(255)) + 3 * 256;
    uint8_t*     q     = nullptr;
    RXG_CUDA_TRY(scratch_alloc((void**)&q, bytes, s));
    uint8_t* base = q;
    a.R     = (T*)q, q += vb;
    a.P     = (T*)q, q += vb;
    a.S     = (T*)q, q += vb;
    a.part  = (double*)q, q += (sizeof(double) * 2 * G + 255) & ~size_t(255);
    a.bar   = (unsigned*)q, q += 256;
    a.dstat = (double*)q, q += 256;
    a.istat = (int*)q;
    a.max_iter = o.max_iter;
    a.abs_tol  = o.abs_tol;
    a.rel_tol  = o.rel_tol;
    cudaError_t e = cudaMemsetAsync(a.bar, 0, 16, s);
    void*       args[] = {&a};
    if (e == cudaSuccess)
        e = cudaLaunchCooperativeKernel((const void*)kern, dim3((unsigned)G), dim3(BT), args, 0, s);
    double ds[2] = {0, 0};
    int    is[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(ds, a.dstat, sizeof(ds), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(is, a.istat, sizeof(is), cudaMemcpyDeviceToHost, s);
    cudaFreeAsync(base, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_status(e, "rxg_arap_cg_matfree");
    rxg_status ce = check_device_error(s);
    if (ce) return ce;
    if (st) {
        st->start_res = ds[0];
        st->final_res = ds[1];
        st->iters     = is[0];
        st->converged = is[1];
    }
    return is[1] ? RXG_OK : RXG_ERR_NOT_CONVERGED;
}

}  // namespace rxg

extern "C" {

rxg_status rxg_arap_hvp(const rxg_mesh* h, int32_t dtype, const void* x, const void* rest,
                        int32_t flags, const int8_t* bc, const void* v, void* y, void* stream)
{
    cudaStream_t s = (cudaStream_t)stream;
    if (!v || !y || !is_device_ptr(v) || !is_device_ptr(y) || (bc && !is_device_ptr(bc))) {
        set_error("rxg_arap_hvp: v, y (and bc) must be device arrays");
        return RXG_ERR_INVALID;
    }
    MatFree    mf;
    rxg_status st = matfree_setup(h, dtype, x, rest, flags, s, mf, "rxg_arap_hvp");
    if (st) return st;
    const bool proj = (flags & RXG_ARAP_PROJECT_HESSIAN) != 0;
    const int  g    = grid_for_items(h->m.nv);
    auto       run  = [&](auto tag) {
        using T = decltype(tag);
        auto a  = matfree_args<T>(h, mf, bc);
        if (proj) k_arap_hvp<T, true><<<g, 128, 0, s>>>(a, (const T*)v, (T*)y);
        else k_arap_hvp<T, false><<<g, 128, 0, s>>>(a, (const T*)v, (T*)y);
    };
    if (dtype == RXG_F64) run(double{});
    else run(float{});
    RXG_CUDA_TRY(cudaGetLastError());
    return RXG_OK;
}

rxg_status rxg_arap_cg_matfree(const rxg_mesh* h, int32_t dtype, const void* x, const void* rest,
                               int32_t flags, const int8_t* bc, const void* B, void* X,
                               const rxg_solver_opts* opts, rxg_solver_stats* stats, void* stream)
{
    cudaStream_t s = (cudaStream_t)stream;
    if (!opts || opts->max_iter < 0 || !B || !X || !is_device_ptr(B) || !is_device_ptr(X) ||
        (bc && !is_device_ptr(bc))) {
        set_error("rxg_arap_cg_matfree: bad argument (B, X, bc must be device arrays)");
        return RXG_ERR_INVALID;
    }
    if (opts->precond) {
        set_error("rxg_arap_cg_matfree: the matrix-free CG has no preconditioner (precond = 0)");
        return RXG_ERR_INVALID;
    }
    MatFree    mf;
    rxg_status st = matfree_setup(h, dtype, x, rest, flags, s, mf, "rxg_arap_cg_matfree");
    if (st) return st;
    const bool proj = (flags & RXG_ARAP_PROJECT_HESSIAN) != 0;
    if (dtype == RXG_F64) {
        auto a = matfree_args<double>(h, mf, bc);
        a.B    = (const double*)B;
        a.X    = (double*)X;
        return proj ? cg_matfree_launch<double, true>(a, *opts, stats, s)
                    : cg_matfree_launch<double, false>(a, *opts, stats, s);
    }
    auto a = matfree_args<float>(h, mf, bc);
    a.B    = (const float*)B;
    a.X    = (float*)X;
    return proj ? cg_matfree_launch<float, true>(a, *opts, stats, s)
                : cg_matfree_launch<float, false>(a, *opts, stats, s);
}

rxg_status rxg_bcsr_to_csr(const rxg_bcsr* H, rxg_csr* out, void* stream)
{
    if (!H || !out || !H->row_ptr || !H->col || !H->val || !out->row_ptr || !out->col ||
        !out->val || (H->dtype != RXG_F32 && H->dtype != RXG_F64)) {
        set_error("rxg_bcsr_to_csr: bad argument");
        return RXG_ERR_INVALID;
    }
    if (9 * H->nnzb > (int64_t)INT32_MAX || 3 * H->n > (int64_t)INT32_MAX) {
        set_error("rxg_bcsr_to_csr: %lld blocks exceed 32-bit scalar indices", (long long)H->nnzb);
        return RXG_ERR_INVALID;
    }
    if (H->block_dim < 0 || H->block_dim > 3) {
        set_error("rxg_bcsr_to_csr: block_dim must be 1, 2 or 3");
        return RXG_ERR_INVALID;
    }
    const int    D = H->block_dim == 0 ? 3 : H->block_dim;
    cudaStream_t s = (cudaStream_t)stream;
    out->n         = D * H->n;
    out->nnz       = (int64_t)D * D * H->nnzb;
    out->dtype     = H->dtype;
    if (H->n == 0) return RXG_OK;
    const int g   = grid_for_items(32 * H->n);  // one warp per block row
    auto      run = [&](auto tag, auto dtag) {
        using T         = decltype(tag);
        constexpr int B = decltype(dtag)::value;
        k_bcsr_expand<T, B><<<g, 256, 0, s>>>(H->n, H->row_ptr, H->col, (const T*)H->val, out->row_ptr,
                                                   out->col, (T*)out->val);
    };
    using C1 = std::integral_constant<int, 1>;
    using C2 = std::integral_constant<int, 2>;
    using C3 = std::integral_constant<int, 3>;
    if (H->dtype == RXG_F64) {
        if (D == 1) run(double{}, C1{});
        else if (D == 2) run(double{}, C2{});
        else run(double{}, C3{});
    } else {
        if (D == 1) run(float{}, C1{});
        else if (D == 2) run(float{}, C2{});
        else run(float{}, C3{});
    }
    RXG_CUDA_TRY(cudaGetLastError());
    return RXG_OK;
}

rxg_status rxg_bcsr_apply_bc(rxg_bcsr* H, const int8_t* bc, void* grad, void* stream)
{
    if (!H || !bc || !H->row_ptr || !H->col || !H->val ||
        (H->dtype != RXG_F32 && H->dtype != RXG_F64)) {
        set_error("rxg_bcsr_apply_bc: bad argument");
        return RXG_ERR_INVALID;
    }
    if (H->block_dim < 0 || H->block_dim > 3) {
        set_error("rxg_bcsr_apply_bc: block_dim must be 1, 2 or 3");
        return RXG_ERR_INVALID;
    }
    cudaStream_t s = (cudaStream_t)stream;
    if (H->n == 0) return RXG_OK;
    const int D   = H->block_dim == 0 ? 3 : H->block_dim;
    const int g   = grid_for_items(H->n);
    auto      run = [&](auto tag, auto dtag) {
        using T         = decltype(tag);
        constexpr int B = decltype(dtag)::value;
        k_bcsr_apply_bc<T, B><<<g, 256, 0, s>>>(H->n, H->row_ptr, H->col, (T*)H->val, bc, (T*)grad);
    };
    using C1 = std::integral_constant<int, 1>;
    using C2 = std::integral_constant<int, 2>;
    using C3 = std::integral_constant<int, 3>;
    if (H->dtype == RXG_F64) {
        if (D == 1) run(double{}, C1{});
        else if (D == 2) run(double{}, C2{});
        else run(double{}, C3{});
    } else {
        if (D == 1) run(float{}, C1{});
        else if (D == 2) run(float{}, C2{});
        else run(float{}, C3{});
    }
    RXG_CUDA_TRY(cudaGetLastError());
    return RXG_OK;
}

}  // extern "C"
