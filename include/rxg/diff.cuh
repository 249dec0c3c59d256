// rxg/diff.cuh -- per-element energies with forward-mode derivatives (nvcc).
//
// The generic term machinery of RXMesh's DiffScalarProblem
// (include/rxmesh/diff/diff_scalar_problem.h:127-194: add_term<Op, Project>
// (lambda) over the TinyAD-style Scalar<T, k, Hess> of diff/scalar.h), of
// this library's own design:
//   Scalar<T, K, HESS>   value, gradient (K) and Hessian (K x K, stored as
//                        its packed upper triangle) of a function of K
//                        variables, propagated by the chain rule through
//                        + - * / and the elementary functions below
//   Vec2 / Mat2 helpers  2x2 matrices of Scalars: col_mat, det, inverse,
//                        squared_norm (the Eigen calls of the reference's
//                        energies)
//   write_term_record    one face's energy, gradient and (projected)
//                        Hessian in the record layout rxg_face_term_gather
//                        reads: [E, g_0..g_{K-1}, H upper triangle row-major]
//   face_term_kernel     runs an energy functor over every face with the
//                        face's 3 vertices x D components as the K = 3D
//                        active variables, writing the records
//   edge_term_kernel,    the same over every edge (K = 2D, the edge's two
//   vertex_term_kernel   ends in EV order) and every vertex (K = D)
// An application compiles its energy with this header and hands the records
// to rxg_face_term_gather / rxg_edge_term_gather / rxg_vertex_term_gather
// (librxg.so), which assemble the gradient and the D x D block Hessian over
// the mesh's [diagonal, one-ring] pattern.
#pragma once

#include <cuda_runtime.h>
#include <float.h>
#include <math.h>
#include <stdint.h>

#if defined(__CUDACC__)
#define RXG_DIFF_HD __host__ __device__ __forceinline__
#else
#define RXG_DIFF_HD inline
#endif

namespace rxg {

// index of (i, j), i <= j, in the packed upper triangle of a K x K matrix
template <int K>
RXG_DIFF_HD constexpr int upper_index(int i, int j)
{
    return i * K - i * (i - 1) / 2 + (j - i);
}

template <typename T, int K, bool HESS = true>
struct Scalar
{
    static constexpr int kVars = K;
    static constexpr int kHess = HESS ? K * (K + 1) / 2 : 0;
    using PassiveT             = T;

    T val;
    T grad[K];
    T hess[kHess > 0 ? kHess : 1];

    RXG_DIFF_HD Scalar() : Scalar(T(0)) {}
    // a constant (passive) value
    RXG_DIFF_HD Scalar(T v) : val(v)
    {
        for (int i = 0; i < K; ++i) grad[i] = T(0);
        for (int i = 0; i < kHess; ++i) hess[i] = T(0);
    }
    // the variable number i with value v
    static RXG_DIFF_HD Scalar make_active(T v, int i)
    {
        Scalar s(v);
        s.grad[i] = T(1);
        return s;
    }
    RXG_DIFF_HD T hessian(int i, int j) const
    {
        if constexpr (HESS)
            return i <= j ? hess[upper_index<K>(i, j)] : hess[upper_index<K>(j, i)];
        else
            return T(0);
    }

    // f(a) with f = fa, f' = d1, f'' = d2 at a.val (the chain rule)
    static RXG_DIFF_HD Scalar chain(const Scalar& a, T fa, T d1, T d2)
    {
        Scalar r(fa);
        for (int i = 0; i < K; ++i) r.grad[i] = d1 * a.grad[i];
        if constexpr (HESS)
            for (int i = 0; i < K; ++i)
                for (int j = i; j < K; ++j)
                    r.hess[upper_index<K>(i, j)] =
                        d1 * a.hess[upper_index<K>(i, j)] + d2 * a.grad[i] * a.grad[j];
        return r;
    }

    RXG_DIFF_HD Scalar& operator+=(const Scalar& b)
    {
        val += b.val;
        for (int i = 0; i < K; ++i) grad[i] += b.grad[i];
        for (int i = 0; i < kHess; ++i) hess[i] += b.hess[i];
        return *this;
    }
    RXG_DIFF_HD Scalar& operator-=(const Scalar& b)
    {
        val -= b.val;
        for (int i = 0; i < K; ++i) grad[i] -= b.grad[i];
        for (int i = 0; i < kHess; ++i) hess[i] -= b.hess[i];
        return *this;
    }
    RXG_DIFF_HD Scalar& operator*=(T s)
    {
        val *= s;
        for (int i = 0; i < K; ++i) grad[i] *= s;
        for (int i = 0; i < kHess; ++i) hess[i] *= s;
        return *this;
    }
    RXG_DIFF_HD Scalar& operator+=(T s)
    {
        val += s;
        return *this;
    }
};

template <typename T, int K, bool H>
RXG_DIFF_HD Scalar<T, K, H> operator+(Scalar<T, K, H> a, const Scalar<T, K, H>& b)
{
    return a += b;
}
template <typename T, int K, bool H>
RXG_DIFF_HD Scalar<T, K, H> operator-(Scalar<T, K, H> a, const Scalar<T, K, H>& b)
{
    return a -= b;
}
template <typename T, int K, bool H>
RXG_DIFF_HD Scalar<T, K, H> operator-(Scalar<T, K, H> a)
{
    return a *= T(-1);
}
template <typename T, int K, bool H>
RXG_DIFF_HD Scalar<T, K, H> operator+(Scalar<T, K, H> a, T s)
{
    return a += s;
}
template <typename T, int K, bool H>
RXG_DIFF_HD Scalar<T, K, H> operator+(T s, Scalar<T, K, H> a)
{
    return a += s;
}
template <typename T, int K, bool H>
RXG_DIFF_HD Scalar<T, K, H> operator-(Scalar<T, K, H> a, T s)
{
    return a += -s;
}
template <typename T, int K, bool H>
RXG_DIFF_HD Scalar<T, K, H> operator-(T s, Scalar<T, K, H> a)
{
    a *= T(-1);
    return a += s;
}
template <typename T, int K, bool H>
RXG_DIFF_HD Scalar<T, K, H> operator*(Scalar<T, K, H> a, T s)
{
    return a *= s;
}
template <typename T, int K, bool H>
RXG_DIFF_HD Scalar<T, K, H> operator*(T s, Scalar<T, K, H> a)
{
    return a *= s;
}
// product rule: (ab)'' = a b'' + b a'' + a' b'^T + b' a'^T
template <typename T, int K, bool H>
RXG_DIFF_HD Scalar<T, K, H> operator*(const Scalar<T, K, H>& a, const Scalar<T, K, H>& b)
{
    Scalar<T, K, H> r(a.val * b.val);
    for (int i = 0; i < K; ++i) r.grad[i] = a.val * b.grad[i] + b.val * a.grad[i];
    if constexpr (H)
        for (int i = 0; i < K; ++i)
            for (int j = i; j < K; ++j) {
                const int u = upper_index<K>(i, j);
                r.hess[u]   = a.val * b.hess[u] + b.val * a.hess[u] + a.grad[i] * b.grad[j] +
                            b.grad[i] * a.grad[j];
            }
    return r;
}
// 1/b: f' = -1/b^2, f'' = 2/b^3
template <typename T, int K, bool H>
RXG_DIFF_HD Scalar<T, K, H> inv(const Scalar<T, K, H>& b)
{
    const T i = T(1) / b.val;
    return Scalar<T, K, H>::chain(b, i, -i * i, T(2) * i * i * i);
}
template <typename T, int K, bool H>
RXG_DIFF_HD Scalar<T, K, H> operator/(const Scalar<T, K, H>& a, const Scalar<T, K, H>& b)
{
    return a * inv(b);
}
template <typename T, int K, bool H>
RXG_DIFF_HD Scalar<T, K, H> operator/(Scalar<T, K, H> a, T s)
{
    return a *= T(1) / s;
}
template <typename T, int K, bool H>
RXG_DIFF_HD Scalar<T, K, H> operator/(T s, const Scalar<T, K, H>& b)
{
    return inv(b) * s;
}
template <typename T, int K, bool H>
RXG_DIFF_HD Scalar<T, K, H> sqr(const Scalar<T, K, H>& a)
{
    return Scalar<T, K, H>::chain(a, a.val * a.val, T(2) * a.val, T(2));
}
template <typename T, int K, bool H>
RXG_DIFF_HD Scalar<T, K, H> sqrt(const Scalar<T, K, H>& a)
{
    const T s = ::sqrt(a.val);
    return Scalar<T, K, H>::chain(a, s, T(0.5) / s, T(-0.25) / (s * a.val));
}
template <typename T, int K, bool H>
RXG_DIFF_HD Scalar<T, K, H> log(const Scalar<T, K, H>& a)
{
    const T i = T(1) / a.val;
    return Scalar<T, K, H>::chain(a, ::log(a.val), i, -i * i);
}
template <typename T, int K, bool H>
RXG_DIFF_HD Scalar<T, K, H> exp(const Scalar<T, K, H>& a)
{
    const T e = ::exp(a.val);
    return Scalar<T, K, H>::chain(a, e, e, e);
}
// a^p for a constant exponent p
template <typename T, int K, bool H>
RXG_DIFF_HD Scalar<T, K, H> pow(const Scalar<T, K, H>& a, T p)
{
    const T f = ::pow(a.val, p);
    return Scalar<T, K, H>::chain(a, f, p * f / a.val, p * (p - T(1)) * f / (a.val * a.val));
}
template <typename T, int K, bool H>
RXG_DIFF_HD bool operator<(const Scalar<T, K, H>& a, T b) { return a.val < b; }
template <typename T, int K, bool H>
RXG_DIFF_HD bool operator<=(const Scalar<T, K, H>& a, T b) { return a.val <= b; }
template <typename T, int K, bool H>
RXG_DIFF_HD bool operator>(const Scalar<T, K, H>& a, T b) { return a.val > b; }
template <typename T, int K, bool H>
RXG_DIFF_HD bool operator>=(const Scalar<T, K, H>& a, T b) { return a.val >= b; }

// the passive value of a Scalar or of a plain number
template <typename T>
RXG_DIFF_HD T passive(T v) { return v; }
template <typename T, int K, bool H>
RXG_DIFF_HD T passive(const Scalar<T, K, H>& v) { return v.val; }

// ---- 2-vectors and 2x2 matrices (column-major: m[col][row]) ----------

template <typename S>
struct Vec2
{
    S x, y;
};
template <typename S>
RXG_DIFF_HD Vec2<S> operator-(const Vec2<S>& a, const Vec2<S>& b)
{
    return {a.x - b.x, a.y - b.y};
}

template <typename S>
struct Mat2
{
    S a, b, c, d;  // [[a, b], [c, d]] (row-major entries)
};
// the 2x2 matrix with u and v as its columns (col_mat)
template <typename S>
RXG_DIFF_HD Mat2<S> col_mat(const Vec2<S>& u, const Vec2<S>& v)
{
    return {u.x, v.x, u.y, v.y};
}
template <typename S>
RXG_DIFF_HD S det(const Mat2<S>& m)
{
    return m.a * m.d - m.b * m.c;
}
template <typename S>
RXG_DIFF_HD Mat2<S> inverse(const Mat2<S>& m)
{
    const S id = S(1) / det(m);
    return {m.d * id, -(m.b * id), -(m.c * id), m.a * id};
}
template <typename S>
RXG_DIFF_HD S squared_norm(const Mat2<S>& m)
{
    return m.a * m.a + m.b * m.b + m.c * m.c + m.d * m.d;
}
// active matrix times a passive one
template <typename S, typename T>
RXG_DIFF_HD Mat2<S> mul(const Mat2<S>& m, const Mat2<T>& r)
{
    return {m.a * r.a + m.b * r.c, m.a * r.b + m.b * r.d, m.c * r.a + m.d * r.c, m.c * r.b + m.d * r.d};
}

// ---- face records -------------------------------------------------------

// words of one face record for D components per vertex (K = 3D variables)
RXG_DIFF_HD constexpr int term_record_words(int D)
{
    return 1 + 3 * D + (3 * D) * (3 * D + 1) / 2;
}
// record words of a term over `corners` vertices of D components (a face
// term: 3; an edge term: 2; a vertex term: 1)
RXG_DIFF_HD constexpr int term_record_words_n(int corners, int D)
{
    return 1 + corners * D + (corners * D) * (corners * D + 1) / 2;
}

// write e's value, gradient and Hessian as a record
template <typename T, int K>
RXG_DIFF_HD void write_term_record(const Scalar<T, K, true>& e, T* rec)
{
    rec[0] = e.val;
    for (int i = 0; i < K; ++i) rec[1 + i] = e.grad[i];
    for (int i = 0; i < K * (K + 1) / 2; ++i) rec[1 + K + i] = e.hess[i];
}

#if defined(__CUDACC__)
__device__ __forceinline__ double term_rsqrt(double x) { return ::rsqrt(x); }
__device__ __forceinline__ float  term_rsqrt(float x) { return ::rsqrtf(x); }

// cyclic Jacobi eigen-decomposition of the symmetric K x K matrix A (row
// major, overwritten by its eigenvalues on the diagonal), V the eigenvectors.
// A rotation's t = sgn(th) / (|th| + sqrt(th^2 + 1)), th = (a_qq - a_pp) /
// (2 a_pq), is formed as sgn(th) |2 a_pq| / (|a_qq - a_pp| + hypot) (one
// division) and c = 1 / sqrt(t^2 + 1) as one reciprocal square root.
template <typename T, int K>
__device__ inline void term_jacobi(T* A, T* V)
{
    for (int i = 0; i < K * K; ++i) V[i] = (i % (K + 1)) == 0 ? T(1) : T(0);
    const T rel = sizeof(T) == 4 ? T(1e-14) : T(1e-30);
    for (int sweep = 0; sweep < 50; ++sweep) {
        T off = 0, all = 0;
        for (int i = 0; i < K * K; ++i) {
            all += A[i] * A[i];
            if (i % (K + 1)) off += A[i] * A[i];
        }
        if (off <= rel * all) break;
        for (int p = 0; p < K - 1; ++p)
            for (int q = p + 1; q < K; ++q) {
                const T apq = A[p * K + q];
                if (apq == T(0)) continue;
                const T    dl  = A[q * K + q] - A[p * K + p], tw = T(2) * apq;
                const bool pos = dl == T(0) || ((dl > T(0)) == (tw > T(0)));  // th >= 0
                const T    t   = (pos ? ::fabs(tw) : -::fabs(tw)) / (::fabs(dl) + ::sqrt(dl * dl + tw * tw));
                const T    c = term_rsqrt(t * t + T(1)), sn = t * c;
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

// project_positive_definite on a packed K x K Hessian, in place: left alone
// when positive diagonally dominant with margin eps, else every eigenvalue
// below eps raised to eps and the matrix rebuilt
template <typename T, int K>
__device__ inline void project_packed(T* hu, T eps)
{
    bool dd = true;
    for (int i = 0; i < K && dd; ++i) {
        T off = 0;
        for (int j = 0; j < K; ++j)
            if (j != i) off += fabs(hu[i <= j ? upper_index<K>(i, j) : upper_index<K>(j, i)]);
        dd = hu[upper_index<K>(i, i)] >= off + eps;
    }
    if (dd) return;
    T A[K * K], V[K * K];
    for (int i = 0; i < K; ++i)
        for (int j = 0; j < K; ++j) A[i * K + j] = hu[i <= j ? upper_index<K>(i, j) : upper_index<K>(j, i)];
    term_jacobi<T, K>(A, V);
    T lam[K];
    for (int j = 0; j < K; ++j) lam[j] = A[j * K + j] < eps ? eps : A[j * K + j];
    for (int i = 0; i < K; ++i)
        for (int j = i; j < K; ++j) {
            T acc = 0;
            for (int m = 0; m < K; ++m) acc += V[i * K + m] * lam[m] * V[j * K + m];
            hu[upper_index<K>(i, j)] = acc;
        }
}

// Evaluate energy(face, v) over every face, where v[k * D + d] is
// component d of the face's corner k (the face's vertices in input order)
// as an active variable; records: nf x term_record_words(D) of T, face
// linear order.  x: nv x D, linear order; fv: nf x 3 linear vertex ids.
// PROJECT: each face's Hessian made positive definite first
// (project_positive_definite; eps 1e-9 FP64, 1e-6 FP32).
template <typename T, int D, bool PROJECT, typename EnergyT>
__global__ void __launch_bounds__(128) face_term_kernel(int64_t nf, const int32_t* __restrict__ fv,
                                                        const T* __restrict__ x, EnergyT energy,
                                                        T* __restrict__ records)
{
    constexpr int K = 3 * D;
    using S         = Scalar<T, K, true>;
    for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < nf;
         f += (int64_t)gridDim.x * blockDim.x) {
        S v[K];
        for (int k = 0; k < 3; ++k) {
            const int32_t vi = fv[3 * f + k];
            for (int d = 0; d < D; ++d) v[k * D + d] = S::make_active(x[(int64_t)vi * D + d], k * D + d);
        }
        S e = energy((int32_t)f, v);
        if (PROJECT) project_packed<T, K>(e.hess, sizeof(T) == 4 ? T(1e-6) : T(1e-9));
        write_term_record<T, K>(e, records + (int64_t)term_record_words(D) * f);
    }
}

// Evaluate energy(edge, v) over every edge, v[k * D + d] component d of the
// edge's end k (its two vertices in EV order) as active variables; records:
// ne x term_record_words_n(2, D), edge linear order.  ev: ne x 2 linear
// vertex ids (the EV query).  add_term<Op::EV> of the reference.
template <typename T, int D, bool PROJECT, typename EnergyT>
__global__ void __launch_bounds__(128) edge_term_kernel(int64_t ne, const int32_t* __restrict__ ev,
                                                        const T* __restrict__ x, EnergyT energy,
                                                        T* __restrict__ records)
{
    constexpr int K = 2 * D;
    using S         = Scalar<T, K, true>;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ne;
         e += (int64_t)gridDim.x * blockDim.x) {
        S v[K];
        for (int k = 0; k < 2; ++k) {
            const int32_t vi = ev[2 * e + k];
            for (int d = 0; d < D; ++d) v[k * D + d] = S::make_active(x[(int64_t)vi * D + d], k * D + d);
        }
        S en = energy((int32_t)e, v);
        if (PROJECT) project_packed<T, K>(en.hess, sizeof(T) == 4 ? T(1e-6) : T(1e-9));
        write_term_record<T, K>(en, records + (int64_t)term_record_words_n(2, D) * e);
    }
}

// Evaluate energy(vertex, v) over every vertex, v[d] its component d as the
// active variables; records: nv x term_record_words_n(1, D), vertex linear
// order.  add_term<Op::V> of the reference.
template <typename T, int D, bool PROJECT, typename EnergyT>
__global__ void __launch_bounds__(128) vertex_term_kernel(int64_t nv, const T* __restrict__ x, EnergyT energy,
                                                          T* __restrict__ records)
{
    using S = Scalar<T, D, true>;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nv;
         i += (int64_t)gridDim.x * blockDim.x) {
        S v[D];
        for (int d = 0; d < D; ++d) v[d] = S::make_active(x[i * D + d], d);
        S en = energy((int32_t)i, v);
        if (PROJECT) project_packed<T, D>(en.hess, sizeof(T) == 4 ? T(1e-6) : T(1e-9));
        write_term_record<T, D>(en, records + (int64_t)term_record_words_n(1, D) * i);
    }
}

inline unsigned term_grid(int64_t n)
{
    const int64_t blocks = (n + 127) / 128;
    return (unsigned)(blocks < 152 * 16 ? blocks : 152 * 16);
}

template <typename T, int D, bool PROJECT, typename EnergyT>
inline cudaError_t launch_edge_term(int64_t ne, const int32_t* ev, const T* x, const EnergyT& energy, T* records,
                                    cudaStream_t stream)
{
    if (ne == 0) return cudaSuccess;
    edge_term_kernel<T, D, PROJECT, EnergyT><<<term_grid(ne), 128, 0, stream>>>(ne, ev, x, energy, records);
    return cudaGetLastError();
}

template <typename T, int D, bool PROJECT, typename EnergyT>
inline cudaError_t launch_vertex_term(int64_t nv, const T* x, const EnergyT& energy, T* records,
                                      cudaStream_t stream)
{
    if (nv == 0) return cudaSuccess;
    vertex_term_kernel<T, D, PROJECT, EnergyT><<<term_grid(nv), 128, 0, stream>>>(nv, x, energy, records);
    return cudaGetLastError();
}

// launch face_term_kernel over nf faces on `stream`
template <typename T, int D, bool PROJECT, typename EnergyT>
inline cudaError_t launch_face_term(int64_t nf, const int32_t* fv, const T* x, const EnergyT& energy,
                                    T* records, cudaStream_t stream)
{
    if (nf == 0) return cudaSuccess;
    const int64_t blocks = (nf + 127) / 128;
    face_term_kernel<T, D, PROJECT, EnergyT>
        <<<(unsigned)(blocks < 152 * 16 ? blocks : 152 * 16), 128, 0, stream>>>(nf, fv, x, energy, records);
    return cudaGetLastError();
}
#endif

}  // namespace rxg
