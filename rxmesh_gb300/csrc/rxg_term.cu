// Generic per-face energy terms (DiffScalarProblem::add_term<Op::FV,
// ProjectHess>, diff/diff_scalar_problem.h:127-194; per-element kernel
// diff/diff_query_kernel.cuh:199-322) on the forward-mode Scalar type of
// include/rxg/diff.cuh.
//
// A term is evaluated face by face into a record [E, gradient (3D),
// Hessian's upper triangle (3D x 3D)], D the components per vertex, optionally
// made positive definite (project_positive_definite, diff/hessian_projection.h:
// 21-95).  rxg_face_term_gather then assembles the records vertex by vertex:
// each vertex walks the faces of its oriented fan and writes its gradient row
// and its D x D Hessian block row [diag, ring...] once (no atomics,
// deterministic).  The records come from the library's built-in terms (the
// symmetric Dirichlet energy of apps/Param/param.cu:146-183) or from an
// application's own kernel compiled with include/rxg/diff.cuh.
#include <algorithm>
#include <cfloat>
#include <type_traits>

#include "../../include/rxg/diff.cuh"
#include "rxg_device.cuh"
#include "rxg_lazy.h"

namespace rxg {

__global__ void k_sum_partials(const double* __restrict__ part, int n, double* __restrict__ out);

template <int BT>
__device__ __forceinline__ double term_block_sum(double v, double* s_red)
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

// ---------------------------------------------------------------------
// Symmetric Dirichlet energy (apps/Param/param.cu:146-183), D = 2: with M =
// [b - a, c - a] the 2x2 matrix of the face's uv edge vectors, Mr its rest
// shape (rest = Mr^{-1}, rxg_arap_rest), A = det(Mr) / 2 and J = M Mr^{-1},
//   E = A (|J|_F^2 + |J^{-1}|_F^2),
// and E = the largest finite value (a constant) when det(M) <= 0 (a flipped
// or degenerate triangle), as the reference returns.
// ---------------------------------------------------------------------

template <typename T>
struct SymDirEnergy
{
    const T* rest;
    template <typename S>
    __device__ S operator()(int32_t f, const S* v) const
    {
        const Vec2<S> a{v[0], v[1]}, b{v[2], v[3]}, c{v[4], v[5]};
        const Mat2<S> M = col_mat(b - a, c - a);
        if (passive(det(M)) <= T(0)) return S(sizeof(T) == 4 ? (T)FLT_MAX : (T)DBL_MAX);
        const Mat2<T> mi{__ldg(rest + 4 * (int64_t)f), __ldg(rest + 4 * (int64_t)f + 1),
                         __ldg(rest + 4 * (int64_t)f + 2), __ldg(rest + 4 * (int64_t)f + 3)};
        const T       A = T(0.5) / (mi.a * mi.d - mi.b * mi.c);  // det(Mr) / 2
        const Mat2<S> J = mul(M, mi);
        return (squared_norm(J) + squared_norm(inverse(J))) * A;
    }
};

// one face record per face from an energy functor (D components per vertex),
// optionally projected; face energies and per-block energy partial sums
template <typename T, int D, bool PROJ, typename EnergyT>
__global__ void __launch_bounds__(128) k_term_face(int64_t nf, const int32_t* __restrict__ fv,
                                                   const T* __restrict__ x, EnergyT energy,
                                                   T* __restrict__ rec, T* __restrict__ face_E,
                                                   double* __restrict__ part)
{
    constexpr int K = 3 * D;
    constexpr int W = term_record_words(D);
    using S         = Scalar<T, K, true>;
    __shared__ double s_red[128 / 32];
    double            esum = 0;
    for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < nf;
         f += (int64_t)gridDim.x * blockDim.x) {
        S v[K];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const int32_t vi = __ldg(fv + 3 * f + k);
#pragma unroll
            for (int d = 0; d < D; ++d) v[k * D + d] = S::make_active(x[(int64_t)vi * D + d], k * D + d);
        }
        S e = energy((int32_t)f, v);
        if (PROJ) project_packed<T, K>(e.hess, sizeof(T) == 4 ? T(1e-6) : T(1e-9));
        write_term_record<T, K>(e, rec + (int64_t)W * f);
        if (face_E) face_E[f] = e.val;
        esum += (double)e.val;
    }
    const double t = term_block_sum<128>(esum, s_red);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// energies of the records (an application's own) into partial sums
template <typename T, int D>
__global__ void __launch_bounds__(128) k_term_energy(int64_t nf, const T* __restrict__ rec,
                                                     T* __restrict__ face_E, double* __restrict__ part)
{
    __shared__ double s_red[128 / 32];
    double            esum = 0;
    for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < nf;
         f += (int64_t)gridDim.x * blockDim.x) {
        const T e = rec[(int64_t)term_record_words(D) * f];
        if (face_E) face_E[f] = e;
        esum += (double)e;
    }
    const double t = term_block_sum<128>(esum, s_red);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// energies of n records of W words into partial sums (and per-element E)
template <typename T, int W>
__global__ void __launch_bounds__(128) k_term_energy_w(int64_t n, const T* __restrict__ rec,
                                                       T* __restrict__ elem_E, double* __restrict__ part)
{
    __shared__ double s_red[128 / 32];
    double            esum = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const T e = rec[(int64_t)W * i];
        if (elem_E) elem_E[i] = e;
        esum += (double)e;
    }
    const double t = term_block_sum<128>(esum, s_red);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// out (D x D row-major) += block (end li, end lj) of a record of C ends
template <typename T, int D, int C>
__device__ __forceinline__ void term_block_c(const T* __restrict__ r, int li, int lj, T* out)
{
    constexpr int K = C * D;
#pragma unroll
    for (int a = 0; a < D; ++a)
#pragma unroll
        for (int c = 0; c < D; ++c) {
            const int i = D * li + a, j = D * lj + c;
            out[D * a + c] += __ldg(r + 1 + K + (i <= j ? upper_index<K>(i, j) : upper_index<K>(j, i)));
        }
}

// For each ring slot of each vertex p, the edge joining p to ring[i] and
// p's end of it, from p's VE row and EV (both computed once for this)
__global__ void k_ring_edge(int64_t nv, const int32_t* __restrict__ ring_off, const int32_t* __restrict__ ring,
                            const int32_t* __restrict__ ve_off, const int32_t* __restrict__ ve,
                            const int32_t* __restrict__ ev, int32_t* __restrict__ ring_edge, int* err)
{
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nv;
         p += (int64_t)gridDim.x * blockDim.x) {
        const int32_t j0 = ve_off[p], j1 = ve_off[p + 1];
        for (int32_t i = ring_off[p]; i < ring_off[p + 1]; ++i) {
            const int32_t r = ring[i];
            int32_t       c = -1;
            for (int32_t j = j0; j < j1 && c < 0; ++j) {
                const int32_t e = ve[j], a = ev[2 * (int64_t)e], b = ev[2 * (int64_t)e + 1];
                if (a == (int32_t)p && b == r) c = 2 * e;
                else if (b == (int32_t)p && a == r) c = 2 * e + 1;
            }
            if (c < 0 && err) atomicOr(err, DEVERR_NONMANIFOLD);
            ring_edge[i] = c < 0 ? 0 : c;
        }
    }
}

// One thread per vertex: the gradient row and the D x D Hessian block row
// [diag, ring...] from the records of the vertex's edges (one per ring
// slot).  ACC: add to grad / hval instead of overwriting them.
template <typename T, int D, bool ACC>
__global__ void __launch_bounds__(128) k_edge_term_gather(int64_t nv, const int32_t* __restrict__ row_ptr,
                                                          const int32_t* __restrict__ ring_off,
                                                          const int32_t* __restrict__ ring_edge,
                                                          const T* __restrict__ rec, T* __restrict__ grad,
                                                          T* __restrict__ hval)
{
    constexpr int W  = term_record_words_n(2, D);
    constexpr int DD = D * D;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nv;
         p += (int64_t)gridDim.x * blockDim.x) {
        const int32_t ro = ring_off[p], k = ring_off[p + 1] - ro, rp = row_ptr[p];
        T             g[D], Dg[DD];
#pragma unroll
        for (int i = 0; i < D; ++i) g[i] = T(0);
#pragma unroll
        for (int i = 0; i < DD; ++i) Dg[i] = T(0);
        for (int32_t i = 0; i < k; ++i) {
            const int32_t c  = __ldg(ring_edge + ro + i);
            const int     lp = c & 1;
            const T*      r  = rec + (int64_t)W * (c >> 1);
#pragma unroll
            for (int t = 0; t < D; ++t) g[t] += __ldg(r + 1 + D * lp + t);
            if (hval) {
                term_block_c<T, D, 2>(r, lp, lp, Dg);
                T bo[DD];
#pragma unroll
                for (int t = 0; t < DD; ++t) bo[t] = T(0);
                term_block_c<T, D, 2>(r, lp, 1 - lp, bo);
                T* slot = hval + DD * (int64_t)(rp + 1 + i);
#pragma unroll
                for (int t = 0; t < DD; ++t) slot[t] = ACC ? slot[t] + bo[t] : bo[t];
            }
        }
        if (hval) {
            T* dslot = hval + DD * (int64_t)rp;
#pragma unroll
            for (int t = 0; t < DD; ++t) dslot[t] = ACC ? dslot[t] + Dg[t] : Dg[t];
        }
        if (grad) {
#pragma unroll
            for (int t = 0; t < D; ++t) grad[D * p + t] = ACC ? grad[D * p + t] + g[t] : g[t];
        }
    }
}

// One thread per vertex: its own record's gradient and diagonal block.  The
// off-diagonal blocks are untouched (the host clears the Hessian when the
// term overwrites it).  ACC: add to grad (else overwrite it).
template <typename T, int D, bool ACC>
__global__ void __launch_bounds__(128) k_vertex_term_gather(int64_t nv, const int32_t* __restrict__ row_ptr,
                                                            const T* __restrict__ rec, T* __restrict__ grad,
                                                            T* __restrict__ hval)
{
    constexpr int W  = term_record_words_n(1, D);
    constexpr int DD = D * D;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nv;
         p += (int64_t)gridDim.x * blockDim.x) {
        const T* r = rec + (int64_t)W * p;
        if (grad) {
#pragma unroll
            for (int t = 0; t < D; ++t) grad[D * p + t] = ACC ? grad[D * p + t] + __ldg(r + 1 + t) : __ldg(r + 1 + t);
        }
        if (hval) {
            T b[DD];
#pragma unroll
            for (int t = 0; t < DD; ++t) b[t] = T(0);
            term_block_c<T, D, 1>(r, 0, 0, b);
            T* dslot = hval + DD * (int64_t)row_ptr[p];
#pragma unroll
            for (int t = 0; t < DD; ++t) dslot[t] += b[t];
        }
    }
}

__device__ __forceinline__ int term_corner(const int32_t v[3], int32_t p)
{
    return v[0] == p ? 0 : (v[1] == p ? 1 : 2);
}

// out (D x D row-major) += the record's block (corner li, corner lj)
template <typename T, int D>
__device__ __forceinline__ void term_block(const T* __restrict__ r, int li, int lj, T* out)
{
    constexpr int K = 3 * D;
#pragma unroll
    for (int a = 0; a < D; ++a)
#pragma unroll
        for (int c = 0; c < D; ++c) {
            const int i = D * li + a, j = D * lj + c;
            out[D * a + c] += __ldg(r + 1 + K + (i <= j ? upper_index<K>(i, j) : upper_index<K>(j, i)));
        }
}

// One thread per vertex: the gradient row and the D x D Hessian block row
// [diag, ring...] from the records of the vertex's fan faces.  ACC: add to
// grad / hval instead of overwriting them.
template <typename T, int D, bool ACC>
__global__ void __launch_bounds__(128) k_term_gather(
    int64_t nv, const int32_t* __restrict__ row_ptr, const int32_t* __restrict__ ring_off,
    const int32_t* __restrict__ ring, const int32_t* __restrict__ ring_face,
    const int8_t* __restrict__ bnd, const int32_t* __restrict__ fv, const T* __restrict__ rec,
    T* __restrict__ grad, T* __restrict__ hval)
{
    constexpr int K  = 3 * D;
    constexpr int W  = term_record_words(D);
    constexpr int DD = D * D;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nv;
         p += (int64_t)gridDim.x * blockDim.x) {
        const int32_t ro = ring_off[p];
        const int32_t k  = ring_off[p + 1] - ro;
        const int32_t nf = bnd[p] ? k - 1 : k;
        const int32_t rp = row_ptr[p];
        T             g[D], Dg[DD], carry[DD];
#pragma unroll
        for (int i = 0; i < D; ++i) g[i] = T(0);
#pragma unroll
        for (int i = 0; i < DD; ++i) Dg[i] = carry[i] = T(0);
        for (int32_t i = 0; i < nf; ++i) {
            const int32_t f    = ring_face[ro + i];
            const int32_t v[3] = {__ldg(fv + 3 * (int64_t)f), __ldg(fv + 3 * (int64_t)f + 1),
                                  __ldg(fv + 3 * (int64_t)f + 2)};
            const T*      r    = rec + (int64_t)W * f;
            const int     lp   = term_corner(v, (int32_t)p);
#pragma unroll
            for (int c = 0; c < D; ++c) g[c] += __ldg(r + 1 + D * lp + c);
            if (hval) {
                const int li = term_corner(v, ring[ro + i]);
                const int lj = term_corner(v, ring[ro + (i + 1 < k ? i + 1 : 0)]);
                term_block<T, D>(r, lp, lp, Dg);
                T bi[DD];
#pragma unroll
                for (int t = 0; t < DD; ++t) bi[t] = carry[t];
                term_block<T, D>(r, lp, li, bi);
                T* slot = hval + DD * (int64_t)(rp + 1 + i);
#pragma unroll
                for (int t = 0; t < DD; ++t) {
                    slot[t]  = ACC ? slot[t] + bi[t] : bi[t];
                    carry[t] = T(0);
                }
                term_block<T, D>(r, lp, lj, carry);
            }
        }
        (void)K;
        if (hval) {
            if (k > 0) {
                // the carry belongs to the last ring entry (open fan) or wraps
                // to the first one (closed fan, already written this call)
                T* slot = hval + DD * (int64_t)(rp + 1 + (bnd[p] ? k - 1 : 0));
#pragma unroll
                for (int t = 0; t < DD; ++t) slot[t] = (bnd[p] && !ACC) ? carry[t] : slot[t] + carry[t];
            }
            T* dslot = hval + DD * (int64_t)rp;
#pragma unroll
            for (int t = 0; t < DD; ++t) dslot[t] = ACC ? dslot[t] + Dg[t] : Dg[t];
        }
        if (grad) {
#pragma unroll
            for (int c = 0; c < D; ++c) grad[D * p + c] = ACC ? grad[D * p + c] + g[c] : g[c];
        }
    }
}

// checks shared by the entry points; fills the Hessian's pattern
static rxg_status term_setup(const rxg_mesh* h, int32_t dtype, int32_t dim, void* grad, void* face_E,
                             rxg_bcsr* hess, bool accumulate, cudaStream_t s, Lazy** z)
{
    if (hess && (!hess->row_ptr || !hess->col || !hess->val || hess->dtype != dtype ||
                 (hess->block_dim == 0 ? 3 : hess->block_dim) != dim)) {
        set_error("term: hess needs row_ptr, col, val of the term's dtype and %dx%d blocks", dim, dim);
        return RXG_ERR_INVALID;
    }
    if ((grad && !is_device_ptr(grad)) || (face_E && !is_device_ptr(face_E)) ||
        (hess && (!is_device_ptr(hess->val) || !is_device_ptr(hess->row_ptr) || !is_device_ptr(hess->col)))) {
        set_error("term: grad, the per-element energies and hess must be device arrays");
        return RXG_ERR_INVALID;
    }
    if (!h->m.edge_manifold) {
        set_error("term: the gather walks oriented vertex rings and needs a manifold mesh");
        return RXG_ERR_NONMANIFOLD;
    }
    rxg_status st = ensure_pattern(&h->m, s, z);
    if (st) return st;
    const int64_t nv = h->m.nv;
    if (hess) {
        hess->n    = nv;
        hess->nnzb = (*z)->nnz;
        if (!accumulate) {
            RXG_CUDA_TRY(cudaMemcpyAsync(hess->row_ptr, (*z)->row_ptr, 4 * (nv + 1), cudaMemcpyDeviceToDevice, s));
            RXG_CUDA_TRY(cudaMemcpyAsync(hess->col, (*z)->col, 4 * (*z)->nnz, cudaMemcpyDeviceToDevice, s));
        }
    }
    return RXG_OK;
}

// sum of the partials into *energy (host or device double)
static rxg_status term_energy_out(double* part, int np, double* energy, cudaStream_t s)
{
    k_sum_partials<<<1, 32, 0, s>>>(part, np, part + np);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && energy) {
        if (is_device_ptr(energy))
            e = cudaMemcpyAsync(energy, part + np, sizeof(double), cudaMemcpyDeviceToDevice, s);
        else {
            e = cudaMemcpyAsync(energy, part + np, sizeof(double), cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        }
    }
    return e == cudaSuccess ? RXG_OK : cuda_status(e, "face term energy");
}

template <typename T, int D>
static void launch_gather(bool acc, int G, int64_t nv, const Lazy* z, const int32_t* fv, const T* rec,
                          T* grad, T* hval, cudaStream_t s)
{
    if (acc)
        k_term_gather<T, D, true><<<G, 128, 0, s>>>(nv, z->row_ptr, z->ring_off, z->ring, z->ring_face,
                                                    z->bnd, fv, rec, grad, hval);
    else
        k_term_gather<T, D, false><<<G, 128, 0, s>>>(nv, z->row_ptr, z->ring_off, z->ring, z->ring_face,
                                                     z->bnd, fv, rec, grad, hval);
}

// Inertia term of a mass-spring system (the reference's add_inertia_term,
// tests/RXMesh_test/test_hess.cu:13-29, an Op::V term): per vertex
// E_v = m/2 |x_v - xt_v|^2, gradient m (x_v - xt_v), Hessian m I on the
// diagonal block.  ACC: add to the gradient (else overwrite it).  HACC: add
// m I to the diagonal blocks (the host has cleared the Hessian when the term
// overwrites it); else write the whole row (m I, zero off-diagonal blocks).
template <typename T, int D, bool ACC, bool HACC>
__global__ void __launch_bounds__(128) k_inertia(int64_t nv, const int32_t* __restrict__ row_ptr,
                                                 const T* __restrict__ x, const T* __restrict__ xt, T m,
                                                 T* __restrict__ grad, T* __restrict__ hval,
                                                 double* __restrict__ part)
{
    constexpr int DD = D * D;
    __shared__ double s_red[128 / 32];
    double            esum = 0;
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < nv;
         v += (int64_t)gridDim.x * blockDim.x) {
        T e = T(0);
#pragma unroll
        for (int c = 0; c < D; ++c) {
            const T d = x[D * v + c] - xt[D * v + c];
            e += d * d;
            if (grad) grad[D * v + c] = ACC ? grad[D * v + c] + m * d : m * d;
        }
        esum += 0.5 * (double)m * (double)e;
        if (hval) {
            const int32_t r0 = row_ptr[v], r1 = row_ptr[v + 1];
            T*            dg = hval + DD * (int64_t)r0;  // the row's first block is the diagonal
#pragma unroll
            for (int t = 0; t < DD; ++t) {
                const T mi = (t % (D + 1) == 0) ? m : T(0);
                dg[t]      = HACC ? dg[t] + mi : mi;
            }
            if (!HACC)
                for (int64_t t = DD * (int64_t)(r0 + 1); t < DD * (int64_t)r1; ++t) hval[t] = T(0);
        }
    }
    const double t = term_block_sum<128>(esum, s_red);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// calls f(T{}, integral_constant<D>) for the record type and 1, 2 or 3 components per vertex
template <typename F>
static void term_dispatch(int32_t dtype, int32_t dim, F&& f)
{
    using C1 = std::integral_constant<int, 1>;
    using C2 = std::integral_constant<int, 2>;
    using C3 = std::integral_constant<int, 3>;
    if (dtype == RXG_F64) {
        if (dim == 1) f(double{}, C1{});
        else if (dim == 2) f(double{}, C2{});
        else f(double{}, C3{});
    } else {
        if (dim == 1) f(float{}, C1{});
        else if (dim == 2) f(float{}, C2{});
        else f(float{}, C3{});
    }
}

// the ring's edges (Lazy::ring_edge), built once per mesh
static rxg_status ensure_ring_edge(const Mesh* m, Lazy* z, cudaStream_t s)
{
    std::lock_guard<std::mutex> g(z->mu);
    if (z->ring_edge) return RXG_OK;
    const int64_t nv = m->nv, ne = m->ne;
    int32_t *     ve_off = nullptr, *ve = nullptr, *ev = nullptr, *re = nullptr;
    RXG_CUDA_TRY(cudaMalloc(&re, 4 * std::max<int64_t>(1, 2 * ne)));
    RXG_CUDA_TRY(scratch_alloc((void**)&ve_off, 4 * (nv + 1), s));
    RXG_CUDA_TRY(scratch_alloc((void**)&ve, 4 * std::max<int64_t>(4, 2 * ne), s));
    RXG_CUDA_TRY(scratch_alloc((void**)&ev, 4 * std::max<int64_t>(4, 2 * ne), s));
    rxg_status st = launch_query(m, RXG_OP_VE, ve_off, ve, s);
    if (!st) st = launch_query(m, RXG_OP_EV, nullptr, ev, s);
    if (!st) {
        k_ring_edge<<<grid_for_items(nv), 256, 0, s>>>(nv, z->ring_off, z->ring, ve_off, ve, ev, re,
                                                       device_error_word());
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) st = cuda_status(e, "ring edges");
    }
    cudaFreeAsync(ve_off, s);
    cudaFreeAsync(ve, s);
    cudaFreeAsync(ev, s);
    if (!st) st = check_device_error(s);
    if (st) {
        cudaFree(re);
        return st;
    }
    z->ring_edge = re;
    return RXG_OK;
}

}  // namespace rxg

using namespace rxg;

extern "C" {

rxg_status rxg_edge_term_gather(const rxg_mesh* h, int32_t dtype, int32_t dim, const void* records,
                                int32_t flags, double* energy, void* edge_E, void* grad, rxg_bcsr* hess,
                                void* stream)
{
    if (!h || !records || (dtype != RXG_F32 && dtype != RXG_F64) || dim < 1 || dim > 3 ||
        (flags & ~RXG_TERM_ACCUMULATE)) {
        set_error("rxg_edge_term_gather: bad argument");
        return RXG_ERR_INVALID;
    }
    if (!is_device_ptr(records)) {
        set_error("rxg_edge_term_gather: records must be a device array");
        return RXG_ERR_INVALID;
    }
    cudaStream_t s   = (cudaStream_t)stream;
    const bool   acc = (flags & RXG_TERM_ACCUMULATE) != 0;
    Lazy*        z;
    rxg_status   st = term_setup(h, dtype, dim, grad, edge_E, hess, acc, s, &z);
    if (st) return st;
    if ((grad || hess) && (st = ensure_ring_edge(&h->m, z, s))) return st;
    const int64_t nv = h->m.nv, ne = h->m.ne;
    const int     G  = std::min<int>(grid_for_items(nv) * 2, 152 * 16);
    const int     GE = std::min<int>(grid_for_items(ne) * 2, 152 * 16);
    double*       part;
    RXG_CUDA_TRY(scratch_alloc((void**)&part, sizeof(double) * (GE + 1), s));
    auto run = [&](auto tag, auto dtag) {
        using T         = decltype(tag);
        constexpr int D = decltype(dtag)::value;
        constexpr int W = term_record_words_n(2, D);
        k_term_energy_w<T, W><<<GE, 128, 0, s>>>(ne, (const T*)records, (T*)edge_E, part);
        if (grad || hess) {
            T* hv = hess ? (T*)hess->val : nullptr;
            if (acc)
                k_edge_term_gather<T, D, true><<<G, 128, 0, s>>>(nv, z->row_ptr, z->ring_off, z->ring_edge,
                                                                 (const T*)records, (T*)grad, hv);
            else
                k_edge_term_gather<T, D, false><<<G, 128, 0, s>>>(nv, z->row_ptr, z->ring_off, z->ring_edge,
                                                                  (const T*)records, (T*)grad, hv);
        }
    };
    term_dispatch(dtype, dim, run);
    st = term_energy_out(part, GE, energy, s);
    cudaFreeAsync(part, s);
    return st;
}

rxg_status rxg_vertex_term_gather(const rxg_mesh* h, int32_t dtype, int32_t dim, const void* records,
                                  int32_t flags, double* energy, void* vertex_E, void* grad, rxg_bcsr* hess,
                                  void* stream)
{
    if (!h || !records || (dtype != RXG_F32 && dtype != RXG_F64) || dim < 1 || dim > 3 ||
        (flags & ~RXG_TERM_ACCUMULATE)) {
        set_error("rxg_vertex_term_gather: bad argument");
        return RXG_ERR_INVALID;
    }
    if (!is_device_ptr(records)) {
        set_error("rxg_vertex_term_gather: records must be a device array");
        return RXG_ERR_INVALID;
    }
    cudaStream_t s   = (cudaStream_t)stream;
    const bool   acc = (flags & RXG_TERM_ACCUMULATE) != 0;
    Lazy*        z;
    rxg_status   st = term_setup(h, dtype, dim, grad, vertex_E, hess, acc, s, &z);
    if (st) return st;
    const int64_t nv = h->m.nv;
    const int     G  = std::min<int>(grid_for_items(nv) * 2, 152 * 16);
    double*       part;
    // overwriting: the whole Hessian cleared, then the diagonal blocks added
    if (hess && !acc)
        RXG_CUDA_TRY(cudaMemsetAsync(hess->val, 0, (size_t)dim * dim * z->nnz * (dtype == RXG_F64 ? 8 : 4), s));
    RXG_CUDA_TRY(scratch_alloc((void**)&part, sizeof(double) * (G + 1), s));
    auto run = [&](auto tag, auto dtag) {
        using T         = decltype(tag);
        constexpr int D = decltype(dtag)::value;
        constexpr int W = term_record_words_n(1, D);
        k_term_energy_w<T, W><<<G, 128, 0, s>>>(nv, (const T*)records, (T*)vertex_E, part);
        if (grad || hess) {
            T* hv = hess ? (T*)hess->val : nullptr;
            if (acc)
                k_vertex_term_gather<T, D, true><<<G, 128, 0, s>>>(nv, z->row_ptr, (const T*)records, (T*)grad, hv);
            else
                k_vertex_term_gather<T, D, false><<<G, 128, 0, s>>>(nv, z->row_ptr, (const T*)records, (T*)grad,
                                                                    hv);
        }
    };
    term_dispatch(dtype, dim, run);
    st = term_energy_out(part, G, energy, s);
    cudaFreeAsync(part, s);
    return st;
}

rxg_status rxg_inertia_eval(const rxg_mesh* h, int32_t dtype, int32_t dim, const void* x,
                            const void* x_target, double mass, int32_t flags, double* energy,
                            void* grad, rxg_bcsr* hess, void* stream)
{
    if (!h || !x || !x_target || (dtype != RXG_F32 && dtype != RXG_F64) || dim < 1 || dim > 3 ||
        (flags & ~RXG_TERM_ACCUMULATE)) {
        set_error("rxg_inertia_eval: bad argument");
        return RXG_ERR_INVALID;
    }
    if (!is_device_ptr(x) || !is_device_ptr(x_target)) {
        set_error("rxg_inertia_eval: x and x_target must be device arrays");
        return RXG_ERR_INVALID;
    }
    cudaStream_t s   = (cudaStream_t)stream;
    const bool   acc = (flags & RXG_TERM_ACCUMULATE) != 0;
    if (hess && (!hess->row_ptr || !hess->col || !hess->val || hess->dtype != dtype ||
                 (hess->block_dim == 0 ? 3 : hess->block_dim) != dim)) {
        set_error("rxg_inertia_eval: hess needs row_ptr, col, val of the term's dtype and %dx%d blocks", dim,
                  dim);
        return RXG_ERR_INVALID;
    }
    if ((grad && !is_device_ptr(grad)) || (hess && !is_device_ptr(hess->val))) {
        set_error("rxg_inertia_eval: grad and hess must be device arrays");
        return RXG_ERR_INVALID;
    }
    Lazy*      z;
    rxg_status st = ensure_pattern(&h->m, s, &z);
    if (st) return st;
    const int64_t nv = h->m.nv;
    if (hess) {
        hess->n    = nv;
        hess->nnzb = z->nnz;
        if (!acc) {
            RXG_CUDA_TRY(cudaMemcpyAsync(hess->row_ptr, z->row_ptr, 4 * (nv + 1), cudaMemcpyDeviceToDevice, s));
            RXG_CUDA_TRY(cudaMemcpyAsync(hess->col, z->col, 4 * z->nnz, cudaMemcpyDeviceToDevice, s));
        }
    }
    const int G = std::min<int>(grid_for_items(nv) * 2, 152 * 16);
    double*   part;
    // overwriting: one coalesced clear of the whole Hessian, then the kernel
    // adds m I to the diagonal blocks as when accumulating
    if (hess && !acc)
        RXG_CUDA_TRY(cudaMemsetAsync(hess->val, 0,
                                     (size_t)dim * dim * z->nnz * (dtype == RXG_F64 ? 8 : 4), s));
    RXG_CUDA_TRY(scratch_alloc((void**)&part, sizeof(double) * (G + 1), s));
    auto run = [&](auto tag, auto dtag) {
        using T         = decltype(tag);
        constexpr int D = decltype(dtag)::value;
        T* hv           = hess ? (T*)hess->val : nullptr;
        if (acc)
            k_inertia<T, D, true, true><<<G, 128, 0, s>>>(nv, z->row_ptr, (const T*)x, (const T*)x_target,
                                                          (T)mass, (T*)grad, hv, part);
        else
            k_inertia<T, D, false, true><<<G, 128, 0, s>>>(nv, z->row_ptr, (const T*)x, (const T*)x_target,
                                                           (T)mass, (T*)grad, hv, part);
    };
    term_dispatch(dtype, dim, run);
    st = term_energy_out(part, G, energy, s);
    cudaFreeAsync(part, s);
    return st;
}

rxg_status rxg_face_term_gather(const rxg_mesh* h, int32_t dtype, int32_t dim, const void* records,
                                int32_t flags, double* energy, void* face_E, void* grad,
                                rxg_bcsr* hess, void* stream)
{
    if (!h || !records || (dtype != RXG_F32 && dtype != RXG_F64) || dim < 1 || dim > 3 ||
        (flags & ~RXG_TERM_ACCUMULATE)) {
        set_error("rxg_face_term_gather: bad argument");
        return RXG_ERR_INVALID;
    }
    if (!is_device_ptr(records)) {
        set_error("rxg_face_term_gather: records must be a device array");
        return RXG_ERR_INVALID;
    }
    cudaStream_t s   = (cudaStream_t)stream;
    const bool   acc = (flags & RXG_TERM_ACCUMULATE) != 0;
    Lazy*        z;
    rxg_status   st = term_setup(h, dtype, dim, grad, face_E, hess, acc, s, &z);
    if (st) return st;
    const int64_t nv = h->m.nv, nf = h->m.nf;
    const int     G  = std::min<int>(grid_for_items(nv) * 2, 152 * 16);
    const int     GF = std::min<int>(grid_for_items(nf) * 2, 152 * 16);
    double*       part;
    RXG_CUDA_TRY(scratch_alloc((void**)&part, sizeof(double) * (GF + 1), s));
    const int32_t* fv = h->m.d.fv_lin;
    term_dispatch(dtype, dim, [&](auto tag, auto dtag) {
        using T         = decltype(tag);
        constexpr int D = decltype(dtag)::value;
        k_term_energy<T, D><<<GF, 128, 0, s>>>(nf, (const T*)records, (T*)face_E, part);
        launch_gather<T, D>(acc, G, nv, z, fv, (const T*)records, (T*)grad, hess ? (T*)hess->val : nullptr, s);
    });
    st = term_energy_out(part, GF, energy, s);
    cudaFreeAsync(part, s);
    return st;
}

rxg_status rxg_symdir_eval(const rxg_mesh* h, int32_t dtype, const void* uv, const void* rest,
                           int32_t flags, double* energy, void* face_E, void* grad, rxg_bcsr* hess,
                           void* stream)
{
    if (!h || !uv || !rest || (dtype != RXG_F32 && dtype != RXG_F64) ||
        (flags & ~(RXG_TERM_ACCUMULATE | RXG_TERM_PROJECT_HESSIAN))) {
        set_error("rxg_symdir_eval: bad argument");
        return RXG_ERR_INVALID;
    }
    if (!is_device_ptr(uv) || !is_device_ptr(rest)) {
        set_error("rxg_symdir_eval: uv and rest must be device arrays");
        return RXG_ERR_INVALID;
    }
    cudaStream_t s    = (cudaStream_t)stream;
    const bool   acc  = (flags & RXG_TERM_ACCUMULATE) != 0;
    const bool   proj = (flags & RXG_TERM_PROJECT_HESSIAN) != 0;
    Lazy*        z;
    rxg_status   st = term_setup(h, dtype, 2, grad, face_E, hess, acc, s, &z);
    if (st) return st;
    const int64_t nv = h->m.nv, nf = h->m.nf;
    const int     G  = std::min<int>(grid_for_items(nv) * 2, 152 * 16);
    const int     GF = std::min<int>(grid_for_items(nf) * 2, 152 * 16);
    const size_t  ts = dtype == RXG_F64 ? 8 : 4;
    double*       part;
    void*         rec = nullptr;
    RXG_CUDA_TRY(scratch_alloc((void**)&part, sizeof(double) * (GF + 1), s));
    cudaError_t ea = scratch_alloc(&rec, (size_t)nf * term_record_words(2) * ts + 16, s);
    if (ea != cudaSuccess) {
        cudaFreeAsync(part, s);
        return cuda_status(ea, "rxg_symdir_eval: face records");
    }
    const int32_t* fv = h->m.d.fv_lin;
    auto run = [&](auto tag) {
        using T = decltype(tag);
        SymDirEnergy<T> en{(const T*)rest};
        if (proj)
            k_term_face<T, 2, true><<<GF, 128, 0, s>>>(nf, fv, (const T*)uv, en, (T*)rec, (T*)face_E, part);
        else
            k_term_face<T, 2, false><<<GF, 128, 0, s>>>(nf, fv, (const T*)uv, en, (T*)rec, (T*)face_E, part);
        if (grad || hess)
            launch_gather<T, 2>(acc, G, nv, z, fv, (const T*)rec, (T*)grad, hess ? (T*)hess->val : nullptr, s);
    };
    if (dtype == RXG_F64) run(double{});
    else run(float{});
    st = term_energy_out(part, GF, energy, s);
    cudaFreeAsync(rec, s);
    cudaFreeAsync(part, s);
    return st;
}

}  // extern "C"
