// Batched implicit MCF: many meshes of uneven size in one persistent launch.
//
// The meshes are packed into one union mesh whose patches never span two
// components (RXG_MESH_SPLIT_COMPONENTS), so every mesh owns one contiguous
// range of linear vertex ids (the reference packs several meshes into one
// RXMeshStatic the same way, rxmesh_static.cu:66-160).  One CTA takes one
// mesh from a work queue (largest first) and runs that mesh's whole
// mixed-precision flow on its own: FP32 cotangent assembly (FP64 for
// near-degenerate triangles), FP64 residual, FP32 Jacobi-PCG refinement
// sweeps, all steps -- synchronising only with __syncthreads, so there are no
// grid barriers and no host round trips, and the call can be captured in a
// CUDA graph.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <mutex>
#include <numeric>
#include <vector>

#include "rxg_gridsum.cuh"
#include "rxg_lazy.h"
#include "rxg_mcf_common.cuh"

struct rxg_batch
{
    rxg_mesh*            mesh  = nullptr;  // union of all meshes
    int32_t              nmesh = 0;
    std::vector<int64_t> voff, foff;       // input offsets per mesh (nmesh+1)
    std::vector<int32_t> vstart, vcount;   // linear vertex range per mesh
    int32_t*             d_order  = nullptr;
    int32_t*             d_vstart = nullptr;
    int32_t*             d_vcount = nullptr;
    int32_t*             d_queue  = nullptr;
    int32_t*             d_iters  = nullptr;
    int32_t*             d_conv   = nullptr;
    void*                buf      = nullptr;
    size_t               buf_size = 0;
    int32_t              threads  = 512;
    int32_t              blocks_per_sm = 2;
    std::mutex           mu;
};

namespace rxg {

struct BatchArgs
{
    int32_t           nmesh;
    const int32_t*    order;
    const int32_t*    vstart;
    const int32_t*    vcount;
    int32_t*          queue;
    const int32_t*    row_ptr;
    const int32_t*    col;
    const int8_t*     bnd;
    Ent<float>*       ent;
    R4<double>*       X;
    R4<double>*       B;
    R4<float>*        R;
    R4<float>*        P;
    R4<float>*        S;
    R4<float>*        Z;
    R4<float>*        D;
    float*            dinv;
    double*           diag;  // FP64 diagonal (2*area + sum of the FP32 weights)
    float             dt;
    int32_t           nsteps;
    double            tol;
    int32_t           max_iter;
    int32_t*          iters;
    int32_t*          conv;
};

__device__ __forceinline__ V3<double> pos4(const R4<double>* X, int32_t i)
{
    const R4<double> v = X[i];
    return {v.x, v.y, v.z};
}

// one row of the MCF system (mcf_A_setup / mcf_B_setup), FP32 weights with
// FP64 for near-degenerate triangles, positions from the packed FP64 state
__device__ __forceinline__ void assemble_row(int64_t p, const BatchArgs& a)
{
    const int32_t    rp   = a.row_ptr[p];
    const int32_t    k    = a.row_ptr[p + 1] - rp - 1;
    const int32_t*   rg   = a.col + rp + 1;
    const bool       wrap = a.bnd[p] == 0;
    const V3<double> P    = pos4(a.X, (int32_t)p);
    double           area = 0.0, sumw = 0.0;  // FP64 row sums (see k_mcf_assemble)
    if (k > 0) {
        V3<double> Q = pos4(a.X, rg[k - 1]), R = pos4(a.X, rg[0]);
        for (int32_t i = 0; i < k; ++i) {
            const V3<double> S     = pos4(a.X, rg[i + 1 < k ? i + 1 : 0]);
            const bool       has_q = wrap || i > 0, has_s = wrap || i < k - 1;
            float            w     = 0.f;
            if (has_q) w += GeoMixed::hc(P, R, Q);
            if (has_s) w += GeoMixed::hc(P, R, S);
            w = (w >= 0.f ? w : 0.f) * a.dt;
            sumw += (double)w;
            Ent<float> e;
            e.col              = rg[i];
            e.val              = -w;
            a.ent[rp + 1 + i]  = e;
            if (has_q) {
                const float ar = GeoMixed::va(P, Q, R);
                area += ar > 0.f ? (double)ar : 0.0;
            }
            Q = R;
            R = S;
        }
    }
    const double vw = 0.5 / area;
    const double dg = 1.0 / vw + sumw;
    Ent<float>   d;
    d.col        = (int32_t)p;
    d.val        = (float)dg;
    a.ent[rp]    = d;
    a.diag[p]    = dg;
    a.dinv[p]    = 1.f / (d.val + FLT_EPSILON);
    R4<double> b;
    b.x     = P.x / vw;
    b.y     = P.y / vw;
    b.z     = P.z / vw;
    b.w     = 0.0;
    a.B[p]  = b;
}

// R = (float)(B - A X) accumulated in FP64; returns the block's r . D^-1 r
template <int BT>
__device__ __forceinline__ double residual(int64_t v0, int64_t v1, const BatchArgs& a, double* s_red)
{
    double part = 0;
    for (int64_t i = v0 + threadIdx.x; i < v1; i += BT) {
        const R4<double> xi = a.X[i];
        const double     dg = a.diag[i];
        double           a0 = dg * xi.x, a1 = dg * xi.y, a2 = dg * xi.z;
        const int32_t    e  = a.row_ptr[i + 1];
        for (int32_t j = a.row_ptr[i] + 1; j < e; ++j) {
            const Ent<float> q  = a.ent[j];
            const R4<double> xv = a.X[q.col];
            a0 += (double)q.val * xv.x;
            a1 += (double)q.val * xv.y;
            a2 += (double)q.val * xv.z;
        }
        const R4<double> b  = a.B[i];
        const double     e0 = b.x - a0, e1 = b.y - a1, e2 = b.z - a2;
        R4<float>        r;
        r.x = (float)e0, r.y = (float)e1, r.z = (float)e2, r.w = 0.f;
        a.R[i] = r;
        part += (e0 * e0 + e1 * e1 + e2 * e2) / dg;
    }
    return block_sum<BT>(part, s_red);
}

// scalar state of a CTA's inner PCG: the FP64 recurrence is touched by
// thread 0 only; every thread reads the FP32 step sizes and the flag
struct BatchPCG
{
    double delta0, delta;
    int    it;
    float  al, bt;
    int    done;
};

// block-level Jacobi-PCG for A D = R (R is overwritten as the residual);
// returns the iterations completed.  Dot products: FP32 per thread and
// warp, FP64 per CTA (rxg_gridsum.cuh).
template <int BT>
__device__ int inner_pcg(int64_t v0, int64_t v1, const BatchArgs& a, double rel2, int max_it,
                         RedSmem& red, BatchPCG& c)
{
    float tp = 0.f;
    for (int64_t i = v0 + threadIdx.x; i < v1; i += BT) {
        const float     di = a.dinv[i];
        const R4<float> r  = a.R[i];
        R4<float>       z;
        z.x = di * r.x, z.y = di * r.y, z.z = di * r.z, z.w = 0.f;
        a.Z[i] = z;
        a.P[i] = z;
        R4<float> zero;
        zero.x = zero.y = zero.z = zero.w = 0.f;
        a.D[i] = zero;
        tp += r.x * z.x + r.y * z.y + r.z * z.z;
    }
    block_sum_post<BT>(tp, red, [&](double t) {
        c.delta0 = c.delta = t;
        c.it               = 0;
        c.done             = !(t > 0) || max_it <= 0;
    });
    while (!c.done) {
        // S = A P, P.S   (the block barriers order P before the gathers)
        tp = 0.f;
        for (int64_t i = v0 + threadIdx.x; i < v1; i += BT) {
            float ax = 0, ay = 0, az = 0;
            row_spmv4<float>(a.row_ptr, a.ent, i, a.P, ax, ay, az, (float*)nullptr);
            R4<float> s;
            s.x = ax, s.y = ay, s.z = az, s.w = 0.f;
            a.S[i]            = s;
            const R4<float> p = a.P[i];
            tp += s.x * p.x + s.y * p.y + s.z * p.z;
        }
        block_sum_post<BT>(tp, red, [&](double sp) { c.al = (float)(c.delta / sp); });
        const float al = c.al;
        tp             = 0.f;
        for (int64_t i = v0 + threadIdx.x; i < v1; i += BT) {
            const float     di = a.dinv[i];
            const R4<float> p = a.P[i], s = a.S[i];
            R4<float>       d = a.D[i], r = a.R[i], z;
            d.x += al * p.x, d.y += al * p.y, d.z += al * p.z;
            r.x -= al * s.x, r.y -= al * s.y, r.z -= al * s.z;
            z.x = di * r.x, z.y = di * r.y, z.z = di * r.z, z.w = 0.f;
            a.D[i] = d;
            a.R[i] = r;
            a.Z[i] = z;
            tp += r.x * z.x + r.y * z.y + r.z * z.z;
        }
        block_sum_post<BT>(tp, red, [&](double dn) {
            if (dn < rel2 * c.delta0) {
                c.done = 1;
                return;
            }
            c.bt    = (float)(dn / c.delta);
            c.delta = dn;
            ++c.it;
            c.done = c.it >= max_it;
        });
        if (c.done) break;
        const float bt = c.bt;
        for (int64_t i = v0 + threadIdx.x; i < v1; i += BT) {
            const R4<float> z = a.Z[i];
            R4<float>       p = a.P[i];
            p.x = z.x + bt * p.x, p.y = z.y + bt * p.y, p.z = z.z + bt * p.z;
            a.P[i] = p;
        }
        __syncthreads();
    }
    return c.it;
}

template <int BT>
__global__ void __launch_bounds__(BT) k_mcf_batch(BatchArgs a)
{
    __shared__ int      s_job;
    __shared__ double   s_red[BT / 32 + 2];
    __shared__ RedSmem  red;
    __shared__ BatchPCG pcg;
    while (true) {
        if (threadIdx.x == 0) s_job = atomicAdd(a.queue, 1);
        __syncthreads();
        const int job = s_job;
        __syncthreads();
        if (job >= a.nmesh) return;
        const int     m  = a.order[job];
        const int64_t v0 = a.vstart[m], v1 = v0 + a.vcount[m];
        int           total_it = 0;
        bool          conv_all = true;
        for (int step = 0; step < a.nsteps; ++step) {
            for (int64_t p = v0 + threadIdx.x; p < v1; p += BT) assemble_row(p, a);
            __syncthreads();
            const double rr0  = residual<BT>(v0, v1, a, s_red);
            double       rr   = rr0;
            bool         conv = !(rr0 > 0);
            for (int sweep = 0; sweep < 16 && !conv && total_it < a.max_iter; ++sweep) {
                const double need  = a.tol * sqrt(rr0 / rr);
                const double inner = fmax(1e-4, 0.3 * need);
                total_it += inner_pcg<BT>(v0, v1, a, inner * inner, a.max_iter - total_it, red, pcg) + 1;
                for (int64_t i = v0 + threadIdx.x; i < v1; i += BT) {
                    R4<double>      x = a.X[i];
                    const R4<float> d = a.D[i];
                    x.x += (double)d.x, x.y += (double)d.y, x.z += (double)d.z;
                    a.X[i] = x;
                }
                __syncthreads();
                rr   = residual<BT>(v0, v1, a, s_red);
                conv = rr < a.tol * a.tol * rr0;
            }
            conv_all = conv_all && conv;
        }
        if (threadIdx.x == 0) {
            a.iters[m] = total_it;
            a.conv[m]  = conv_all ? 1 : 0;
        }
    }
}

__global__ void k_batch_pack(int64_t n, const int32_t* __restrict__ l2i, const double* __restrict__ x,
                             R4<double>* __restrict__ X)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = 3 * (int64_t)l2i[i];
        R4<double>    v;
        v.x = x[s], v.y = x[s + 1], v.z = x[s + 2], v.w = 0.0;
        X[i] = v;
    }
}

__global__ void k_batch_unpack(int64_t n, const int32_t* __restrict__ l2i,
                               const R4<double>* __restrict__ X, double* __restrict__ x)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t    s = 3 * (int64_t)l2i[i];
        const R4<double> v = X[i];
        x[s] = v.x, x[s + 1] = v.y, x[s + 2] = v.z;
    }
}

}  // namespace rxg

using namespace rxg;

static int batch_sms()
{
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return std::max(1, sms);
}

template <int BT>
static int batch_max_per_sm()
{
    int per = 1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_mcf_batch<BT>, BT, 0) != cudaSuccess)
        per = 1;
    return std::max(1, per);
}

static int max_per_sm(int bt)
{
    switch (bt) {
        case 256: return batch_max_per_sm<256>();
        case 1024: return batch_max_per_sm<1024>();
        default: return batch_max_per_sm<512>();
    }
}

static rxg_status batch_buffers(rxg_batch* b, size_t bytes)
{
    if (b->buf_size >= bytes) return RXG_OK;
    cudaFree(b->buf);
    b->buf      = nullptr;
    b->buf_size = 0;
    RXG_CUDA_TRY(cudaMalloc(&b->buf, bytes));
    b->buf_size = bytes;
    return RXG_OK;
}

static size_t a256(size_t x) { return (x + 255) & ~size_t(255); }

// lays the union's work arrays out in b->buf (allocating once)
static rxg_status batch_args(rxg_batch* b, cudaStream_t s, BatchArgs* out, R4<double>** X4)
{
    Lazy*      z;
    rxg_status st = ensure_pattern(&b->mesh->m, s, &z);
    if (st) return st;
    const int64_t n = b->mesh->m.nv, nnz = z->nnz;
    const size_t  bytes = a256(sizeof(Ent<float>) * nnz) + 2 * a256(sizeof(R4<double>) * n) +
                         5 * a256(sizeof(R4<float>) * n) + a256(sizeof(float) * n) +
                         a256(sizeof(double) * n);
    {
        std::lock_guard<std::mutex> g(b->mu);
        if ((st = batch_buffers(b, bytes))) return st;
    }
    uint8_t* q = (uint8_t*)b->buf;
    BatchArgs a;
    a.nmesh   = b->nmesh;
    a.order   = b->d_order;
    a.vstart  = b->d_vstart;
    a.vcount  = b->d_vcount;
    a.queue   = b->d_queue;
    a.row_ptr = z->row_ptr;
    a.col     = z->col;
    a.bnd     = z->bnd;
    a.ent = (Ent<float>*)q, q += a256(sizeof(Ent<float>) * nnz);
    a.X = (R4<double>*)q, q += a256(sizeof(R4<double>) * n);
    a.B = (R4<double>*)q, q += a256(sizeof(R4<double>) * n);
    a.R = (R4<float>*)q, q += a256(sizeof(R4<float>) * n);
    a.P = (R4<float>*)q, q += a256(sizeof(R4<float>) * n);
    a.S = (R4<float>*)q, q += a256(sizeof(R4<float>) * n);
    a.Z = (R4<float>*)q, q += a256(sizeof(R4<float>) * n);
    a.D = (R4<float>*)q, q += a256(sizeof(R4<float>) * n);
    a.dinv  = (float*)q, q += a256(sizeof(float) * n);
    a.diag  = (double*)q;
    a.iters = b->d_iters;
    a.conv  = b->d_conv;
    *out    = a;
    *X4     = a.X;
    return RXG_OK;
}

static rxg_status batch_launch(rxg_batch* b, BatchArgs a, int bt, int bps, cudaStream_t s)
{
    RXG_CUDA_TRY(cudaMemsetAsync(b->d_queue, 0, sizeof(int32_t), s));
    const int grid = std::min(b->nmesh, batch_sms() * std::min(bps, max_per_sm(bt)));
    switch (bt) {
        case 256: k_mcf_batch<256><<<grid, 256, 0, s>>>(a); break;
        case 1024: k_mcf_batch<1024><<<grid, 1024, 0, s>>>(a); break;
        default: k_mcf_batch<512><<<grid, 512, 0, s>>>(a); break;
    }
    RXG_CUDA_TRY(cudaGetLastError());
    return RXG_OK;
}

extern "C" {

rxg_status rxg_batch_create(int32_t nmesh, const int32_t* fv, const int64_t* nf, const int64_t* nv,
                            int32_t patch_faces, rxg_batch** out)
{
    if (!out || nmesh <= 0 || !fv || !nf || !nv) {
        set_error("rxg_batch_create: bad argument");
        return RXG_ERR_INVALID;
    }
    *out         = nullptr;
    rxg_batch* b = new (std::nothrow) rxg_batch();
    if (!b) {
        set_error("rxg_batch_create: host allocation failed");
        return RXG_ERR_NOMEM;
    }
    b->nmesh = nmesh;
    b->voff.assign(nmesh + 1, 0);
    b->foff.assign(nmesh + 1, 0);
    for (int m = 0; m < nmesh; ++m) {
        if (nf[m] <= 0 || nv[m] <= 0) {
            delete b;
            set_error("rxg_batch_create: mesh %d is empty", m);
            return RXG_ERR_INVALID;
        }
        b->voff[m + 1] = b->voff[m] + nv[m];
        b->foff[m + 1] = b->foff[m] + nf[m];
    }
    const int64_t        F = b->foff[nmesh], V = b->voff[nmesh];
    std::vector<int32_t> all(3 * F);
    for (int m = 0; m < nmesh; ++m)
        for (int64_t i = 3 * b->foff[m]; i < 3 * b->foff[m + 1]; ++i) {
            if (fv[i] < 0 || fv[i] >= nv[m]) {
                delete b;
                set_error("rxg_batch_create: mesh %d references vertex %d outside [0, %lld)", m,
                          fv[i], (long long)nv[m]);
                return RXG_ERR_INVALID;
            }
            all[i] = fv[i] + (int32_t)b->voff[m];
        }
    rxg_status st = rxg_mesh_create_ex(all.data(), F, V, patch_faces, RXG_MESH_SPLIT_COMPONENTS, &b->mesh);
    if (st) {
        delete b;
        return st;
    }
    // linear vertex range of every mesh (contiguous by construction)
    const std::vector<int32_t>& i2l = b->mesh->m.v_i2l;
    b->vstart.resize(nmesh);
    b->vcount.resize(nmesh);
    for (int m = 0; m < nmesh; ++m) {
        int32_t lo = INT32_MAX, hi = -1;
        for (int64_t v = b->voff[m]; v < b->voff[m + 1]; ++v) {
            lo = std::min(lo, i2l[v]);
            hi = std::max(hi, i2l[v]);
        }
        if (hi - lo + 1 != nv[m]) {
            rxg_mesh_destroy(b->mesh);
            delete b;
            set_error("rxg_batch_create: mesh %d has vertices in no face", m);
            return RXG_ERR_INVALID;
        }
        b->vstart[m] = lo;
        b->vcount[m] = (int32_t)nv[m];
    }
    // largest meshes first (longest-processing-time order for the work queue)
    std::vector<int32_t> order(nmesh);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(),
                     [&](int32_t x, int32_t y) { return b->vcount[x] > b->vcount[y]; });
    auto up = [&](int32_t** d, const void* h, size_t n) -> cudaError_t {
        cudaError_t e = cudaMalloc(d, std::max<size_t>(n, 1) * 4);
        if (e == cudaSuccess && h) e = cudaMemcpy(*d, h, n * 4, cudaMemcpyHostToDevice);
        return e;
    };
    cudaError_t e = up(&b->d_order, order.data(), nmesh);
    if (e == cudaSuccess) e = up(&b->d_vstart, b->vstart.data(), nmesh);
    if (e == cudaSuccess) e = up(&b->d_vcount, b->vcount.data(), nmesh);
    if (e == cudaSuccess) e = up(&b->d_queue, nullptr, 1);
    if (e == cudaSuccess) e = up(&b->d_iters, nullptr, nmesh);
    if (e == cudaSuccess) e = up(&b->d_conv, nullptr, nmesh);
    if (e != cudaSuccess) {
        rxg_batch_destroy(b);
        return cuda_status(e, "rxg_batch_create");
    }
    *out = b;
    return RXG_OK;
}

void rxg_batch_destroy(rxg_batch* b)
{
    if (!b) return;
    cudaFree(b->d_order);
    cudaFree(b->d_vstart);
    cudaFree(b->d_vcount);
    cudaFree(b->d_queue);
    cudaFree(b->d_iters);
    cudaFree(b->d_conv);
    cudaFree(b->buf);
    rxg_mesh_destroy(b->mesh);
    delete b;
}

rxg_status rxg_batch_mesh(const rxg_batch* b, const rxg_mesh** mesh)
{
    if (!b || !mesh) {
        set_error("rxg_batch_mesh: NULL argument");
        return RXG_ERR_INVALID;
    }
    *mesh = b->mesh;
    return RXG_OK;
}

rxg_status rxg_batch_mcf(rxg_batch* b, double dt, int32_t nsteps, double tol, int32_t max_iter,
                         double* xyz, void* stream)
{
    if (!b || !xyz || nsteps < 0 || !(tol > 0) || max_iter <= 0) {
        set_error("rxg_batch_mcf: bad argument");
        return RXG_ERR_INVALID;
    }
    if (!is_device_ptr(xyz)) {
        set_error("rxg_batch_mcf: xyz must be a device array");
        return RXG_ERR_INVALID;
    }
    cudaStream_t s = (cudaStream_t)stream;
    BatchArgs    a;
    R4<double>*  X4;
    rxg_status   st = batch_args(b, s, &a, &X4);
    if (st) return st;
    a.dt       = (float)dt;
    a.nsteps   = nsteps;
    a.tol      = tol;
    a.max_iter = max_iter;
    const int64_t n = b->mesh->m.nv;
    const int     g = (int)std::min<int64_t>((n + 255) / 256, 152 * 32);
    k_batch_pack<<<g, 256, 0, s>>>(n, b->mesh->m.d.v_l2i, xyz, X4);
    if ((st = batch_launch(b, a, b->threads, b->blocks_per_sm, s))) return st;
    k_batch_unpack<<<g, 256, 0, s>>>(n, b->mesh->m.d.v_l2i, X4, xyz);
    RXG_CUDA_TRY(cudaGetLastError());
    return RXG_OK;
}

rxg_status rxg_batch_stats(const rxg_batch* b, int32_t* iters, int32_t* converged)
{
    if (!b) {
        set_error("rxg_batch_stats: NULL batch");
        return RXG_ERR_INVALID;
    }
    if (iters) RXG_CUDA_TRY(cudaMemcpy(iters, b->d_iters, 4 * b->nmesh, cudaMemcpyDeviceToHost));
    if (converged) RXG_CUDA_TRY(cudaMemcpy(converged, b->d_conv, 4 * b->nmesh, cudaMemcpyDeviceToHost));
    return RXG_OK;
}

rxg_status rxg_batch_autotune(rxg_batch* b, double dt, int32_t nsteps, double tol, int32_t max_iter,
                              const double* xyz, int32_t* threads, int32_t* blocks_per_sm,
                              float* best_ms, void* stream)
{
    if (!b || !xyz || !is_device_ptr(xyz)) {
        set_error("rxg_batch_autotune: xyz must be a device array");
        return RXG_ERR_INVALID;
    }
    cudaStream_t s = (cudaStream_t)stream;
    BatchArgs    a;
    R4<double>*  X4;
    rxg_status   st = batch_args(b, s, &a, &X4);
    if (st) return st;
    a.dt       = (float)dt;
    a.nsteps   = nsteps;
    a.tol      = tol;
    a.max_iter = max_iter;
    const int64_t n = b->mesh->m.nv;
    const int     g = (int)std::min<int64_t>((n + 255) / 256, 152 * 32);
    cudaEvent_t   e0, e1;
    RXG_CUDA_TRY(cudaEventCreate(&e0));
    RXG_CUDA_TRY(cudaEventCreate(&e1));
    float best = 1e30f;
    int   bt_best = b->threads, bps_best = b->blocks_per_sm;
    for (int bt : {256, 512, 1024}) {
        for (int bps : {1, 2, 4, 8}) {
            if (bps > max_per_sm(bt)) continue;
            float t = 0;
            for (int rep = 0; rep < 2 && st == RXG_OK; ++rep) {
                k_batch_pack<<<g, 256, 0, s>>>(n, b->mesh->m.d.v_l2i, xyz, X4);
                cudaEventRecord(e0, s);
                st = batch_launch(b, a, bt, bps, s);
                cudaEventRecord(e1, s);
                cudaEventSynchronize(e1);
                cudaEventElapsedTime(&t, e0, e1);  // second repetition is kept
            }
            if (st) break;
            if (t < best) {
                best     = t;
                bt_best  = bt;
                bps_best = bps;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st) return st;
    b->threads       = bt_best;
    b->blocks_per_sm = bps_best;
    if (threads) *threads = bt_best;
    if (blocks_per_sm) *blocks_per_sm = bps_best;
    if (best_ms) *best_ms = best;
    return check_device_error(s);
}

}  // extern "C"
