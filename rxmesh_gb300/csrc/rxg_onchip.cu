// Mixed-precision implicit MCF solve with the solver state on chip.
//
// One cooperative launch per flow step runs the whole iterative refinement
// of the mixed path: FP64 residual r = B - A x (FP32 off-diagonals promoted,
// FP64 diagonal), FP32 Jacobi-PCG sweeps for A d = r, x += d, repeated until
// r . D^-1 r < tol^2 r0 . D^-1 r0 (the stop rule of the plain PCG,
// pcg_solver.h:14-213, on the FP64 residual).  One CTA per SM owns a
// contiguous chunk of rows and keeps that chunk's PCG vectors (p, s, r, d and
// D^-1) in shared memory for the whole launch: 52 bytes a row, so a GB300's
// 152 x 227 KB hold up to ~680 K rows.  Only z = D^-1 r, the vector the SpMV
// gathers from neighbouring rows, goes through global memory (and L2); the
// matrix is read as slot-major ELL (one coalesced 8-byte load per slot).
// Dot products are FP32 per thread and warp, FP64 per CTA and grid
// (rxg_gridsum.cuh); the FP64 scalar recurrence runs on thread 0 only.
#include <algorithm>
#include <cfloat>
#include <climits>
#include <cstdio>
#include <cstdlib>
#include <initializer_list>

#include "rxg_gridsum.cuh"
#include "rxg_lazy.h"
#include "rxg_mcf_common.cuh"

namespace rxg {

// CSR (diagonal first) -> slot-major ELL of width W: entry u of row i at
// ell[u * n + i]; short rows padded with (i, 0).  Every row must have at
// most W entries.
template <int W>
__global__ void k_csr_to_ell(int64_t n, const int32_t* __restrict__ rp, const Ent<float>* __restrict__ ent,
                             Ent<float>* __restrict__ ell)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t b = rp[i], len = rp[i + 1] - b;
#pragma unroll
        for (int u = 0; u < W; ++u) {
            Ent<float> e;
            if (u < len) {
                e = ent[b + u];
            } else {
                e.col = (int32_t)i;
                e.val = 0.f;
            }
            ell[u * n + i] = e;
        }
    }
}

struct OnchipArgs
{
    int64_t           n;
    const int32_t*    bounds; // CTA b owns rows [bounds[b], bounds[b+1])
    int32_t           cp;     // shared-memory stride of one component (>= any CTA's rows)
    const Ent<float>* ell;    // FP32 matrix, slot-major ELL, diagonal in slot 0
    const double*     diag;   // FP64 diagonal (2*area + sum of the FP32 weights)
    const R4<double>* B;
    R4<double>*       X;      // FP64 positions, updated in place
    R4<float>*        Z;      // z = D^-1 r, the gathered vector
    unsigned*         bar;
    double*           part;   // 2 * gridDim.x
    double*           dstat;  // rr0, rr
    int*              istat;  // iterations, converged, residual replacements
    double            tol;
    int               max_iter;
    int*              err;
};

// Residual replacement: r = B - A x in FP64 (FP32 off-diagonals promoted,
// FP64 diagonal), z = D^-1 r in FP32 into the CTA's shared copy and the
// global Z.  Returns this thread's share of r . diag^-1 r (FP64).
template <int BT, int W>
__device__ __forceinline__ double onchip_residual(const OnchipArgs& a, int64_t r0, int m,
                                                  const float* Dv, float* Zx, float* Zy, float* Zz)
{
    double part = 0.0;
    for (int l = threadIdx.x; l < m; l += BT) {
        const int64_t    i  = r0 + l;
        const R4<double> xi = a.X[i];
        const double     d  = a.diag[i];
        double           a0 = d * xi.x, a1 = d * xi.y, a2 = d * xi.z;
#pragma unroll
        for (int u0 = 1; u0 < W; u0 += 4) {
            Ent<float> q[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                if (u0 + u < W) {
                    q[u] = a.ell[(u0 + u) * a.n + i];
                } else {
                    q[u].col = (int32_t)i;
                    q[u].val = 0.f;
                }
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const double     v  = (double)q[u].val;
                const R4<double> xv = a.X[q[u].col];
                a0 += v * xv.x, a1 += v * xv.y, a2 += v * xv.z;
            }
        }
        const R4<double> b  = a.B[i];
        const double     e0 = b.x - a0, e1 = b.y - a1, e2 = b.z - a2;
        const float      di = Dv[l];
        R4<float>        z;
        z.x = di * (float)e0, z.y = di * (float)e1, z.z = di * (float)e2, z.w = 0.f;
        Zx[l] = z.x, Zy[l] = z.y, Zz[l] = z.z;
        a.Z[i] = z;
        part += (e0 * e0 + e1 * e1 + e2 * e2) * (double)di;  // ~ / diag, no FP64 divide
    }
    return part;
}

// scalar state of the solve, in shared memory (only thread 0 touches it, so
// it costs the other threads no registers)
struct OnchipScalars
{
    double rr0, rr, delta, rep;
    int    it, reps;
    bool   conv;
};

// values every thread reads after a reduction
struct OnchipShared
{
    float al, bt;
    int   first;    // next SpMV pass starts a new direction (s = A z, p = z)
    int   replace;  // replace the recursive residual by the FP64 one now
    int   stop;
};

// One FP32 Jacobi-PCG run on A d = r with FP64 residual replacement (van der
// Vorst & Ye, "Residual replacement strategies for Krylov subspace iterative
// methods for the convergence of true residuals", SIAM J. Sci. Comput. 2000):
// when the recursive r . z has dropped 1e4-fold since the last replacement,
// or below a quarter of the target, x += d in FP64, r = B - A x in FP64 and
// the iteration continues with the same direction.  The solve stops when the
// replaced residual meets r . diag^-1 r < tol^2 r0 . diag^-1 r0.
//
// Shared memory per row: p, s, z, d (3 floats each) and D^-1.  z = D^-1 r is
// kept instead of r (r . z = |z|^2 / D^-1), and it doubles as the local copy
// of the gathered vector: neighbours inside the CTA's chunk are read from
// shared memory, the others from the global Z.
template <int BT, int W>
__global__ void __launch_bounds__(BT, 1) k_mcf_onchip(OnchipArgs a)
{
    extern __shared__ __align__(16) float sm[];
    __shared__ RedSmem       red;
    __shared__ OnchipShared  sh;
    __shared__ OnchipScalars c;

    const int32_t cp = a.cp;
    float *Px = sm, *Py = Px + cp, *Pz = Py + cp;
    float *Sx = Pz + cp, *Sy = Sx + cp, *Sz = Sy + cp;
    float *Zx = Sz + cp, *Zy = Zx + cp, *Zz = Zy + cp;
    float *Dx = Zz + cp, *Dy = Dx + cp, *Dz = Dy + cp;
    float* Dv = Dz + cp;

    const int32_t r0i = a.bounds[blockIdx.x];
    const int64_t r0  = r0i;
    const int     m   = a.bounds[blockIdx.x + 1] - r0i;
    GridSum       g{a.bar, a.part, a.err, gridDim.x, 0u, blockIdx.x};
    const double  target = a.tol * a.tol;  // on rr / rr0

    for (int l = threadIdx.x; l < m; l += BT) {
        Dv[l] = 1.f / (a.ell[r0 + l].val + FLT_EPSILON);
        Dx[l] = Dy[l] = Dz[l] = 0.f;
        Px[l] = Py[l] = Pz[l] = 0.f;
        Sx[l] = Sy[l] = Sz[l] = 0.f;
    }
    __syncthreads();

    if (!grid_sum<BT>(onchip_residual<BT, W>(a, r0, m, Dv, Zx, Zy, Zz), g, red, [&](double t) {
            c.rr0 = c.rr = c.delta = c.rep = t;
            c.it = c.reps = 0;
            c.conv        = !(t > 0.0);
            sh.stop       = c.conv || a.max_iter <= 0;
            sh.first      = 1;
            sh.bt         = 0.f;
        }))
        return;

    while (!sh.stop) {
        const float bt    = sh.bt;
        const bool  first = sh.first != 0;
        // ---- s = A z + beta s, p = z + beta p, s . p
        float tp = 0.f;
        // W <= 8: the next row's ELL entries are loaded before this row's
        // gathers and arithmetic, so two rows' L2 round trips are in flight
        // per thread (one CTA of BT threads per SM leaves few warps to hide
        // them); the 16-slot form has no registers to spare for it
        constexpr bool PF = W <= 8;
        Ent<float>     qn[PF ? W : 1];
        if (PF && (int)threadIdx.x < m) {
#pragma unroll
            for (int u = 0; u < (PF ? W : 1); ++u) qn[u] = a.ell[u * a.n + r0 + threadIdx.x];
        }
        for (int l = threadIdx.x; l < m; l += BT) {
            Ent<float> q[W];
            if constexpr (PF) {
#pragma unroll
                for (int u = 0; u < W; ++u) q[u] = qn[u];
                if (l + BT < m) {
#pragma unroll
                    for (int u = 0; u < W; ++u) qn[u] = a.ell[u * a.n + r0 + l + BT];
                }
            } else {
#pragma unroll
                for (int u = 0; u < W; ++u) q[u] = a.ell[u * a.n + r0 + l];
            }
            float ax = 0.f, ay = 0.f, az = 0.f;
#pragma unroll
            for (int u = 0; u < W; ++u) {
                const int32_t lc = q[u].col - r0i;
                float         zx, zy, zz;
                if ((uint32_t)lc < (uint32_t)m) {
                    zx = Zx[lc], zy = Zy[lc], zz = Zz[lc];
                } else {
                    const R4<float> zv = a.Z[q[u].col];
                    zx = zv.x, zy = zv.y, zz = zv.z;
                }
                ax += q[u].val * zx, ay += q[u].val * zy, az += q[u].val * zz;
            }
            const float zx = Zx[l], zy = Zy[l], zz = Zz[l];
            float       sx, sy, sz, px, py, pz;
            if (first) {
                sx = ax, sy = ay, sz = az;
                px = zx, py = zy, pz = zz;
            } else {
                sx = ax + bt * Sx[l], sy = ay + bt * Sy[l], sz = az + bt * Sz[l];
                px = zx + bt * Px[l], py = zy + bt * Py[l], pz = zz + bt * Pz[l];
            }
            Sx[l] = sx, Sy[l] = sy, Sz[l] = sz;
            Px[l] = px, Py[l] = py, Pz[l] = pz;
            tp += sx * px + sy * py + sz * pz;
        }
        if (!grid_sum<BT>(tp, g, red, [&](double sp) { sh.al = (float)(c.delta / sp); })) return;
        const float al = sh.al;
        // ---- d += alpha p, z -= alpha D^-1 s, r . z
        tp = 0.f;
        for (int l = threadIdx.x; l < m; l += BT) {
            const float di = Dv[l];
            Dx[l] += al * Px[l], Dy[l] += al * Py[l], Dz[l] += al * Pz[l];
            const float ad = al * di;
            R4<float>   z;
            z.x = Zx[l] - ad * Sx[l], z.y = Zy[l] - ad * Sy[l], z.z = Zz[l] - ad * Sz[l], z.w = 0.f;
            Zx[l] = z.x, Zy[l] = z.y, Zz[l] = z.z;
            a.Z[r0 + l] = z;
            tp += __fdividef(z.x * z.x + z.y * z.y + z.z * z.z, di);
        }
        if (!grid_sum<BT>(tp, g, red, [&](double dn) {
                ++c.it;
                sh.replace = dn < 1e-4 * c.rep || dn < 0.25 * target * c.rr0 || c.it >= a.max_iter ||
                             !(dn > 0.0);
                if (!sh.replace) {
                    sh.bt    = (float)(dn / c.delta);
                    c.delta  = dn;
                    sh.first = 0;
                }
            }))
            return;
        if (sh.replace) {
            // x += d in FP64; every CTA's x in place before the residual gathers it
            for (int l = threadIdx.x; l < m; l += BT) {
                R4<double> x = a.X[r0 + l];
                x.x += (double)Dx[l], x.y += (double)Dy[l], x.z += (double)Dz[l];
                a.X[r0 + l] = x;
                Dx[l] = Dy[l] = Dz[l] = 0.f;
            }
            if (!grid_sum<BT>(0.f, g, red, [](double) {})) return;
            if (!grid_sum<BT>(onchip_residual<BT, W>(a, r0, m, Dv, Zx, Zy, Zz), g, red, [&](double t) {
                    ++c.reps;
                    c.rr     = t;
                    c.conv   = t < target * c.rr0;
                    sh.stop  = c.conv || c.it >= a.max_iter || !(t > 0.0);
                    sh.bt    = (float)(t / c.delta);
                    c.delta  = t;
                    c.rep    = t;
                    sh.first = 0;
                }))
                return;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.dstat[0] = c.rr0;
        a.dstat[1] = c.rr;
        a.istat[0] = c.it;
        a.istat[1] = c.conv ? 1 : 0;
        a.istat[2] = c.reps;
    }
}

// ---------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------

constexpr int kOnchipVecs = 13;  // p, s, r, d (3 each) and D^-1

static int env_choice(const char* name, int dflt, std::initializer_list<int> allowed)
{
    const char* e = getenv(name);
    if (!e) return dflt;
    const int v = atoi(e);
    for (int a : allowed)
        if (a == v) return v;
    return dflt;
}

// CTA size: RXG_MCF_ONCHIP_THREADS=512|1024 (default 512)
static int onchip_threads()
{
    static int t = env_choice("RXG_MCF_ONCHIP_THREADS", 512, {512, 1024});
    return t;
}

// RXG_MCF_ONCHIP=0 turns the on-chip solve off (the launch-per-sweep path runs)
static bool onchip_enabled()
{
    static int v = env_choice("RXG_MCF_ONCHIP", 1, {0, 1});
    return v == 1;
}

struct OnchipPlan
{
    int     G   = 0;
    int     W   = 0;
    int32_t cap = 0;  // most rows one CTA's shared memory holds (multiple of 32)
};

static bool onchip_plan(int64_t n, int64_t max_row, OnchipPlan* p)
{
    if (!onchip_enabled() || n <= 0 || n >= INT32_MAX) return false;
    p->W = max_row <= 8 ? 8 : (max_row <= 16 ? 16 : 0);
    if (!p->W) return false;
    int dev = 0, sms = 0, optin = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return false;
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
        return false;
    const int64_t static_smem = 1024;  // reduction scratch and scalars, with slack
    p->cap = (int32_t)(((optin - static_smem) / (kOnchipVecs * 4)) & ~int64_t(31));
    // one CTA per SM; small systems use fewer CTAs (at least 64 rows each)
    const int64_t G = std::max<int64_t>(1, std::min<int64_t>(sms, (n + 63) / 64));
    p->G            = (int)G;
    return p->cap > 0 && (n + G - 1) / G <= p->cap;
}

// Row ranges of the CTAs, balanced by cost: a row costs 1 plus 1 per entry
// whose column lies in another CTA's range (those gathers go to L2, the
// others to shared memory).  Two passes (the ranges decide which entries are
// remote); every range stays within the shared-memory cap.  Cached per mesh.
static rxg_status onchip_balance(Lazy* z, int64_t n, const OnchipPlan& p, cudaStream_t s)
{
    std::lock_guard<std::mutex> lk(z->mu);
    if ((int)z->oc_bounds.size() == p.G + 1 && z->d_oc_bounds) return RXG_OK;
    std::vector<int32_t> rp((size_t)n + 1), col((size_t)z->nnz);
    RXG_CUDA_TRY(cudaMemcpyAsync(rp.data(), z->row_ptr, 4 * (n + 1), cudaMemcpyDeviceToHost, s));
    RXG_CUDA_TRY(cudaMemcpyAsync(col.data(), z->col, 4 * z->nnz, cudaMemcpyDeviceToHost, s));
    RXG_CUDA_TRY(cudaStreamSynchronize(s));
    const int            G = p.G;
    std::vector<int32_t> B(G + 1), owner((size_t)n);
    for (int k = 0; k <= G; ++k) B[k] = (int32_t)((n * k) / G);
    std::vector<double> prefix((size_t)n + 1);
    for (int pass = 0; pass < 2; ++pass) {
        for (int k = 0; k < G; ++k)
            for (int32_t i = B[k]; i < B[k + 1]; ++i) owner[i] = k;
        prefix[0] = 0.0;
        for (int64_t i = 0; i < n; ++i) {
            int remote = 0;
            for (int32_t j = rp[i]; j < rp[i + 1]; ++j) remote += owner[col[j]] != owner[i];
            prefix[i + 1] = prefix[i] + 1.0 + remote;
        }
        std::vector<int32_t> nb(G + 1);
        nb[0] = 0;
        for (int k = 1; k < G; ++k) {
            const double target = prefix[n] * k / G;
            int64_t      idx = std::lower_bound(prefix.begin(), prefix.end(), target) - prefix.begin();
            idx = std::max<int64_t>(idx, (int64_t)nb[k - 1] + 1);
            idx = std::min<int64_t>(idx, (int64_t)nb[k - 1] + p.cap);
            idx = std::max<int64_t>(idx, n - (int64_t)(G - k) * p.cap);  // the rest must fit
            nb[k] = (int32_t)idx;
        }
        nb[G]   = (int32_t)n;
        bool ok = true;
        for (int k = 0; k < G && ok; ++k) ok = nb[k + 1] > nb[k] && nb[k + 1] - nb[k] <= p.cap;
        if (!ok) break;  // keep the previous (feasible) ranges
        B = nb;
    }
    int32_t mx = 0;
    for (int k = 0; k < G; ++k) mx = std::max(mx, B[k + 1] - B[k]);
    cudaFree(z->d_oc_bounds);
    z->d_oc_bounds = nullptr;
    RXG_CUDA_TRY(cudaMalloc(&z->d_oc_bounds, 4 * (G + 1)));
    RXG_CUDA_TRY(cudaMemcpyAsync(z->d_oc_bounds, B.data(), 4 * (G + 1), cudaMemcpyHostToDevice, s));
    RXG_CUDA_TRY(cudaStreamSynchronize(s));
    z->oc_bounds = B;
    z->oc_cp     = (mx + 31) & ~31;
    return RXG_OK;
}

bool mcf_onchip_fits(int64_t n, int64_t max_row)
{
    OnchipPlan p;
    return onchip_plan(n, max_row, &p);
}

static size_t a256(size_t b) { return (b + 255) & ~size_t(255); }

// scratch: barrier words (256 B), stats (256 B), partials (2 * G doubles),
// then the ELL copy of the matrix (W * n entries)
size_t mcf_onchip_scratch_bytes(int64_t n, int64_t max_row)
{
    OnchipPlan p;
    if (!onchip_plan(n, max_row, &p)) return 0;
    return 512 + a256(sizeof(double) * 2 * (size_t)p.G) + a256(sizeof(Ent<float>) * p.W * (size_t)n);
}

template <int BT, int W>
static rxg_status onchip_launch(const OnchipPlan& p, size_t smem, OnchipArgs& a, cudaStream_t s)
{
    const void* kern = (const void*)k_mcf_onchip<BT, W>;
    RXG_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    void* args[] = {&a};
    RXG_CUDA_TRY(cudaLaunchCooperativeKernel(kern, dim3(p.G), dim3(BT), args, smem, s));
    return RXG_OK;
}

rxg_status mcf_onchip_solve(Lazy* z, int64_t n, int64_t max_row, const void* ent_f32,
                            const double* diag, const void* B4, void* X4, void* Z4, void* scratch,
                            double tol, int max_iter, cudaStream_t s)
{
    OnchipPlan p;
    if (!onchip_plan(n, max_row, &p)) {
        set_error("mixed MCF: %lld rows do not fit the on-chip solver", (long long)n);
        return RXG_ERR_UNSUPPORTED;
    }
    rxg_status st = onchip_balance(z, n, p, s);
    if (st) return st;
    const size_t smem = (size_t)kOnchipVecs * 4 * (size_t)z->oc_cp;
    uint8_t*     q    = (uint8_t*)scratch;
    Ent<float>*  ell  = (Ent<float>*)(q + 512 + a256(sizeof(double) * 2 * (size_t)p.G));
    const int    gc   = (int)std::min<int64_t>((n + 255) / 256, 4096);
    if (p.W == 8)
        k_csr_to_ell<8><<<gc, 256, 0, s>>>(n, z->row_ptr, (const Ent<float>*)ent_f32, ell);
    else
        k_csr_to_ell<16><<<gc, 256, 0, s>>>(n, z->row_ptr, (const Ent<float>*)ent_f32, ell);
    RXG_CUDA_TRY(cudaGetLastError());
    OnchipArgs a;
    a.n          = n;
    a.bounds     = z->d_oc_bounds;
    a.cp         = z->oc_cp;
    a.ell        = ell;
    a.diag       = diag;
    a.B          = (const R4<double>*)B4;
    a.X          = (R4<double>*)X4;
    a.Z          = (R4<float>*)Z4;
    a.bar        = (unsigned*)q;
    a.dstat      = (double*)(q + 256);
    a.istat      = (int*)(q + 256 + 64);
    a.part       = (double*)(q + 512);
    a.tol        = tol;
    a.max_iter   = max_iter;
    a.err        = device_error_word();
    RXG_CUDA_TRY(cudaMemsetAsync(a.bar, 0, 16, s));
    const int bt = onchip_threads();
#define RXG_ONCHIP_CASE(BTV, WV) \
    if (bt == BTV && p.W == WV) return onchip_launch<BTV, WV>(p, smem, a, s);
    RXG_ONCHIP_CASE(512, 8)
    RXG_ONCHIP_CASE(1024, 8)
    RXG_ONCHIP_CASE(512, 16)
    RXG_ONCHIP_CASE(1024, 16)
#undef RXG_ONCHIP_CASE
    set_error("mixed MCF: no on-chip kernel for %d threads, width %d", bt, p.W);
    return RXG_ERR_UNSUPPORTED;
}

// statistics of the last mcf_onchip_solve on this scratch (synchronises s)
rxg_status mcf_onchip_stats(const void* scratch, rxg_solver_stats* st, cudaStream_t s)
{
    const uint8_t* q = (const uint8_t*)scratch;
    double         ds[2];
    int            is[3];
    RXG_CUDA_TRY(cudaMemcpyAsync(ds, q + 256, sizeof(ds), cudaMemcpyDeviceToHost, s));
    RXG_CUDA_TRY(cudaMemcpyAsync(is, q + 256 + 64, sizeof(is), cudaMemcpyDeviceToHost, s));
    RXG_CUDA_TRY(cudaStreamSynchronize(s));
    rxg_status e = check_device_error(s);
    if (e) return e;
    st->start_res = ds[0];
    st->final_res = ds[1];
    st->iters     = is[0];
    st->converged = is[1];
    if (getenv("RXG_MCF_VERBOSE"))
        fprintf(stderr, "rxg mcf onchip: replacements %d iterations %d converged %d rr %.3g -> %.3g\n",
                is[2], is[0], is[1], ds[0], ds[1]);
    return RXG_OK;
}

}  // namespace rxg
