// Batched implicit MCF: many meshes of uneven size in one persistent launch.
//
// The meshes are packed into one union mesh whose patches never span two
// components (RXG_MESH_SPLIT_COMPONENTS), so every mesh owns one contiguous
// range of linear vertex ids (the reference packs several meshes into one
// RXMeshStatic the same way, rxmesh_static.cu:66-160).
//
// Scheduling.  A mesh is a job for a gang of k CTAs: enough that no CTA holds
// more rows than the tile (its PCG state lives in shared memory) and that no
// job runs longer than half the ideal makespan.  Gangs run in waves: the
// host packs them longest first into waves of G CTAs, and all CTAs start
// each wave together after a grid barrier, so a gang's members arrive at
// once.  One-CTA jobs then come off a queue, largest first.  A gang
// synchronises through its own ticket counter (rxg_gridsum.cuh protocol with
// the gang's size), a one-CTA job only with __syncthreads; the launch is
// cooperative, so every CTA is resident.
//
// Per job, all flow steps run inside the launch: FP32 cotangent assembly (FP64
// for near-degenerate triangles and near-right Voronoi corners), FP64
// residual, and one FP32 Jacobi-PCG per step with FP64 residual replacement
// (the mixed solver of rxg_onchip.cu, here on global vectors).  No host round
// trips, so the call can be captured in a CUDA graph.  rxg_batch_autotune
// times the CTA size, CTAs per SM and the tile on the caller's batch.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <mutex>
#include <numeric>
#include <queue>
#include <vector>

#include "rxg_gridsum.cuh"
#include "rxg_lazy.h"
#include "rxg_mcf_common.cuh"

namespace rxg {

// one gang schedule (device arrays), built for a grid of G CTAs
struct GangPlan
{
    int      G = 0, bt = 0, bps = 0, tile = 0, kmax = 1, njobs = 0, cp = 0, nwaves = 0, nsingle = 0;
    size_t   smem  = 0;  // dynamic shared memory per CTA
    int      hints = 0;  // built with measured iteration counts
    int32_t* d_job_mesh  = nullptr;  // per job: mesh
    int32_t* d_job_k     = nullptr;  // per job: CTAs in its gang
    int32_t* d_wave_job  = nullptr;  // nwaves x G: the gang job CTA c runs in wave w, or -1
    int32_t* d_wave_rank = nullptr;  // nwaves x G: its rank in that gang
    int32_t* d_single    = nullptr;  // one-CTA jobs, largest first, taken from a queue
    unsigned* d_bar      = nullptr;  // 4 words per job, 4 for the grid barrier, 1 queue counter
    double*   d_part     = nullptr;  // 2 * kmax per job, then 2 * G for the grid barrier
    void free_all()
    {
        cudaFree(d_job_mesh);
        cudaFree(d_job_k);
        cudaFree(d_wave_job);
        cudaFree(d_wave_rank);
        cudaFree(d_single);
        cudaFree(d_bar);
        cudaFree(d_part);
        *this = GangPlan();
    }
};

}  // namespace rxg

struct rxg_batch
{
    rxg_mesh*            mesh  = nullptr;  // union of all meshes
    int32_t              nmesh = 0;
    std::vector<int64_t> voff, foff;       // input offsets per mesh (nmesh+1)
    std::vector<int32_t> vstart, vcount;   // linear vertex range per mesh
    int32_t*             d_vstart = nullptr;
    int32_t*             d_vcount = nullptr;
    int32_t*             d_iters  = nullptr;
    int32_t*             d_conv   = nullptr;
    void*                buf      = nullptr;
    size_t               buf_size = 0;
    int32_t              threads  = 512;
    int32_t              blocks_per_sm = 1;
    int32_t              tile          = 4096;
    std::vector<int32_t> iters_hint;  // PCG iterations per mesh seen by the autotuner (0: unknown)
    rxg::GangPlan        plan;
    std::mutex           mu;
};

namespace rxg {

struct BatchArgs
{
    const int32_t*    vstart;
    const int32_t*    vcount;
    const int32_t*    job_mesh;
    const int32_t*    job_k;
    int               nwaves, nsingle, njobs;
    const int32_t*    wave_job;
    const int32_t*    wave_rank;
    const int32_t*    single;
    unsigned*         bar;
    double*           part;
    int               kmax;
    int32_t           cp;    // shared-memory stride of one component (>= any CTA's rows)
    const int32_t*    row_ptr;
    const int32_t*    col;
    const int8_t*     bnd;
    int64_t           n;     // rows of the union (ELL slot stride)
    Ent<float>*       ent;   // CSR entries (W = 0) or slot-major ELL of width W
    R4<double>*       X;
    R4<double>*       B;
    R4<float>*        Z;     // z = D^-1 r of every row (read by the other CTAs of a gang)
    float*            dinv;
    double*           diag;  // FP64 diagonal (2*area + sum of the FP32 weights)
    float             dt;
    int32_t           nsteps;
    double            tol;
    int32_t           max_iter;
    int32_t*          iters;
    int32_t*          conv;
    int*              err;
};

__device__ __forceinline__ V3<double> pos4(const R4<double>* X, int32_t i)
{
    const R4<double> v = X[i];
    return {v.x, v.y, v.z};
}

// one row of the MCF system (mcf_A_setup / mcf_B_setup), FP32 weights with
// FP64 for near-degenerate triangles, positions from the packed FP64 state
// entry u of row p: CSR position row_ptr[p] + u, or ELL slot u
template <int W>
__device__ __forceinline__ int64_t ent_at(const BatchArgs& a, int64_t p, int32_t rp, int u)
{
    return W ? u * a.n + p : (int64_t)rp + u;
}

template <int W>
__device__ __forceinline__ void assemble_row(int64_t p, const BatchArgs& a)
{
    const int32_t    rp   = a.row_ptr[p];
    const int32_t    k    = a.row_ptr[p + 1] - rp - 1;
    const int32_t*   rg   = a.col + rp + 1;
    const bool       wrap = a.bnd[p] == 0;
    const V3<double> P    = pos4(a.X, (int32_t)p);
    double           area = 0.0, sumw = 0.0;  // FP64 row sums (see k_mcf_assemble)
    if (k > 0) {
        // FP64 and FP32 copies of each position made once (GeoMixed::Pt)
        const MixedPt Pp = GeoMixed::make(P);
        MixedPt       Q = GeoMixed::make(pos4(a.X, rg[k - 1])), R = GeoMixed::make(pos4(a.X, rg[0]));
        for (int32_t i = 0; i < k; ++i) {
            const MixedPt S     = GeoMixed::make(pos4(a.X, rg[i + 1 < k ? i + 1 : 0]));
            const bool    has_q = wrap || i > 0, has_s = wrap || i < k - 1;
            float         w     = 0.f;
            if (has_q) w += GeoMixed::hc(Pp, R, Q);
            if (has_s) w += GeoMixed::hc(Pp, R, S);
            w = (w >= 0.f ? w : 0.f) * a.dt;
            sumw += (double)w;
            Ent<float> e;
            e.col              = rg[i];
            e.val              = -w;
            a.ent[ent_at<W>(a, p, rp, 1 + i)] = e;
            if (has_q) {
                const float ar = GeoMixed::va(Pp, Q, R);
                area += ar > 0.f ? (double)ar : 0.0;
            }
            Q = R;
            R = S;
        }
    }
    const double vw = 0.5 / area;
    const double iv = 1.0 / vw;  // then products: GB300's FP64 divide is slow
    const double dg = iv + sumw;
    Ent<float>   d;
    d.col        = (int32_t)p;
    d.val        = (float)dg;
    a.ent[ent_at<W>(a, p, rp, 0)] = d;
    if (W) {
        Ent<float> z;
        z.col = (int32_t)p;
        z.val = 0.f;
        for (int u = k + 1; u < W; ++u) a.ent[ent_at<W>(a, p, rp, u)] = z;
    }
    a.diag[p]    = dg;
    a.dinv[p]    = 1.f / (d.val + FLT_EPSILON);
    R4<double> b;
    b.x     = P.x * iv;
    b.y     = P.y * iv;
    b.z     = P.z * iv;
    b.w     = 0.0;
    a.B[p]  = b;
}

// Per job, the CTA keeps its rows' PCG state in shared memory (the on-chip
// solver's layout, rxg_onchip.cu): p, s, z = D^-1 r, d (3 floats each) and
// D^-1, 52 bytes a row.  Neighbours inside the CTA's own rows are gathered
// from shared memory, the others (rows of the same mesh on another CTA of
// its gang) from the global z.
struct BatchSmem
{
    float *Px, *Py, *Pz, *Sx, *Sy, *Sz, *Zx, *Zy, *Zz, *Dx, *Dy, *Dz, *Dv;
};

// entry u of row i (ELL slot, or CSR position within the row)
template <int W>
__device__ __forceinline__ int32_t row_len(const BatchArgs& a, int64_t i)
{
    return W ? W : a.row_ptr[i + 1] - a.row_ptr[i];
}
template <int W>
__device__ __forceinline__ Ent<float> row_ent(const BatchArgs& a, int64_t i, int32_t u)
{
    return a.ent[W ? u * a.n + i : a.row_ptr[i] + u];
}

// r = B - A x in FP64 for rows [r0, r0 + m) (FP32 off-diagonals promoted,
// FP64 diagonal), z = D^-1 r into shared memory and the global z, d = 0;
// returns the thread's r . D^-1 r
template <int BT, int W>
__device__ __forceinline__ double batch_residual(int64_t r0, int m, const BatchArgs& a,
                                                 const BatchSmem& q)
{
    double part = 0;
    for (int l = threadIdx.x; l < m; l += BT) {
        const int64_t    i  = r0 + l;
        const R4<double> xi = a.X[i];
        const double     dg = a.diag[i];
        double           a0 = dg * xi.x, a1 = dg * xi.y, a2 = dg * xi.z;
        const int32_t    len = row_len<W>(a, i);
        for (int32_t u = 1; u < len; ++u) {
            const Ent<float> e  = row_ent<W>(a, i, u);
            const R4<double> xv = a.X[e.col];
            a0 += (double)e.val * xv.x;
            a1 += (double)e.val * xv.y;
            a2 += (double)e.val * xv.z;
        }
        const R4<double> b  = a.B[i];
        const double     e0 = b.x - a0, e1 = b.y - a1, e2 = b.z - a2;
        const float      di = q.Dv[l];
        R4<float>        z;
        z.x = di * (float)e0, z.y = di * (float)e1, z.z = di * (float)e2, z.w = 0.f;
        q.Zx[l] = z.x, q.Zy[l] = z.y, q.Zz[l] = z.z;
        q.Dx[l] = q.Dy[l] = q.Dz[l] = 0.f;
        a.Z[i] = z;
        part += (e0 * e0 + e1 * e1 + e2 * e2) * (double)di;  // ~ / diag, no FP64 divide
    }
    return part;
}

// scalar state of the job's solve (thread 0) and the values all threads read
struct BatchScalars
{
    double rr0, rr, delta, rep;
    int    it, total;
    bool   conv, conv_all;
};
struct BatchShared
{
    float al, bt;
    int   first, replace, stop;
};

// all flow steps of one mesh, rows [r0, r0 + m) of it on this CTA, gang g
template <int BT, int W>
__device__ bool batch_job(int64_t r0, int m, const BatchArgs& a, const BatchSmem& q, GridSum& g,
                          RedSmem& red, BatchScalars& c, BatchShared& sh)
{
    const double  target = a.tol * a.tol;
    const int32_t r0i    = (int32_t)r0;
    if (threadIdx.x == 0) {
        c.total    = 0;
        c.conv_all = true;
    }
    for (int step = 0; step < a.nsteps; ++step) {
        // positions of the whole mesh are final (the previous step ended with
        // a gang barrier after its last x update)
        for (int l = threadIdx.x; l < m; l += BT) {
            assemble_row<W>(r0 + l, a);
            q.Dv[l] = a.dinv[r0 + l];
            q.Px[l] = q.Py[l] = q.Pz[l] = q.Sx[l] = q.Sy[l] = q.Sz[l] = 0.f;
        }
        __syncthreads();
        if (!grid_sum<BT>(batch_residual<BT, W>(r0, m, a, q), g, red, [&](double t) {
                c.rr0 = c.rr = c.delta = c.rep = t;
                c.it                           = 0;
                c.conv                         = !(t > 0.0);
                sh.stop                        = c.conv || a.max_iter - c.total <= 0;
                sh.first                       = 1;
                sh.bt                          = 0.f;
            }))
            return false;
        while (!sh.stop) {
            const float bt    = sh.bt;
            const bool  first = sh.first != 0;
            // s = A z + beta s, p = z + beta p, s . p
            float tp = 0.f;
            for (int l = threadIdx.x; l < m; l += BT) {
                const int64_t i   = r0 + l;
                const int32_t len = row_len<W>(a, i);
                float         ax = 0.f, ay = 0.f, az = 0.f;
                for (int32_t u0 = 0; u0 < len; u0 += 8) {
                    Ent<float> e[8];
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        if (u0 + u < len) {
                            e[u] = row_ent<W>(a, i, u0 + u);
                        } else {
                            e[u].col = (int32_t)i;
                            e[u].val = 0.f;
                        }
                    }
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        const int32_t lc = e[u].col - r0i;
                        float         zx, zy, zz;
                        if ((uint32_t)lc < (uint32_t)m) {
                            zx = q.Zx[lc], zy = q.Zy[lc], zz = q.Zz[lc];
                        } else {
                            const R4<float> zv = a.Z[e[u].col];
                            zx = zv.x, zy = zv.y, zz = zv.z;
                        }
                        ax += e[u].val * zx, ay += e[u].val * zy, az += e[u].val * zz;
                    }
                }
                const float zx = q.Zx[l], zy = q.Zy[l], zz = q.Zz[l];
                float       sx, sy, sz, px, py, pz;
                if (first) {
                    sx = ax, sy = ay, sz = az;
                    px = zx, py = zy, pz = zz;
                } else {
                    sx = ax + bt * q.Sx[l], sy = ay + bt * q.Sy[l], sz = az + bt * q.Sz[l];
                    px = zx + bt * q.Px[l], py = zy + bt * q.Py[l], pz = zz + bt * q.Pz[l];
                }
                q.Sx[l] = sx, q.Sy[l] = sy, q.Sz[l] = sz;
                q.Px[l] = px, q.Py[l] = py, q.Pz[l] = pz;
                tp += sx * px + sy * py + sz * pz;
            }
            if (!grid_sum<BT>(tp, g, red, [&](double sp) { sh.al = (float)(c.delta / sp); })) return false;
            const float al = sh.al;
            // d += alpha p, z -= alpha D^-1 s, r . z
            tp = 0.f;
            for (int l = threadIdx.x; l < m; l += BT) {
                const float di = q.Dv[l];
                q.Dx[l] += al * q.Px[l], q.Dy[l] += al * q.Py[l], q.Dz[l] += al * q.Pz[l];
                const float ad = al * di;
                R4<float>   z;
                z.x = q.Zx[l] - ad * q.Sx[l], z.y = q.Zy[l] - ad * q.Sy[l], z.z = q.Zz[l] - ad * q.Sz[l];
                z.w = 0.f;
                q.Zx[l] = z.x, q.Zy[l] = z.y, q.Zz[l] = z.z;
                a.Z[r0 + l] = z;
                tp += __fdividef(z.x * z.x + z.y * z.y + z.z * z.z, di);
            }
            if (!grid_sum<BT>(tp, g, red, [&](double dn) {
                    ++c.it;
                    sh.replace = dn < 1e-4 * c.rep || dn < 0.25 * target * c.rr0 ||
                                 c.total + c.it >= a.max_iter || !(dn > 0.0);
                    if (!sh.replace) {
                        sh.bt    = (float)(dn / c.delta);
                        c.delta  = dn;
                        sh.first = 0;
                    }
                }))
                return false;
            if (sh.replace) {
                for (int l = threadIdx.x; l < m; l += BT) {
                    R4<double> x = a.X[r0 + l];
                    x.x += (double)q.Dx[l], x.y += (double)q.Dy[l], x.z += (double)q.Dz[l];
                    a.X[r0 + l] = x;
                }
                if (!grid_sum<BT>(0.f, g, red, [](double) {})) return false;
                if (!grid_sum<BT>(batch_residual<BT, W>(r0, m, a, q), g, red, [&](double t) {
                        c.rr     = t;
                        c.conv   = t < target * c.rr0;
                        sh.stop  = c.conv || c.total + c.it >= a.max_iter || !(t > 0.0);
                        sh.bt    = (float)(t / c.delta);
                        c.delta  = t;
                        c.rep    = t;
                        sh.first = 0;
                    }))
                    return false;
            }
        }
        if (threadIdx.x == 0) {
            c.total += c.it;
            c.conv_all = c.conv_all && c.conv;
        }
        __syncthreads();
    }
    return true;
}

// MINB: CTAs per SM the register allocation must allow (occupancy knob)
template <int BT, int W, int MINB>
__global__ void __launch_bounds__(BT, MINB) k_mcf_batch(BatchArgs a)
{
    extern __shared__ __align__(16) float sm[];
    __shared__ RedSmem      red;
    __shared__ BatchScalars c;
    __shared__ BatchShared  sh;
    const int32_t cp = a.cp;
    BatchSmem     q;
    q.Px = sm, q.Py = q.Px + cp, q.Pz = q.Py + cp;
    q.Sx = q.Pz + cp, q.Sy = q.Sx + cp, q.Sz = q.Sy + cp;
    q.Zx = q.Sz + cp, q.Zy = q.Zx + cp, q.Zz = q.Zy + cp;
    q.Dx = q.Zz + cp, q.Dy = q.Dx + cp, q.Dz = q.Dy + cp;
    q.Dv = q.Dz + cp;
    __shared__ int s_job;
    GridSum         grid{a.bar + 4 * a.njobs, a.part + 2 * a.kmax * a.njobs, a.err, gridDim.x, 0u,
                 blockIdx.x};
    // waves of gangs: every CTA takes part in every wave barrier
    for (int w = 0; w < a.nwaves; ++w) {
        const int32_t job = a.wave_job[w * gridDim.x + blockIdx.x];
        if (job >= 0) {
            const int32_t rank = a.wave_rank[w * gridDim.x + blockIdx.x];
            const int32_t mesh = a.job_mesh[job], k = a.job_k[job];
            const int64_t v0 = a.vstart[mesh], nv = a.vcount[mesh];
            const int64_t chunk = (nv + k - 1) / k;
            const int64_t lo    = rank * chunk, hi = lo + chunk;
            const int64_t r0    = v0 + (lo < nv ? lo : nv);
            const int64_t r1    = v0 + (hi < nv ? hi : nv);
            GridSum       g{a.bar + 4 * job, a.part + 2 * a.kmax * job, a.err, (unsigned)k, 0u,
                      (unsigned)rank};
            if (!batch_job<BT, W>(r0, (int)(r1 - r0), a, q, g, red, c, sh)) return;
            if (rank == 0 && threadIdx.x == 0) {
                a.iters[mesh] = c.total;
                a.conv[mesh]  = c.conv_all ? 1 : 0;
            }
        }
        if (!grid_sum<BT>(0.f, grid, red, [](double) {})) return;
    }
    // one-CTA jobs from a queue, largest first
    unsigned* queue = a.bar + 4 * a.njobs + 4;
    while (true) {
        if (threadIdx.x == 0) s_job = (int)atomicAdd(queue, 1u);
        __syncthreads();
        const int t = s_job;
        __syncthreads();
        if (t >= a.nsingle) break;
        const int32_t job  = a.single[t];
        const int32_t mesh = a.job_mesh[job];
        GridSum       g{a.bar + 4 * job, a.part + 2 * a.kmax * job, a.err, 1u, 0u, 0u};
        if (!batch_job<BT, W>(a.vstart[mesh], a.vcount[mesh], a, q, g, red, c, sh)) return;
        if (threadIdx.x == 0) {
            a.iters[mesh] = c.total;
            a.conv[mesh]  = c.conv_all ? 1 : 0;
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

// the kernel for a CTA size, ELL width and CTAs per SM
static const void* batch_kernel(int bt, int w, int bps)
{
#define RXG_BK(BTV, MB) (w == 8 ? (const void*)k_mcf_batch<BTV, 8, MB>       \
                         : w == 16 ? (const void*)k_mcf_batch<BTV, 16, MB> \
                                   : (const void*)k_mcf_batch<BTV, 0, MB>)
    if (bt == 256) return bps >= 4 ? RXG_BK(256, 4) : RXG_BK(256, 2);
    if (bt == 1024) return RXG_BK(1024, 1);
    return bps >= 2 ? RXG_BK(512, 2) : RXG_BK(512, 1);
#undef RXG_BK
}

static int max_per_sm(int bt, int w, int bps, size_t smem = 0)
{
    const void* kern = batch_kernel(bt, w, bps);
    if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int per = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, bt, smem) != cudaSuccess) per = 0;
    return per;
}

constexpr int kGangMax     = 64;    // most CTAs one mesh is split across
constexpr int kBatchStatic = 1024;  // static shared memory of the kernel, with slack

static int batch_optin_smem()
{
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    return optin;
}

// Schedule for G CTAs and the given tile (most rows per CTA).  A job's work
// is rows x PCG iterations: the iterations the autotuner measured when
// known, else sqrt(rows) (a mesh Laplacian's PCG count grows like its
// diameter).
static int batch_ell_width(const rxg_batch* b);

static rxg_status build_plan(rxg_batch* b, int bt, int bps, int tile, GangPlan* out)
{
    const int  w    = batch_ell_width(b);
    const int  nm   = b->nmesh;
    const bool hint = (int)b->iters_hint.size() == nm;
    std::vector<double> it(nm), work(nm);
    double              total = 0.0;
    for (int m = 0; m < nm; ++m) {
        it[m]   = hint && b->iters_hint[m] > 0 ? (double)b->iters_hint[m] : std::sqrt((double)b->vcount[m]);
        work[m] = it[m] * (double)b->vcount[m];
        total += work[m];
    }
    // rows per CTA bound the shared memory: 13 floats a row
    const int optin = batch_optin_smem();
    const int G     = batch_sms() * bps;
    // gang sizes
    std::vector<int32_t> kk(nm);
    int                  kmax      = 1;
    int64_t              max_chunk = 1;
    for (int m = 0; m < nm; ++m) {
        const int64_t nv = b->vcount[m];
        int64_t       k  = (nv + tile - 1) / tile;
        k = std::max<int64_t>(k, (int64_t)std::ceil(work[m] * G / (0.5 * total)));
        k = std::max<int64_t>(1, std::min<int64_t>({k, (int64_t)kGangMax, (int64_t)G, nv}));
        kk[m]     = (int32_t)k;
        kmax      = std::max(kmax, (int)k);
        max_chunk = std::max(max_chunk, (nv + k - 1) / k);
    }
    const int    cp   = (int)((max_chunk + 31) & ~int64_t(31));
    const size_t smem = (size_t)13 * 4 * cp;
    if ((int64_t)smem + kBatchStatic > optin || max_per_sm(bt, w, bps, smem) < bps) {
        set_error("rxg_batch: %d CTAs of %d threads per SM with %lld rows each do not fit an SM",
                  bps, bt, (long long)max_chunk);
        return RXG_ERR_UNSUPPORTED;
    }
    // Gangs (k >= 2) run in waves that start together after a grid barrier,
    // longest first, first-fit into G CTAs; one-CTA jobs then come off a queue,
    // largest first, so their durations need no estimate.
    const double         sync_rows = 1000.0;  // a gang's two grid sums, in row-iterations
    std::vector<int32_t> gangs, singles;
    for (int m = 0; m < nm; ++m) (kk[m] > 1 ? gangs : singles).push_back(m);
    auto dur = [&](int32_t m) { return work[m] / kk[m] + (kk[m] > 1 ? it[m] * sync_rows : 0.0); };
    std::stable_sort(gangs.begin(), gangs.end(), [&](int32_t x, int32_t y) { return dur(x) > dur(y); });
    std::stable_sort(singles.begin(), singles.end(), [&](int32_t x, int32_t y) { return work[x] > work[y]; });
    std::vector<std::vector<int32_t>> waves;
    std::vector<int>                  used;
    for (int32_t m : gangs) {
        size_t wv = 0;
        while (wv < waves.size() && used[wv] + kk[m] > G) ++wv;
        if (wv == waves.size()) {
            waves.emplace_back();
            used.push_back(0);
        }
        waves[wv].push_back(m);
        used[wv] += kk[m];
    }
    // jobs: gangs in wave order, then the singles; job index = position
    std::vector<int32_t> job_mesh, job_k, wave_job(waves.size() * (size_t)G, -1),
        wave_rank(waves.size() * (size_t)G, 0), single;
    for (size_t wv = 0; wv < waves.size(); ++wv) {
        int c = 0;
        for (int32_t m : waves[wv]) {
            const int32_t job = (int32_t)job_mesh.size();
            job_mesh.push_back(m);
            job_k.push_back(kk[m]);
            for (int r = 0; r < kk[m]; ++r, ++c) {
                wave_job[wv * G + c]  = job;
                wave_rank[wv * G + c] = r;
            }
        }
    }
    for (int32_t m : singles) {
        single.push_back((int32_t)job_mesh.size());
        job_mesh.push_back(m);
        job_k.push_back(1);
    }
    GangPlan p;
    p.G = G, p.bt = bt, p.bps = bps, p.tile = tile, p.kmax = kmax, p.njobs = nm;
    p.cp = cp, p.smem = smem, p.hints = hint ? 1 : 0;
    p.nwaves = (int)waves.size(), p.nsingle = (int)single.size();
    auto up = [](int32_t** d, const std::vector<int32_t>& h) -> cudaError_t {
        cudaError_t e = cudaMalloc(d, std::max<size_t>(h.size(), 1) * 4);
        if (e == cudaSuccess && !h.empty())
            e = cudaMemcpy(*d, h.data(), h.size() * 4, cudaMemcpyHostToDevice);
        return e;
    };
    cudaError_t e = up(&p.d_job_mesh, job_mesh);
    if (e == cudaSuccess) e = up(&p.d_job_k, job_k);
    if (e == cudaSuccess) e = up(&p.d_wave_job, wave_job);
    if (e == cudaSuccess) e = up(&p.d_wave_rank, wave_rank);
    if (e == cudaSuccess) e = up(&p.d_single, single);
    if (e == cudaSuccess) e = cudaMalloc(&p.d_bar, sizeof(unsigned) * (4 * nm + 8));
    if (e == cudaSuccess) e = cudaMalloc(&p.d_part, sizeof(double) * (2 * kmax * nm + 2 * G));
    if (e != cudaSuccess) {
        p.free_all();
        return cuda_status(e, "rxg_batch: gang schedule");
    }
    *out = p;
    return RXG_OK;
}

// the batch's current plan for (threads, CTAs per SM, tile), rebuilt on change
static rxg_status ensure_plan(rxg_batch* b, int bt, int bps, int tile)
{
    std::lock_guard<std::mutex> g(b->mu);
    const int hints = (int)b->iters_hint.size() == b->nmesh ? 1 : 0;
    if (b->plan.G && b->plan.bt == bt && b->plan.bps == bps && b->plan.tile == tile &&
        b->plan.hints == hints)
        return RXG_OK;
    b->plan.free_all();
    return build_plan(b, bt, bps, tile, &b->plan);
}

// ELL width of the union's matrix (rows = valence + 1), 0 for CSR
static int batch_ell_width(const rxg_batch* b)
{
    const int64_t r = b->mesh->m.max_valence + 1;
    return r <= 8 ? 8 : (r <= 16 ? 16 : 0);
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
    const int64_t n = b->mesh->m.nv, w = batch_ell_width(b);
    const int64_t nnz   = w ? w * n : z->nnz;
    const size_t  bytes = a256(sizeof(Ent<float>) * nnz) + 2 * a256(sizeof(R4<double>) * n) +
                         a256(sizeof(R4<float>) * n) + a256(sizeof(float) * n) +
                         a256(sizeof(double) * n);
    {
        std::lock_guard<std::mutex> g(b->mu);
        if ((st = batch_buffers(b, bytes))) return st;
    }
    uint8_t*  q = (uint8_t*)b->buf;
    BatchArgs a;
    a.vstart  = b->d_vstart;
    a.vcount  = b->d_vcount;
    a.row_ptr = z->row_ptr;
    a.col     = z->col;
    a.bnd     = z->bnd;
    a.n       = n;
    a.ent = (Ent<float>*)q, q += a256(sizeof(Ent<float>) * nnz);
    a.X = (R4<double>*)q, q += a256(sizeof(R4<double>) * n);
    a.B = (R4<double>*)q, q += a256(sizeof(R4<double>) * n);
    a.Z = (R4<float>*)q, q += a256(sizeof(R4<float>) * n);
    a.dinv  = (float*)q, q += a256(sizeof(float) * n);
    a.diag  = (double*)q;
    a.iters = b->d_iters;
    a.conv  = b->d_conv;
    a.err   = device_error_word();
    *out    = a;
    *X4     = a.X;
    return RXG_OK;
}

static rxg_status batch_launch(rxg_batch* b, BatchArgs a, int bt, int bps, int tile, cudaStream_t s)
{
    rxg_status st = ensure_plan(b, bt, bps, tile);
    if (st) return st;
    const GangPlan& p = b->plan;
    a.job_mesh  = p.d_job_mesh;
    a.job_k     = p.d_job_k;
    a.nwaves    = p.nwaves;
    a.nsingle   = p.nsingle;
    a.njobs     = p.njobs;
    a.wave_job  = p.d_wave_job;
    a.wave_rank = p.d_wave_rank;
    a.single    = p.d_single;
    a.bar      = p.d_bar;
    a.part     = p.d_part;
    a.kmax     = p.kmax;
    a.cp       = p.cp;
    RXG_CUDA_TRY(cudaMemsetAsync(p.d_bar, 0, sizeof(unsigned) * (4 * p.njobs + 8), s));
    void*       args[] = {&a};
    const void* kern = batch_kernel(bt, batch_ell_width(b), bps);
    RXG_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p.smem));
    cudaLaunchConfig_t   cfg  = {};
    cudaLaunchAttribute  attr = {};
    attr.id               = cudaLaunchAttributeCooperative;
    attr.val.cooperative  = 1;
    cfg.gridDim           = dim3(p.G);
    cfg.blockDim          = dim3(bt);
    cfg.dynamicSmemBytes  = p.smem;
    cfg.stream            = s;
    cfg.attrs             = &attr;
    cfg.numAttrs          = 1;
    RXG_CUDA_TRY(cudaLaunchKernelExC(&cfg, kern, args));
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
    auto up = [&](int32_t** d, const void* h, size_t n) -> cudaError_t {
        cudaError_t e = cudaMalloc(d, std::max<size_t>(n, 1) * 4);
        if (e == cudaSuccess && h) e = cudaMemcpy(*d, h, n * 4, cudaMemcpyHostToDevice);
        return e;
    };
    cudaError_t e = up(&b->d_vstart, b->vstart.data(), nmesh);
    if (e == cudaSuccess) e = up(&b->d_vcount, b->vcount.data(), nmesh);
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
    b->plan.free_all();
    cudaFree(b->d_vstart);
    cudaFree(b->d_vcount);
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
    if ((st = batch_launch(b, a, b->threads, b->blocks_per_sm, b->tile, s))) return st;
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

// Runs the batch once to learn each mesh's PCG iteration count (the cost of
// its job in every later schedule), then times CTA size x CTAs per SM x tile
// (most rows per CTA) on the caller's batch and keeps the fastest (xyz is
// not modified).
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
    // one run of the current configuration gives every mesh's iteration count,
    // which the schedules below use as the cost of its job
    k_batch_pack<<<g, 256, 0, s>>>(n, b->mesh->m.d.v_l2i, xyz, X4);
    if ((st = batch_launch(b, a, b->threads, b->blocks_per_sm, b->tile, s))) return st;
    {
        std::vector<int32_t> it(b->nmesh);
        RXG_CUDA_TRY(cudaMemcpyAsync(it.data(), b->d_iters, 4 * b->nmesh, cudaMemcpyDeviceToHost, s));
        RXG_CUDA_TRY(cudaStreamSynchronize(s));
        std::lock_guard<std::mutex> lk(b->mu);
        b->iters_hint = it;
    }
    float best = 1e30f;
    int   bt_best = b->threads, bps_best = b->blocks_per_sm, tile_best = b->tile;
    for (int bt : {256, 512, 1024}) {
        for (int bps : {1, 2}) {
            if (bt * bps > 2048) continue;
            for (int tile : {1024, 2048, 4096}) {
                float t = 0;
                bool  ok = true;
                for (int rep = 0; rep < 2; ++rep) {
                    k_batch_pack<<<g, 256, 0, s>>>(n, b->mesh->m.d.v_l2i, xyz, X4);
                    cudaEventRecord(e0, s);
                    rxg_status r = batch_launch(b, a, bt, bps, tile, s);
                    cudaEventRecord(e1, s);
                    cudaEventSynchronize(e1);
                    if (r == RXG_ERR_UNSUPPORTED) {  // this shape does not fit an SM
                        ok = false;
                        break;
                    }
                    if (r) {
                        st = r;
                        break;
                    }
                    cudaEventElapsedTime(&t, e0, e1);  // second repetition is kept
                }
                if (st) break;
                if (ok && t < best) {
                    best      = t;
                    bt_best   = bt;
                    bps_best  = bps;
                    tile_best = tile;
                }
            }
            if (st) break;
        }
        if (st) break;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st) return st;
    b->threads       = bt_best;
    b->blocks_per_sm = bps_best;
    b->tile          = tile_best;
    if ((st = ensure_plan(b, bt_best, bps_best, tile_best))) return st;
    if (threads) *threads = bt_best;
    if (blocks_per_sm) *blocks_per_sm = bps_best;
    if (best_ms) *best_ms = best;
    return check_device_error(s);
}

}  // extern "C"
