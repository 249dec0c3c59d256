// Oriented one-ring, cotangent-Laplacian assembly, SpMM, persistent CG/PCG
// and the implicit mean-curvature-flow step (plain FP64 and mixed FP32 with
// FP64 iterative refinement).
#include <algorithm>
#include <cfloat>
#include <mutex>

#include "rxg_device.cuh"

namespace rxg {

constexpr int kQT2 = 256;

size_t query_smem_bytes(const Mesh* m, int kind);

// ---------------------------------------------------------------------
// per-mesh lazily built structures
// ---------------------------------------------------------------------

struct Lazy
{
    std::mutex mu;
    bool       ring_ready = false;
    int32_t*   ring_off   = nullptr;  // nv+1, linear ids
    int32_t*   ring       = nullptr;  // 2*ne
    int8_t*    bnd        = nullptr;  // nv
    int32_t*   row_ptr    = nullptr;  // nv+1  (= ring_off + p)
    int32_t*   col        = nullptr;  // nnz   (diagonal first, then the ring)
    int64_t    nnz        = 0;
    // MCF step scratch (sized for this mesh)
    void*   buf      = nullptr;
    size_t  buf_size = 0;
};

static std::mutex g_lazy_mu;

Lazy* lazy_of(const Mesh* cm)
{
    Mesh*                       m = const_cast<Mesh*>(cm);
    std::lock_guard<std::mutex> g(g_lazy_mu);
    if (!m->lazy) m->lazy = new Lazy();
    return static_cast<Lazy*>(m->lazy);
}

void lazy_free(Mesh* m)
{
    Lazy* z = static_cast<Lazy*>(m->lazy);
    if (!z) return;
    cudaFree(z->ring_off);
    cudaFree(z->ring);
    cudaFree(z->bnd);
    cudaFree(z->row_ptr);
    cudaFree(z->col);
    cudaFree(z->buf);
    delete z;
    m->lazy = nullptr;
}

// ---------------------------------------------------------------------
// input <-> linear permutation of per-element arrays
// ---------------------------------------------------------------------

template <typename W>
__global__ void k_permute(int64_t n, int32_t nc, const int32_t* __restrict__ l2i, int32_t to_lin,
                          const W* __restrict__ src, W* __restrict__ dst)
{
    const int64_t total = n * nc;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t lin = i / nc, c = i - lin * nc;
        const int64_t inp = l2i[lin];
        if (to_lin)
            dst[i] = src[inp * nc + c];
        else
            dst[inp * nc + c] = src[i];
    }
}

static int grid_for(int64_t work, int threads = 256)
{
    int64_t b = (work + threads - 1) / threads;
    return (int)std::max<int64_t>(1, std::min<int64_t>(b, 152 * 32));
}

// ---------------------------------------------------------------------
// Oriented VV: per patch, VF transpose in shared memory, then one thread per
// owned vertex walks its fan (face (p,a,b) is followed by the face whose
// second vertex is b), as orient_edges_around_vertices does
// (kernels/rxmesh_queries.cuh:376-499).  A boundary fan starts at the face
// whose 'a' ends no other face; an interior fan at its lowest local face.
// ---------------------------------------------------------------------

__device__ __forceinline__ uint32_t fv_of(const uint16_t* fe16, const uint32_t* s_ev, int f, int k)
{
    uint32_t fe = fe16[3 * f + k];
    uint32_t ev = s_ev[fe >> 1];
    return (fe & 1u) ? (ev >> 16) : (ev & 0xffffu);
}

__global__ void __launch_bounds__(kQT2) k_oriented_vv(const PatchHdr* __restrict__ hdrs,
                                                      const uint32_t* __restrict__ arena,
                                                      int32_t* __restrict__ out_off,
                                                      int32_t* __restrict__ out_val,
                                                      int8_t* __restrict__ out_bnd, int* err)
{
    extern __shared__ __align__(16) uint32_t smem[];
    __shared__ uint64_t bar;
    __shared__ int32_t  s_warp[kQT2 / 32];

    PatchHdr h;
    {
        const int4* p = reinterpret_cast<const int4*>(hdrs + blockIdx.x);
        int4*       q = reinterpret_cast<int4*>(&h);
        for (int i = 0; i < 4; ++i) q[i] = __ldg(p + i);
    }
    const int32_t nVo = h.nVo, nVr = h.nVl - h.nVo;
    const int32_t few = pad4i((3 * h.nFl + 1) / 2);
    uint32_t* s_ev   = smem;
    uint32_t* s_fe   = s_ev + pad4i(h.nEl);
    uint32_t* s_rv   = s_fe + few;
    int32_t*  s_fcnt = reinterpret_cast<int32_t*>(s_rv + pad4i(nVr));  // VF offsets
    int32_t*  s_ecnt = s_fcnt + pad4i(nVo + 1);                           // valences
    int32_t*  s_vf   = s_ecnt + pad4i(nVo + 1);                           // VF values (local)

    if (threadIdx.x == 0) mbar_init(&bar, 1);
    for (int i = threadIdx.x; i <= nVo; i += kQT2) {
        s_fcnt[i] = 0;
        s_ecnt[i] = 0;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const uint32_t b0 = pad16_bytes(h.nEl), b1 = (uint32_t)few * 4, b2 = pad16_bytes(nVr);
        mbar_arrive_expect_tx(&bar, b0 + b1 + b2);
        if (b0) bulk_g2s(s_ev, arena + h.ev_off, b0, &bar);
        if (b1) bulk_g2s(s_fe, arena + h.fe_off, b1, &bar);
        if (b2) bulk_g2s(s_rv, arena + h.rv_off, b2, &bar);
    }
    if (!mbar_wait_bounded(&bar, 0, err)) return;
    const uint16_t* fe16 = reinterpret_cast<const uint16_t*>(s_fe);

    for (int i = threadIdx.x; i < 3 * h.nFl; i += kQT2) {
        uint32_t v = fv_of(fe16, s_ev, i / 3, i % 3);
        if ((int32_t)v < nVo) atomicAdd(&s_fcnt[v], 1);
    }
    for (int e = threadIdx.x; e < h.nEl; e += kQT2) {
        uint32_t ev = s_ev[e];
        if ((int32_t)(ev & 0xffffu) < nVo) atomicAdd(&s_ecnt[ev & 0xffffu], 1);
        if ((int32_t)(ev >> 16) < nVo) atomicAdd(&s_ecnt[ev >> 16], 1);
    }
    __syncthreads();
    block_exclusive_scan<kQT2>(s_fcnt, nVo + 1, s_warp);
    block_exclusive_scan<kQT2>(s_ecnt, nVo + 1, s_warp);
    for (int v = threadIdx.x; v <= nVo; v += kQT2) out_off[h.v_base + v] = h.vv_base + s_ecnt[v];
    __syncthreads();
    // VF scatter: cursor = s_fcnt shifted copy kept in s_fcnt; use a second pass
    // with atomics on a cursor array laid over s_vf's tail would cost memory;
    // instead recount with atomics into the offsets and restore afterwards.
    for (int i = threadIdx.x; i < 3 * h.nFl; i += kQT2) {
        int      f = i / 3;
        uint32_t v = fv_of(fe16, s_ev, f, i % 3);
        if ((int32_t)v < nVo) s_vf[atomicAdd(&s_fcnt[v], 1)] = f;
    }
    __syncthreads();
    // s_fcnt[v] now holds the end of row v; row v starts at s_fcnt[v-1] (0 for v=0)

    auto lin = [&](uint32_t l) -> int32_t {
        return (int32_t)l < nVo ? h.v_base + (int32_t)l : (int32_t)s_rv[l - nVo];
    };
    for (int v = threadIdx.x; v < nVo; v += kQT2) {
        const int32_t beg = v == 0 ? 0 : s_fcnt[v - 1], end = s_fcnt[v], k = end - beg;
        const int32_t obeg = h.vv_base + s_ecnt[v], olen = s_ecnt[v + 1] - s_ecnt[v];
        int32_t*      o    = out_val + obeg;
        if (k == 0) {
            out_bnd[h.v_base + v] = 0;
            continue;
        }
        // (a, b): the vertices following v in face order
        auto ab = [&](int j, uint32_t& a, uint32_t& b) {
            int f = s_vf[beg + j];
            int c = fv_of(fe16, s_ev, f, 0) == (uint32_t)v ? 0 : (fv_of(fe16, s_ev, f, 1) == (uint32_t)v ? 1 : 2);
            a     = fv_of(fe16, s_ev, f, (c + 1) % 3);
            b     = fv_of(fe16, s_ev, f, (c + 2) % 3);
        };
        int start = -1, jmin = 0, fmin = 1 << 30;
        for (int j = 0; j < k && start < 0; ++j) {
            uint32_t a, b;
            ab(j, a, b);
            if (s_vf[beg + j] < fmin) {
                fmin = s_vf[beg + j];
                jmin = j;
            }
            bool found = false;
            for (int t = 0; t < k; ++t) {
                uint32_t a2, b2;
                ab(t, a2, b2);
                if (b2 == a) {
                    found = true;
                    break;
                }
            }
            if (!found) start = j;
        }
        const bool is_b = start >= 0;
        if (!is_b) {
            for (int j = 0; j < k; ++j)
                if (s_vf[beg + j] < fmin) {
                    fmin = s_vf[beg + j];
                    jmin = j;
                }
            start = jmin;
        }
        int      cur = start, nvis = 0, pos = 0;
        uint32_t a, b;
        ab(cur, a, b);
        if (pos < olen) o[pos] = lin(a);
        ++pos;
        bool bad = false;
        while (true) {
            ++nvis;
            ab(cur, a, b);
            int nxt = -1;
            for (int t = 0; t < k; ++t) {
                uint32_t a2, b2;
                ab(t, a2, b2);
                if (a2 == b) {
                    nxt = t;
                    break;
                }
            }
            if (nxt < 0 || nxt == start) {
                if (is_b) {
                    if (pos < olen) o[pos] = lin(b);
                    ++pos;
                }
                break;
            }
            if (nvis >= k) {
                bad = true;
                break;
            }
            if (pos < olen) o[pos] = lin(b);
            ++pos;
            cur = nxt;
        }
        if (bad || nvis != k || pos != olen) atomicOr(err, DEVERR_NONMANIFOLD);
        out_bnd[h.v_base + v] = is_b ? 1 : 0;
    }
}

// A pattern from the ring: row_ptr[p] = ring_off[p] + p, col = [p, ring...]
__global__ void k_pattern(int64_t nv, const int32_t* __restrict__ ring_off,
                          const int32_t* __restrict__ ring, int32_t* __restrict__ row_ptr,
                          int32_t* __restrict__ col)
{
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p <= nv;
         p += (int64_t)gridDim.x * blockDim.x) {
        const int32_t rp = ring_off[p] + (int32_t)p;
        row_ptr[p]       = rp;
        if (p == nv) break;
        col[rp] = (int32_t)p;
        for (int32_t j = ring_off[p]; j < ring_off[p + 1]; ++j) col[rp + 1 + (j - ring_off[p])] = ring[j];
    }
}

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
        if (near_degenerate(pf, qf, rf)) return (float)voronoi<double>(p, q, r);
        return voronoi<float>(pf, qf, rf);
    }
};

__device__ __forceinline__ V3<double> ld3(const double* __restrict__ x, int32_t i)
{
    return {__ldg(x + 3 * (int64_t)i), __ldg(x + 3 * (int64_t)i + 1), __ldg(x + 3 * (int64_t)i + 2)};
}

// ---------------------------------------------------------------------
// MCF system (mcf_A_setup / mcf_B_setup, apps/MCF/mcf_kernels.cuh:302-426).
// One thread per vertex walks its oriented ring with a rolling window of
// three positions; the row is [diag, ring...] so no column search is done.
// Interior rows wrap (q of the first neighbour is the last one); boundary
// rows use only the fan's real triangles.
// ---------------------------------------------------------------------

template <typename T, typename G, typename TB>
__global__ void __launch_bounds__(256) k_mcf_assemble(int64_t nv, const int32_t* __restrict__ row_ptr,
                                                      const int32_t* __restrict__ col,
                                                      const int8_t* __restrict__ bnd,
                                                      const double* __restrict__ xyz, T dt,
                                                      T* __restrict__ val, TB* __restrict__ B)
{
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nv;
         p += (int64_t)gridDim.x * blockDim.x) {
        const int32_t rp   = row_ptr[p];
        const int32_t k    = row_ptr[p + 1] - rp - 1;
        const int32_t* rg  = col + rp + 1;
        const bool    wrap = bnd[p] == 0;
        const V3<double> P = ld3(xyz, (int32_t)p);
        T                area = T(0), sumw = T(0);
        if (k > 0) {
            V3<double> Q = ld3(xyz, rg[k - 1]), R = ld3(xyz, rg[0]);
            for (int32_t i = 0; i < k; ++i) {
                const V3<double> S = ld3(xyz, rg[i + 1 < k ? i + 1 : 0]);
                const bool has_q = wrap || i > 0, has_s = wrap || i < k - 1;
                T          w     = T(0);
                if (has_q) w += G::hc(P, R, Q);
                if (has_s) w += G::hc(P, R, S);
                w = (w >= T(0) ? w : T(0)) * dt;
                sumw += w;
                val[rp + 1 + i] = -w;
                if (has_q) {
                    const T a = G::va(P, Q, R);
                    area += a > T(0) ? a : T(0);
                }
                Q = R;
                R = S;
            }
        }
        const T vw  = T(0.5) / area;
        val[rp]     = T(1) / vw + sumw;
        if (B) {
            B[3 * p + 0] = (TB)P.x / (TB)vw;
            B[3 * p + 1] = (TB)P.y / (TB)vw;
            B[3 * p + 2] = (TB)P.z / (TB)vw;
        }
    }
}

// ---------------------------------------------------------------------
// SpMM / residual: one thread per row, nc right-hand sides row-major
// ---------------------------------------------------------------------

template <typename TA, typename TX, typename TACC, int NC, bool RESID>
__global__ void __launch_bounds__(256) k_spmm(int64_t n, const int32_t* __restrict__ rp,
                                              const int32_t* __restrict__ col,
                                              const TA* __restrict__ val, const TX* __restrict__ x,
                                              const TACC* __restrict__ b, TACC* __restrict__ y)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        TACC acc[NC];
#pragma unroll
        for (int c = 0; c < NC; ++c) acc[c] = TACC(0);
        const int32_t e = rp[i + 1];
        for (int32_t j = rp[i]; j < e; ++j) {
            const TACC    a  = (TACC)val[j];
            const int64_t cj = (int64_t)col[j] * NC;
#pragma unroll
            for (int c = 0; c < NC; ++c) acc[c] += a * (TACC)x[cj + c];
        }
#pragma unroll
        for (int c = 0; c < NC; ++c) y[i * NC + c] = RESID ? b[i * NC + c] - acc[c] : acc[c];
    }
}

// ---------------------------------------------------------------------
// Persistent CG / Jacobi-PCG (CGSolver / PCGSolver, cg_solver.h:37-125,
// pcg_solver.h:34-144).  One cooperative launch runs the whole solve; the
// grid synchronises twice per iteration through a bounded barrier and every
// block reduces the per-block partial dot products itself in a fixed order,
// so all blocks take the same (deterministic) alpha, beta and stop decision
// without a host round trip.  The search-direction update p = z + beta p is
// fused into the next SpMM (double-buffered p).
// ---------------------------------------------------------------------

// bar[0] arrivals, bar[1] generation, bar[2] abort
__device__ __forceinline__ bool grid_sync(unsigned* bar, unsigned nblocks, int* err, int* s_ok)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* vgen = bar + 1;
        volatile unsigned* vab  = bar + 2;
        const unsigned     g    = *vgen;
        int                ok   = 1;
        __threadfence();
        const unsigned a = atomicAdd(bar, 1u);
        if (a == nblocks - 1) {
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            uint32_t i = 0;
            while (*vgen == g) {
                if (*vab) {
                    ok = 0;
                    break;
                }
                if (++i > kWaitLimit) {
                    atomicOr(err, DEVERR_GRID_TIMEOUT);
                    atomicExch(bar + 2, 1u);
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        *s_ok = ok;
    }
    __syncthreads();
    return *s_ok != 0;
}

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

// sum of the grid's partials in a fixed order (identical in every block)
template <int BT>
__device__ __forceinline__ double grid_partials_sum(const double* part, int G, double* s_red)
{
    double v = 0;
    if (threadIdx.x < 32) {
        for (int i = threadIdx.x; i < G; i += 32) v += *((volatile const double*)(part + i));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (threadIdx.x == 0) s_red[BT / 32 + 1] = v;
    }
    __syncthreads();
    double r = s_red[BT / 32 + 1];
    __syncthreads();
    return r;
}

template <typename T>
struct CGArgs
{
    int64_t        n;
    const int32_t* rp;
    const int32_t* col;
    const T*       val;
    const T*       B;
    T*             X;
    T*             R;
    T*             P0;
    T*             P1;
    T*             S;
    T*             Z;
    T*             dinv;
    double*        part;   // 2 * gridDim
    unsigned*      bar;    // 4
    double*        dstat;  // start, final
    int*           istat;  // iters, converged
    int            max_iter;
    double         abs_tol, rel_tol;
    int*           err;
};

constexpr int kCGT = 256;

template <typename T, int NC, bool PC>
__global__ void __launch_bounds__(kCGT) k_cg(CGArgs<T> a)
{
    __shared__ double s_red[kCGT / 32 + 2];
    __shared__ int    s_ok;
    const unsigned G     = gridDim.x;
    const int64_t  chunk = (a.n + G - 1) / G;
    const int64_t  r0    = blockIdx.x * chunk;
    const int64_t  r1    = min(a.n, r0 + chunk);
    T* const       src   = PC ? a.Z : a.R;  // vector the direction is built from

    // ---- pre_solve: S = A X, R = B - S, Z = D^-1 R, delta = R.Z (or R.R)
    double part = 0;
    for (int64_t i = r0 + threadIdx.x; i < r1; i += kCGT) {
        const int32_t b = __ldg(a.rp + i), e = __ldg(a.rp + i + 1);
        T             acc[NC];
#pragma unroll
        for (int c = 0; c < NC; ++c) acc[c] = T(0);
        T diag = T(0);
        for (int32_t j = b; j < e; ++j) {
            const int32_t cj = __ldg(a.col + j);
            const T       v  = __ldg(a.val + j);
            if (cj == i) diag = v;
#pragma unroll
            for (int c = 0; c < NC; ++c) acc[c] += v * a.X[(int64_t)cj * NC + c];
        }
        const T di = T(1) / (diag + (sizeof(T) == 4 ? (T)FLT_EPSILON : (T)DBL_EPSILON));
        if (PC) a.dinv[i] = di;
        T tp = T(0);
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            const T r = a.B[i * NC + c] - acc[c];
            a.R[i * NC + c] = r;
            if (PC) {
                const T z       = di * r;
                a.Z[i * NC + c] = z;
                tp += r * z;
            } else {
                tp += r * r;
            }
        }
        part += (double)tp;
    }
    part = block_sum<kCGT>(part, s_red);
    if (threadIdx.x == 0) a.part[blockIdx.x] = part;
    if (!grid_sync(a.bar, G, a.err, &s_ok)) return;
    const double delta0 = grid_partials_sum<kCGT>(a.part, G, s_red);
    double       delta  = delta0;
    auto conv = [&](double d) { return d < a.abs_tol || d / delta0 < a.rel_tol; };
    if (conv(delta0)) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            a.dstat[0] = delta0;
            a.dstat[1] = delta0;
            a.istat[0] = 0;
            a.istat[1] = 1;
        }
        return;
    }
    double beta = 0;
    int    it   = 0;
    bool   done = false;
    while (it < a.max_iter) {
        T* const Pold = (it & 1) ? a.P1 : a.P0;
        T* const Pnew = (it & 1) ? a.P0 : a.P1;
        const T  bt   = (T)beta;
        // ---- phase A: p = src + beta p_old (fused), S = A p, part = S.p
        part = 0;
        for (int64_t i = r0 + threadIdx.x; i < r1; i += kCGT) {
            const int32_t b = __ldg(a.rp + i), e = __ldg(a.rp + i + 1);
            T             acc[NC];
#pragma unroll
            for (int c = 0; c < NC; ++c) acc[c] = T(0);
            for (int32_t j = b; j < e; ++j) {
                const int64_t cj = (int64_t)__ldg(a.col + j) * NC;
                const T       v  = __ldg(a.val + j);
#pragma unroll
                for (int c = 0; c < NC; ++c) {
                    const T pj = it == 0 ? src[cj + c] : src[cj + c] + bt * Pold[cj + c];
                    acc[c] += v * pj;
                }
            }
            T tp = T(0);
#pragma unroll
            for (int c = 0; c < NC; ++c) {
                const T pi = it == 0 ? src[i * NC + c] : src[i * NC + c] + bt * Pold[i * NC + c];
                Pnew[i * NC + c] = pi;
                a.S[i * NC + c]  = acc[c];
                tp += acc[c] * pi;
            }
            part += (double)tp;
        }
        part = block_sum<kCGT>(part, s_red);
        if (threadIdx.x == 0) a.part[G + blockIdx.x] = part;
        if (!grid_sync(a.bar, G, a.err, &s_ok)) return;
        const double alpha = delta / grid_partials_sum<kCGT>(a.part + G, G, s_red);
        const T      al    = (T)alpha;
        // ---- phase B: X += alpha p, R -= alpha S, Z = D^-1 R, delta' = R.Z
        part = 0;
        for (int64_t i = r0 + threadIdx.x; i < r1; i += kCGT) {
            const T di = PC ? a.dinv[i] : T(1);
            T       tp = T(0);
#pragma unroll
            for (int c = 0; c < NC; ++c) {
                a.X[i * NC + c] += al * Pnew[i * NC + c];
                const T r = a.R[i * NC + c] - al * a.S[i * NC + c];
                a.R[i * NC + c] = r;
                if (PC) {
                    const T z       = di * r;
                    a.Z[i * NC + c] = z;
                    tp += r * z;
                } else {
                    tp += r * r;
                }
            }
            part += (double)tp;
        }
        part = block_sum<kCGT>(part, s_red);
        if (threadIdx.x == 0) a.part[blockIdx.x] = part;
        if (!grid_sync(a.bar, G, a.err, &s_ok)) return;
        const double dn = grid_partials_sum<kCGT>(a.part, G, s_red);
        if (conv(dn)) {
            delta = dn;
            done  = true;
            break;
        }
        beta  = dn / delta;
        delta = dn;
        ++it;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.dstat[0] = delta0;
        a.dstat[1] = delta;
        a.istat[0] = it;
        a.istat[1] = done ? 1 : 0;
    }
}

// ---------------------------------------------------------------------
// host side: CG launch
// ---------------------------------------------------------------------

static int num_sms()
{
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    return sms;
}

template <typename T, int NC, bool PC>
static int cg_grid(int64_t n)
{
    static int per_sm = -1;
    if (per_sm < 0) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cg<T, NC, PC>, kCGT, 0) !=
            cudaSuccess)
            per_sm = 1;
        per_sm = std::max(1, std::min(per_sm, 4));
    }
    int64_t g = (int64_t)num_sms() * per_sm;
    g         = std::min<int64_t>(g, std::max<int64_t>(1, (n + 31) / 32));
    return (int)g;
}

static size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

template <typename T>
static size_t cg_scratch_bytes(int64_t n, int nc, int G)
{
    return 5 * align256(sizeof(T) * n * nc) + align256(sizeof(T) * n) +
           align256(sizeof(double) * 2 * G) + 3 * 256;
}

template <typename T, int NC, bool PC>
static rxg_status cg_launch(int64_t n, const int32_t* rp, const int32_t* col, const T* val,
                            const T* B, T* X, const rxg_solver_opts& o, rxg_solver_stats* st,
                            uint8_t* scratch, cudaStream_t s)
{
    const int  G = cg_grid<T, NC, PC>(n);
    CGArgs<T>  a;
    uint8_t*   q  = scratch;
    const size_t vb = align256(sizeof(T) * n * NC);
    a.n   = n;
    a.rp  = rp;
    a.col = col;
    a.val = val;
    a.B   = B;
    a.X   = X;
    a.R   = (T*)q, q += vb;
    a.P0  = (T*)q, q += vb;
    a.P1  = (T*)q, q += vb;
    a.S   = (T*)q, q += vb;
    a.Z   = (T*)q, q += vb;
    a.dinv = (T*)q, q += align256(sizeof(T) * n);
    a.part  = (double*)q, q += align256(sizeof(double) * 2 * G);
    a.bar   = (unsigned*)q, q += 256;
    a.dstat = (double*)q, q += 256;
    a.istat = (int*)q, q += 256;
    a.max_iter = o.max_iter;
    a.abs_tol  = o.abs_tol;
    a.rel_tol  = o.rel_tol;
    a.err      = device_error_word();
    RXG_CUDA_TRY(cudaMemsetAsync(a.bar, 0, 256, s));
    void* args[] = {&a};
    RXG_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)k_cg<T, NC, PC>, dim3(G), dim3(kCGT),
                                             args, 0, s));
    if (st) {
        double ds[2];
        int    is[2];
        RXG_CUDA_TRY(cudaMemcpyAsync(ds, a.dstat, sizeof(ds), cudaMemcpyDeviceToHost, s));
        RXG_CUDA_TRY(cudaMemcpyAsync(is, a.istat, sizeof(is), cudaMemcpyDeviceToHost, s));
        RXG_CUDA_TRY(cudaStreamSynchronize(s));
        rxg_status e = check_device_error(s);
        if (e) return e;
        st->start_res = ds[0];
        st->final_res = ds[1];
        st->iters     = is[0];
        st->converged = is[1];
    }
    return RXG_OK;
}

template <typename T>
static rxg_status cg_dispatch(int nc, int64_t n, const int32_t* rp, const int32_t* col,
                              const T* val, const T* B, T* X, const rxg_solver_opts& o,
                              rxg_solver_stats* st, uint8_t* scratch, cudaStream_t s)
{
#define RXG_CG_CASE(NCV)                                                                         \
    case NCV:                                                                                    \
        return o.precond ? cg_launch<T, NCV, true>(n, rp, col, val, B, X, o, st, scratch, s)    \
                         : cg_launch<T, NCV, false>(n, rp, col, val, B, X, o, st, scratch, s);
    switch (nc) {
        RXG_CG_CASE(1)
        RXG_CG_CASE(2)
        RXG_CG_CASE(3)
        RXG_CG_CASE(4)
    }
#undef RXG_CG_CASE
    set_error("cg: nc must be 1..4");
    return RXG_ERR_INVALID;
}

template <typename T>
static int cg_grid_any(int nc, bool pc, int64_t n)
{
    switch (nc * 2 + (pc ? 1 : 0)) {
        case 2: return cg_grid<T, 1, false>(n);
        case 3: return cg_grid<T, 1, true>(n);
        case 4: return cg_grid<T, 2, false>(n);
        case 5: return cg_grid<T, 2, true>(n);
        case 6: return cg_grid<T, 3, false>(n);
        case 7: return cg_grid<T, 3, true>(n);
        case 8: return cg_grid<T, 4, false>(n);
        default: return cg_grid<T, 4, true>(n);
    }
}

template <typename TA, typename TX, typename TACC>
static rxg_status spmm_launch(int nc, int64_t n, const int32_t* rp, const int32_t* col,
                              const TA* val, const TX* x, const TACC* b, TACC* y, cudaStream_t s)
{
    const int g = grid_for(n);
#define RXG_SPMM_CASE(NCV)                                                                     \
    case NCV:                                                                                  \
        if (b)                                                                                 \
            k_spmm<TA, TX, TACC, NCV, true><<<g, 256, 0, s>>>(n, rp, col, val, x, b, y);       \
        else                                                                                   \
            k_spmm<TA, TX, TACC, NCV, false><<<g, 256, 0, s>>>(n, rp, col, val, x, b, y);      \
        break;
    switch (nc) {
        RXG_SPMM_CASE(1)
        RXG_SPMM_CASE(2)
        RXG_SPMM_CASE(3)
        RXG_SPMM_CASE(4)
        default: set_error("spmm: nc must be 1..4"); return RXG_ERR_INVALID;
    }
#undef RXG_SPMM_CASE
    RXG_CUDA_TRY(cudaGetLastError());
    return RXG_OK;
}

// ---------------------------------------------------------------------
// host side: oriented ring and pattern (built once per mesh)
// ---------------------------------------------------------------------

static size_t oriented_smem_bytes(const Mesh* m)
{
    size_t w = 0;
    for (const PatchHdr& h : m->hdr) {
        const size_t few = pad4i((3 * h.nFl + 1) / 2);
        w = std::max(w, (size_t)pad4i(h.nEl) + few + pad4i(h.nVl - h.nVo) + 2 * pad4i(h.nVo + 1) +
                            3 * (size_t)h.nFl);
    }
    return w * 4;
}

static rxg_status launch_oriented(const Mesh* m, int32_t* off, int32_t* val, int8_t* bnd,
                                  cudaStream_t s)
{
    const size_t smem = oriented_smem_bytes(m);
    if (smem > 227 * 1024) {
        set_error("oriented VV: a patch needs %zu bytes of shared memory", smem);
        return RXG_ERR_PATCH_LIMIT;
    }
    if (smem > 48 * 1024)
        RXG_CUDA_TRY(cudaFuncSetAttribute(k_oriented_vv, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem));
    k_oriented_vv<<<m->num_patches, kQT2, smem, s>>>(m->d.hdr, m->d.arena, off, val, bnd,
                                                      device_error_word());
    RXG_CUDA_TRY(cudaGetLastError());
    return RXG_OK;
}

static rxg_status ensure_pattern(const Mesh* m, cudaStream_t s, Lazy** out)
{
    Lazy* z = lazy_of(m);
    std::lock_guard<std::mutex> g(z->mu);
    *out = z;
    if (z->ring_ready) return RXG_OK;
    if (!m->edge_manifold) {
        set_error("the MCF system needs an edge-manifold mesh (apps/MCF/mcf.cu:103-106)");
        return RXG_ERR_NONMANIFOLD;
    }
    const int64_t nv = m->nv, ne = m->ne;
    z->nnz           = nv + 2 * ne;
    RXG_CUDA_TRY(cudaMalloc(&z->ring_off, 4 * (nv + 1)));
    RXG_CUDA_TRY(cudaMalloc(&z->ring, 4 * std::max<int64_t>(1, 2 * ne)));
    RXG_CUDA_TRY(cudaMalloc(&z->bnd, std::max<int64_t>(16, nv)));
    RXG_CUDA_TRY(cudaMalloc(&z->row_ptr, 4 * (nv + 1)));
    RXG_CUDA_TRY(cudaMalloc(&z->col, 4 * z->nnz));
    rxg_status st = launch_oriented(m, z->ring_off, z->ring, z->bnd, s);
    if (st) return st;
    k_pattern<<<grid_for(nv + 1), 256, 0, s>>>(nv, z->ring_off, z->ring, z->row_ptr, z->col);
    RXG_CUDA_TRY(cudaGetLastError());
    st = check_device_error(s);
    if (st) return st;
    z->ring_ready = true;
    return RXG_OK;
}

// ---------------------------------------------------------------------
// mixed-precision helpers
// ---------------------------------------------------------------------

// x += d ; returns nothing
__global__ void k_add_correction(int64_t m, double* __restrict__ x, const float* __restrict__ d)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m;
         i += (int64_t)gridDim.x * blockDim.x)
        x[i] += (double)d[i];
}

// r = B - A x in FP64 with FP32 matrix entries; r32 = (float) r; per-block |r|^2
__global__ void __launch_bounds__(256) k_resid_mixed(int64_t n, const int32_t* __restrict__ rp,
                                                     const int32_t* __restrict__ col,
                                                     const float* __restrict__ val,
                                                     const double* __restrict__ x,
                                                     const double* __restrict__ B,
                                                     float* __restrict__ r32,
                                                     double* __restrict__ part)
{
    __shared__ double s_red[256 / 32 + 2];
    double            acc2 = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        double a0 = 0, a1 = 0, a2 = 0;
        for (int32_t j = rp[i]; j < rp[i + 1]; ++j) {
            const double  v = (double)val[j];
            const int64_t c = 3 * (int64_t)col[j];
            a0 += v * x[c];
            a1 += v * x[c + 1];
            a2 += v * x[c + 2];
        }
        const double e0 = B[3 * i] - a0, e1 = B[3 * i + 1] - a1, e2 = B[3 * i + 2] - a2;
        r32[3 * i]     = (float)e0;
        r32[3 * i + 1] = (float)e1;
        r32[3 * i + 2] = (float)e2;
        acc2 += e0 * e0 + e1 * e1 + e2 * e2;
    }
    acc2 = block_sum<256>(acc2, s_red);
    if (threadIdx.x == 0) part[blockIdx.x] = acc2;
}

static rxg_status reduce_partials(const double* d_part, int G, cudaStream_t s, double* out)
{
    std::vector<double> h(G);
    RXG_CUDA_TRY(cudaMemcpyAsync(h.data(), d_part, sizeof(double) * G, cudaMemcpyDeviceToHost, s));
    RXG_CUDA_TRY(cudaStreamSynchronize(s));
    double t = 0;
    for (double v : h) t += v;
    *out = t;
    return RXG_OK;
}

}  // namespace rxg

using namespace rxg;

static cudaStream_t S_(void* s) { return (cudaStream_t)s; }

extern "C" {

rxg_status rxg_permute(const rxg_mesh* h, int32_t elem, int32_t to_linear, int32_t dtype,
                       int32_t ncomp, const void* src, void* dst, void* stream)
{
    if (!h || !src || !dst || elem < 0 || elem > 2 || ncomp <= 0 || (dtype != RXG_F32 && dtype != RXG_F64)) {
        set_error("rxg_permute: bad argument");
        return RXG_ERR_INVALID;
    }
    if (!is_device_ptr(src) || !is_device_ptr(dst)) {
        set_error("rxg_permute: src and dst must be device arrays");
        return RXG_ERR_INVALID;
    }
    const Mesh&    M   = h->m;
    const int64_t  n   = elem == 0 ? M.nv : (elem == 1 ? M.ne : M.nf);
    const int32_t* l2i = elem == 0 ? M.d.v_l2i : (elem == 1 ? M.d.e_l2i : M.d.f_l2i);
    const int      g   = grid_for(n * ncomp);
    if (dtype == RXG_F32)
        k_permute<uint32_t><<<g, 256, 0, S_(stream)>>>(n, ncomp, l2i, to_linear, (const uint32_t*)src,
                                                        (uint32_t*)dst);
    else
        k_permute<uint64_t><<<g, 256, 0, S_(stream)>>>(n, ncomp, l2i, to_linear, (const uint64_t*)src,
                                                        (uint64_t*)dst);
    RXG_CUDA_TRY(cudaGetLastError());
    return RXG_OK;
}

rxg_status rxg_query_oriented_vv(const rxg_mesh* h, int32_t* offsets, int32_t* values,
                                 int8_t* boundary, void* stream)
{
    if (!h || !offsets || !values) {
        set_error("rxg_query_oriented_vv: offsets and values must not be NULL");
        return RXG_ERR_INVALID;
    }
    if (!is_device_ptr(offsets) || !is_device_ptr(values) || (boundary && !is_device_ptr(boundary))) {
        set_error("rxg_query_oriented_vv: outputs must be device arrays");
        return RXG_ERR_INVALID;
    }
    if (!h->m.edge_manifold) {
        set_error("rxg_query_oriented_vv: needs an edge-manifold mesh");
        return RXG_ERR_NONMANIFOLD;
    }
    int8_t* b = boundary;
    if (!b) RXG_CUDA_TRY(cudaMallocAsync((void**)&b, std::max<int64_t>(16, h->m.nv), S_(stream)));
    rxg_status st = launch_oriented(&h->m, offsets, values, b, S_(stream));
    if (!boundary) cudaFreeAsync(b, S_(stream));
    if (st) return st;
    return check_device_error(S_(stream));
}

rxg_status rxg_mcf_pattern_size(const rxg_mesh* h, int64_t* n, int64_t* nnz)
{
    if (!h || !n || !nnz) {
        set_error("rxg_mcf_pattern_size: NULL argument");
        return RXG_ERR_INVALID;
    }
    *n   = h->m.nv;
    *nnz = h->m.nv + 2 * h->m.ne;
    return RXG_OK;
}

rxg_status rxg_mcf_assemble(const rxg_mesh* h, double dt, const double* xyz, rxg_csr* A, void* B,
                            void* stream)
{
    if (!h || !xyz || !A || !A->row_ptr || !A->col || !A->val ||
        (A->dtype != RXG_F32 && A->dtype != RXG_F64)) {
        set_error("rxg_mcf_assemble: bad argument");
        return RXG_ERR_INVALID;
    }
    if (!is_device_ptr(xyz) || !is_device_ptr(A->val) || (B && !is_device_ptr(B))) {
        set_error("rxg_mcf_assemble: xyz, A and B must be device arrays");
        return RXG_ERR_INVALID;
    }
    Lazy*        z;
    cudaStream_t s  = S_(stream);
    rxg_status   st = ensure_pattern(&h->m, s, &z);
    if (st) return st;
    const int64_t nv = h->m.nv;
    A->n   = nv;
    A->nnz = z->nnz;
    RXG_CUDA_TRY(cudaMemcpyAsync(A->row_ptr, z->row_ptr, 4 * (nv + 1), cudaMemcpyDeviceToDevice, s));
    RXG_CUDA_TRY(cudaMemcpyAsync(A->col, z->col, 4 * z->nnz, cudaMemcpyDeviceToDevice, s));
    const int g = grid_for(nv);
    if (A->dtype == RXG_F64)
        k_mcf_assemble<double, Geo<double>, double><<<g, 256, 0, s>>>(
            nv, z->row_ptr, z->col, z->bnd, xyz, dt, (double*)A->val, (double*)B);
    else
        k_mcf_assemble<float, GeoMixed, float><<<g, 256, 0, s>>>(
            nv, z->row_ptr, z->col, z->bnd, xyz, (float)dt, (float*)A->val, (float*)B);
    RXG_CUDA_TRY(cudaGetLastError());
    return RXG_OK;
}

rxg_status rxg_spmm(const rxg_csr* A, int32_t nc, const void* X, void* Y, void* stream)
{
    if (!A || !X || !Y || nc < 1 || nc > 4) {
        set_error("rxg_spmm: bad argument");
        return RXG_ERR_INVALID;
    }
    if (A->dtype == RXG_F64)
        return spmm_launch<double, double, double>(nc, A->n, A->row_ptr, A->col, (const double*)A->val,
                                                   (const double*)X, (const double*)nullptr,
                                                   (double*)Y, S_(stream));
    return spmm_launch<float, float, float>(nc, A->n, A->row_ptr, A->col, (const float*)A->val,
                                            (const float*)X, (const float*)nullptr, (float*)Y,
                                            S_(stream));
}

rxg_status rxg_cg_solve(const rxg_csr* A, int32_t nc, const void* B, void* X,
                        const rxg_solver_opts* opts, rxg_solver_stats* stats, void* stream)
{
    if (!A || !B || !X || !opts || nc < 1 || nc > 4 || A->n <= 0 || opts->max_iter < 0) {
        set_error("rxg_cg_solve: bad argument");
        return RXG_ERR_INVALID;
    }
    if (!is_device_ptr(B) || !is_device_ptr(X) || !is_device_ptr(A->val)) {
        set_error("rxg_cg_solve: A, B and X must be device arrays");
        return RXG_ERR_INVALID;
    }
    cudaStream_t s  = S_(stream);
    const bool   pc = opts->precond != 0;
    rxg_solver_stats local;
    rxg_status       st;
    uint8_t*         scratch = nullptr;
    if (A->dtype == RXG_F64) {
        const size_t bytes = cg_scratch_bytes<double>(A->n, nc, cg_grid_any<double>(nc, pc, A->n));
        RXG_CUDA_TRY(cudaMallocAsync((void**)&scratch, bytes, s));
        st = cg_dispatch<double>(nc, A->n, A->row_ptr, A->col, (const double*)A->val,
                                 (const double*)B, (double*)X, *opts, &local, scratch, s);
    } else {
        const size_t bytes = cg_scratch_bytes<float>(A->n, nc, cg_grid_any<float>(nc, pc, A->n));
        RXG_CUDA_TRY(cudaMallocAsync((void**)&scratch, bytes, s));
        st = cg_dispatch<float>(nc, A->n, A->row_ptr, A->col, (const float*)A->val,
                                (const float*)B, (float*)X, *opts, &local, scratch, s);
    }
    cudaFreeAsync(scratch, s);
    if (st) return st;
    if (stats) *stats = local;
    return local.converged ? RXG_OK : RXG_ERR_NOT_CONVERGED;
}

static rxg_status mcf_buffers(Lazy* z, size_t bytes, cudaStream_t s)
{
    if (z->buf_size >= bytes) return RXG_OK;
    RXG_CUDA_TRY(cudaStreamSynchronize(s));
    cudaFree(z->buf);
    z->buf      = nullptr;
    z->buf_size = 0;
    RXG_CUDA_TRY(cudaMalloc(&z->buf, bytes));
    z->buf_size = bytes;
    return RXG_OK;
}

rxg_status rxg_mcf_step(const rxg_mesh* h, double dt, int32_t nsteps, int32_t precision, double tol,
                        int32_t max_iter, double* xyz, rxg_solver_stats* stats, void* stream)
{
    if (!h || !xyz || nsteps < 0 || max_iter <= 0 || !(tol > 0) ||
        (precision != RXG_F32 && precision != RXG_F64)) {
        set_error("rxg_mcf_step: bad argument");
        return RXG_ERR_INVALID;
    }
    cudaStream_t s = S_(stream);
    Lazy*        z;
    rxg_status   st = ensure_pattern(&h->m, s, &z);
    if (st) return st;
    const int64_t n = h->m.nv, nnz = z->nnz;
    const int     Gd = cg_grid_any<double>(3, true, n), Gf = cg_grid_any<float>(3, true, n);
    const int     Gr = grid_for(n);
    const size_t  plain = align256(8 * nnz) + align256(24 * n) + cg_scratch_bytes<double>(n, 3, Gd);
    const size_t  mixed = align256(4 * nnz) + align256(24 * n) + 2 * align256(12 * n) +
                         align256(8 * Gr) + cg_scratch_bytes<float>(n, 3, Gf);
    {
        std::lock_guard<std::mutex> g(z->mu);
        if ((st = mcf_buffers(z, std::max(plain, mixed), s))) return st;
    }
    // positions: device, or staged from host
    double* X         = xyz;
    bool    staged    = false;
    if (!is_device_ptr(xyz)) {
        RXG_CUDA_TRY(cudaMallocAsync((void**)&X, 24 * n, s));
        RXG_CUDA_TRY(cudaMemcpyAsync(X, xyz, 24 * n, cudaMemcpyHostToDevice, s));
        staged = true;
    }
    uint8_t*         q    = (uint8_t*)z->buf;
    rxg_solver_stats last = {0, 1, 0.0, 0.0};
    const int        ga   = grid_for(n);
    for (int step = 0; step < nsteps && st == RXG_OK; ++step) {
        if (precision == RXG_F64) {
            double*  val = (double*)q;
            double*  B   = (double*)(q + align256(8 * nnz));
            uint8_t* scr = q + align256(8 * nnz) + align256(24 * n);
            k_mcf_assemble<double, Geo<double>, double><<<ga, 256, 0, s>>>(
                n, z->row_ptr, z->col, z->bnd, X, dt, val, B);
            RXG_CUDA_TRY(cudaGetLastError());
            rxg_solver_opts o = {max_iter, 0.0, tol * tol, 1};
            st = cg_dispatch<double>(3, n, z->row_ptr, z->col, val, B, X, o, &last, scr, s);
        } else {
            float*   val  = (float*)q;
            uint8_t* p    = q + align256(4 * nnz);
            double*  B    = (double*)p;
            p += align256(24 * n);
            float* r32 = (float*)p;
            p += align256(12 * n);
            float* d32 = (float*)p;
            p += align256(12 * n);
            double* part = (double*)p;
            p += align256(8 * Gr);
            uint8_t* scr = p;
            k_mcf_assemble<float, GeoMixed, double><<<ga, 256, 0, s>>>(n, z->row_ptr, z->col, z->bnd,
                                                                       X, (float)dt, val, B);
            RXG_CUDA_TRY(cudaGetLastError());
            k_resid_mixed<<<Gr, 256, 0, s>>>(n, z->row_ptr, z->col, val, X, B, r32, part);
            double rr0;
            if ((st = reduce_partials(part, Gr, s, &rr0))) break;
            double rr = rr0;
            int    total_it = 0;
            bool   conv = rr0 == 0.0;
            for (int sweep = 0; sweep < 16 && !conv && total_it < max_iter; ++sweep) {
                // solve only as far as this sweep needs, but not below FP32's reach
                const double need  = tol * std::sqrt(rr0 / rr);
                const double inner = std::max(1e-4, 0.3 * need);
                RXG_CUDA_TRY(cudaMemsetAsync(d32, 0, 12 * n, s));
                rxg_solver_opts  o = {max_iter - total_it, 0.0, inner * inner, 1};
                rxg_solver_stats si;
                st = cg_dispatch<float>(3, n, z->row_ptr, z->col, val, r32, d32, o, &si, scr, s);
                if (st) break;
                total_it += si.iters + 1;
                k_add_correction<<<grid_for(3 * n), 256, 0, s>>>(3 * n, X, d32);
                k_resid_mixed<<<Gr, 256, 0, s>>>(n, z->row_ptr, z->col, val, X, B, r32, part);
                if ((st = reduce_partials(part, Gr, s, &rr))) break;
                conv = rr < tol * tol * rr0;
            }
            last.iters     = total_it;
            last.converged = conv ? 1 : 0;
            last.start_res = rr0;
            last.final_res = rr;
        }
    }
    if (st == RXG_OK && staged) {
        RXG_CUDA_TRY(cudaMemcpyAsync(xyz, X, 24 * n, cudaMemcpyDeviceToHost, s));
        RXG_CUDA_TRY(cudaStreamSynchronize(s));
    }
    if (staged) cudaFreeAsync(X, s);
    if (st) return st;
    if (stats) *stats = last;
    return last.converged ? RXG_OK : RXG_ERR_NOT_CONVERGED;
}

}  // extern "C"

// ---------------------------------------------------------------------
// CG without device allocation.
//
// Some callers may not call cudaMalloc (or any allocating routine) at solve
// time: a host application that owns all device memory through its own pool
// and budget, a plugin that must not allocate behind its host's back, or code
// that allocates only at start-up.  rxg_cg_solve_noalloc runs the same
// persistent CG/PCG kernel as rxg_cg_solve, but its work vectors, partial
// sums, grid-barrier words and statistics live in the file-scope array below
// instead of a cudaMallocAsync'd buffer.  The array is part of the library's
// device image: every GPU that loads this code holds it until the process
// exits, so its size is fixed and modest (just over 16 MiB).
// ---------------------------------------------------------------------

namespace rxg {

constexpr int64_t kNoAllocMaxRows = 131072;  // rows of A
constexpr int     kNoAllocMaxCols = 3;       // right-hand sides
constexpr int     kNoAllocMaxGrid = 1024;    // cooperative CTAs (partials)
constexpr size_t  kNoAllocBytes =
    5 * ((sizeof(double) * kNoAllocMaxRows * kNoAllocMaxCols + 255) & ~size_t(255)) +
    ((sizeof(double) * kNoAllocMaxRows + 255) & ~size_t(255)) +
    ((sizeof(double) * 2 * kNoAllocMaxGrid + 255) & ~size_t(255)) + 3 * 256;

static __device__ __align__(256) unsigned char g_cg_noalloc_scratch[kNoAllocBytes];

// Device address of the scratch array for the current device.  Host code
// cannot use the symbol itself (it names a host-side stand-in), so the
// address is taken once per device with cudaGetSymbolAddress and cached.
static rxg_status noalloc_scratch(uint8_t** out)
{
    static std::mutex mu;
    static uint8_t*   addr[64] = {nullptr};
    int               dev      = 0;
    RXG_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) {
        set_error("rxg_cg_solve_noalloc: device ordinal %d out of range", dev);
        return RXG_ERR_UNSUPPORTED;
    }
    std::lock_guard<std::mutex> g(mu);
    if (!addr[dev]) {
        void*       p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_cg_noalloc_scratch);
        if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress(g_cg_noalloc_scratch)");
        addr[dev] = static_cast<uint8_t*>(p);
    }
    *out = addr[dev];
    return RXG_OK;
}

}  // namespace rxg

extern "C" rxg_status rxg_cg_solve_noalloc(const rxg_csr* A, int32_t nc, const void* B, void* X,
                                           const rxg_solver_opts* opts, rxg_solver_stats* stats,
                                           void* stream)
{
    using namespace rxg;
    if (!A || !B || !X || !opts || nc < 1 || A->n <= 0 || opts->max_iter < 0 ||
        (A->dtype != RXG_F32 && A->dtype != RXG_F64)) {
        set_error("rxg_cg_solve_noalloc: bad argument");
        return RXG_ERR_INVALID;
    }
    if (A->n > kNoAllocMaxRows || nc > kNoAllocMaxCols) {
        set_error("rxg_cg_solve_noalloc: %lld rows x %d columns exceeds the fixed scratch "
                  "(at most %lld rows and %d columns); use rxg_cg_solve",
                  (long long)A->n, nc, (long long)kNoAllocMaxRows, kNoAllocMaxCols);
        return RXG_ERR_INVALID;
    }
    if (!is_device_ptr(B) || !is_device_ptr(X) || !is_device_ptr(A->val)) {
        set_error("rxg_cg_solve_noalloc: A, B and X must be device arrays");
        return RXG_ERR_INVALID;
    }
    uint8_t*   scratch = nullptr;
    rxg_status st      = noalloc_scratch(&scratch);
    if (st) return st;
    const bool   pc    = opts->precond != 0;
    const int    G     = A->dtype == RXG_F64 ? cg_grid_any<double>(nc, pc, A->n)
                                             : cg_grid_any<float>(nc, pc, A->n);
    const size_t bytes = A->dtype == RXG_F64 ? cg_scratch_bytes<double>(A->n, nc, G)
                                             : cg_scratch_bytes<float>(A->n, nc, G);
    if (G > kNoAllocMaxGrid || bytes > kNoAllocBytes) {
        set_error("rxg_cg_solve_noalloc: needs %zu scratch bytes for %d CTAs, the fixed array "
                  "holds %zu",
                  bytes, G, kNoAllocBytes);
        return RXG_ERR_UNSUPPORTED;
    }
    // Every call reuses the same array and the kernel writes each work vector
    // before reading it; cg_launch zeroes the grid-barrier words on `stream`.
    cudaStream_t     s = (cudaStream_t)stream;
    rxg_solver_stats local;
    if (A->dtype == RXG_F64)
        st = cg_dispatch<double>(nc, A->n, A->row_ptr, A->col, (const double*)A->val,
                                 (const double*)B, (double*)X, *opts, &local, scratch, s);
    else
        st = cg_dispatch<float>(nc, A->n, A->row_ptr, A->col, (const float*)A->val,
                                (const float*)B, (float*)X, *opts, &local, scratch, s);
    if (st) return st;
    if (stats) *stats = local;
    return local.converged ? RXG_OK : RXG_ERR_NOT_CONVERGED;
}
