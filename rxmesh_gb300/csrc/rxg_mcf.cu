// Oriented one-ring, cotangent-Laplacian assembly, SpMM, persistent CG/PCG
// and the implicit mean-curvature-flow step (plain FP64 and mixed FP32 with
// FP64 iterative refinement).
#include <algorithm>
#include <type_traits>
#include <cfloat>
#include <cstdio>
#include <cstdlib>
#include <mutex>

#include "rxg_device.cuh"
#include "rxg_lazy.h"
#include "rxg_gridsum.cuh"
#include "rxg_mcf_common.cuh"

namespace rxg {

constexpr int kQT2 = 256;

size_t query_smem_bytes(const Mesh* m, int kind);

// ---------------------------------------------------------------------
// per-mesh lazily built structures
// ---------------------------------------------------------------------

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
    cudaFree(z->ring_face);
    cudaFree(z->ring_edge);
    cudaFree(z->row_ptr);
    cudaFree(z->col);
    cudaFree(z->buf);
    cudaFree(z->d_oc_bounds);
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

int grid_for_items(int64_t work) { return grid_for(work); }

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
                                                      int8_t* __restrict__ out_bnd,
                                                      int32_t* __restrict__ out_rface, int* err)
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
    uint32_t* s_rf   = s_rv + pad4i(nVr);
    int32_t*  s_fcnt = reinterpret_cast<int32_t*>(s_rf + pad4i(h.nFl - h.nFo));  // VF offsets
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
        const uint32_t b3 = pad16_bytes(h.nFl - h.nFo);
        mbar_arrive_expect_tx(&bar, b0 + b1 + b2 + b3);
        if (b0) bulk_g2s(s_ev, arena + h.ev_off, b0, &bar);
        if (b1) bulk_g2s(s_fe, arena + h.fe_off, b1, &bar);
        if (b2) bulk_g2s(s_rv, arena + h.rv_off, b2, &bar);
        if (b3) bulk_g2s(s_rf, arena + h.rf_off, b3, &bar);
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
    auto linf = [&](int f) -> int32_t { return f < h.nFo ? h.f_base + f : (int32_t)s_rf[f - h.nFo]; };
    for (int v = threadIdx.x; v < nVo; v += kQT2) {
        const int32_t beg = v == 0 ? 0 : s_fcnt[v - 1], end = s_fcnt[v], k = end - beg;
        const int32_t obeg = h.vv_base + s_ecnt[v], olen = s_ecnt[v + 1] - s_ecnt[v];
        int32_t*      o    = out_val + obeg;
        int32_t*      of   = out_rface ? out_rface + obeg : nullptr;  // face after ring[i]
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
            if (of && pos - 1 < olen) of[pos - 1] = linf(s_vf[beg + cur]);
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
                    if (pos < olen) {
                        o[pos] = lin(b);
                        if (of) of[pos] = -1;  // no face after the last boundary neighbour
                    }
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
        if ((bad || nvis != k || pos != olen) && err) atomicOr(err, DEVERR_NONMANIFOLD);
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
// MCF system (mcf_A_setup / mcf_B_setup, apps/MCF/mcf_kernels.cuh:302-426).
// One thread per vertex walks its oriented ring with a rolling window of
// three positions; the row is [diag, ring...] so no column search is done.
// Interior rows wrap (q of the first neighbour is the last one); boundary
// rows use only the fan's real triangles.
// ---------------------------------------------------------------------

// output policies of the assembly kernel: CSR values + n x 3 B, or packed
// entries + 4-wide B
template <typename T, typename TB>
struct CsrOut
{
    T*  val;
    TB* B;
    __device__ void entry(int32_t idx, int32_t, T v) const { val[idx] = v; }
    __device__ void diag_full(int64_t, TB) const {}
    __device__ void rhs(int64_t p, TB x, TB y, TB z) const
    {
        if (B) {
            B[3 * p + 0] = x;
            B[3 * p + 1] = y;
            B[3 * p + 2] = z;
        }
    }
};
template <typename T, typename TB>
struct PackedOut
{
    Ent<T>* ent;
    R4<TB>* B;
    TB*     diag;  // optional: the diagonal in TB before rounding to T
    __device__ void entry(int32_t idx, int32_t c, T v) const
    {
        Ent<T> e;
        e.col    = c;
        e.val    = v;
        ent[idx] = e;
    }
    __device__ void diag_full(int64_t p, TB d) const
    {
        if (diag) diag[p] = d;
    }
    __device__ void rhs(int64_t p, TB x, TB y, TB z) const
    {
        R4<TB> b;
        b.x  = x;
        b.y  = y;
        b.z  = z;
        b.w  = TB(0);
        B[p] = b;
    }
};

template <typename T, typename G, typename TB, typename Out>
__global__ void __launch_bounds__(256) k_mcf_assemble(int64_t nv, const int32_t* __restrict__ row_ptr,
                                                      const int32_t* __restrict__ col,
                                                      const int8_t* __restrict__ bnd,
                                                      const double* __restrict__ xyz, T dt, Out out)
{
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nv;
         p += (int64_t)gridDim.x * blockDim.x) {
        const int32_t rp   = row_ptr[p];
        const int32_t k    = row_ptr[p + 1] - rp - 1;
        const int32_t* rg  = col + rp + 1;
        const bool    wrap = bnd[p] == 0;
        const V3<double> P = ld3(xyz, (int32_t)p);
        // row sums accumulate in TB (FP64 on the MCF paths): the diagonal is
        // 2*area + sum of the T-rounded weights, so the Laplacian part keeps
        // exactly zero row sums when the FP64 residual uses it
        TB area = TB(0), sumw = TB(0);
        if (k > 0 && std::is_same<G, Geo<T>>::value) {
            // each fan triangle evaluated once (bit for bit the values of
            // the per-call loop below)
            area = fan_row<T, TB>(
                P, k, wrap, dt, [&](int32_t i) { return ld3(xyz, rg[i]); },
                [&](int32_t i, T w) {
                    sumw += (TB)w;
                    out.entry(rp + 1 + i, rg[i], -w);
                });
        } else if (k > 0) {
            // points made once per position (G::Pt: FP64 and FP32 copies)
            const typename G::Pt Pp = G::make(P);
            typename G::Pt       Q = G::make(ld3(xyz, rg[k - 1])), R = G::make(ld3(xyz, rg[0]));
            for (int32_t i = 0; i < k; ++i) {
                const typename G::Pt S = G::make(ld3(xyz, rg[i + 1 < k ? i + 1 : 0]));
                const bool has_q = wrap || i > 0, has_s = wrap || i < k - 1;
                T          w     = T(0);
                if (has_q) w += G::hc(Pp, R, Q);
                if (has_s) w += G::hc(Pp, R, S);
                w = (w >= T(0) ? w : T(0)) * dt;
                sumw += (TB)w;
                out.entry(rp + 1 + i, rg[i], -w);
                if (has_q) {
                    const T a = G::va(Pp, Q, R);
                    area += a > T(0) ? (TB)a : TB(0);
                }
                Q = R;
                R = S;
            }
        }
        // v_weight = 0.5 / area and its inverse as the reference forms them;
        // one more division, then products (GB300's FP64 divide is slow)
        const TB vw = TB(0.5) / area;
        const TB iv = TB(1) / vw;
        const TB dg = iv + sumw;
        out.entry(rp, (int32_t)p, (T)dg);
        out.diag_full(p, dg);
        out.rhs(p, (TB)P.x * iv, (TB)P.y * iv, (TB)P.z * iv);
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
        const int32_t e = __ldg(rp + i + 1);
        // seven entries per round: all column/value loads, then all gathers,
        // in flight together.  A vertex of valence 6 (the average of a
        // closed triangle mesh) has a row of seven entries, so most rows take
        // one round with no padded entry: no FP64 multiply-add is spent on
        // padding, which matters where the FP64 pipe is the bound.
        constexpr int RW = 7;
        for (int32_t j0 = __ldg(rp + i); j0 < e; j0 += RW) {
            int32_t cj[RW];
            TACC    v[RW];
#pragma unroll
            for (int u = 0; u < RW; ++u) {
                const bool ok = j0 + u < e;
                cj[u]         = ok ? __ldg(col + j0 + u) : (int32_t)i;
                v[u]          = ok ? (TACC)__ldg(val + j0 + u) : TACC(0);
            }
#pragma unroll
            for (int u = 0; u < RW; ++u)
#pragma unroll
                for (int c = 0; c < NC; ++c) acc[c] += v[u] * (TACC)__ldg(x + (int64_t)cj[u] * NC + c);
        }
#pragma unroll
        for (int c = 0; c < NC; ++c) y[i * NC + c] = RESID ? b[i * NC + c] - acc[c] : acc[c];
    }
}


// ---------------------------------------------------------------------
// Persistent CG / Jacobi-PCG (CGSolver / PCGSolver, cg_solver.h:37-125,
// pcg_solver.h:34-144).  One cooperative launch runs the whole solve; the
// grid synchronises twice per iteration, each time through a bounded barrier
// that also sums the per-block partial dot products in a fixed order, so all
// blocks take the same (deterministic) alpha, beta and stop decision without
// a host round trip.  The search-direction update p = z + beta p needs no
// barrier of its own: S = A p is carried as A z + beta S.
// ---------------------------------------------------------------------

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
    // matrix-free MCF operator (k_cg with MF = true): the mesh's
    // [diagonal, oriented ring] pattern, FP64 positions, the time step
    const int8_t*  mf_bnd;
    const double*  mf_xyz;
    const float*   mf_xyzf;  // the positions rounded to FP32 (T = float)
    double         mf_dt;
    int            mf_uniform;
};

// host side of the grid-sum state (rxg_gridsum.cuh): ticket counter and
// abort word to 0 before every launch
static cudaError_t reset_grid_sum(unsigned* bar, cudaStream_t s) { return cudaMemsetAsync(bar, 0, 16, s); }

// acc = sum_j A_ij x_j over row i, seven non-zeros per round so that all
// column/value loads and then all gathers of a round are in flight together
// (a valence-6 vertex's row of the MCF matrix has seven entries: one round,
// no padding).  Padding lanes read row i itself with weight zero.  diag (may
// be null) receives A_ii.
template <typename T, int NC>
__device__ __forceinline__ void row_spmv(const int32_t* __restrict__ rp, const int32_t* __restrict__ col,
                                         const T* __restrict__ val, int64_t i, const T* x, T* acc,
                                         T* diag)
{
    constexpr int RW = 7;
    const int32_t b  = __ldg(rp + i), e = __ldg(rp + i + 1);
    for (int32_t j0 = b; j0 < e; j0 += RW) {
        int32_t cj[RW];
        T       v[RW];
#pragma unroll
        for (int u = 0; u < RW; ++u) {
            const bool ok = j0 + u < e;
            cj[u]         = ok ? __ldg(col + j0 + u) : (int32_t)i;
            v[u]          = ok ? __ldg(val + j0 + u) : T(0);
        }
#pragma unroll
        for (int u = 0; u < RW; ++u) {
            if (diag && j0 + u < e && cj[u] == i) *diag = v[u];
#pragma unroll
            for (int c = 0; c < NC; ++c) acc[c] += v[u] * x[(int64_t)cj[u] * NC + c];
        }
    }
}

// row i of A times x by a group of L lanes (L = 2, 4, 8; the group is L
// aligned lanes of one warp): lane l takes entries b+l, b+l+L, ... (adjacent
// lanes read adjacent entries), then the group sums its partials.  diag
// (may be null) receives A_ii in every lane of the group.
template <typename T, int NC, int L>
__device__ __forceinline__ void row_spmv_group(const int32_t* __restrict__ rp,
                                               const int32_t* __restrict__ col,
                                               const T* __restrict__ val, int64_t i, const T* x,
                                               T* acc, T* diag, int lane)
{
    const int32_t b = __ldg(rp + i), e = __ldg(rp + i + 1);
    T             d = T(0);
    for (int32_t j = b + lane; j < e; j += L) {
        const int32_t c = __ldg(col + j);
        const T       v = __ldg(val + j);
        if (c == i) d = v;
#pragma unroll
        for (int k = 0; k < NC; ++k) acc[k] += v * x[(int64_t)c * NC + k];
    }
    const unsigned mask = ((1u << L) - 1u) << ((threadIdx.x & 31) & ~(L - 1));
#pragma unroll
    for (int o = L / 2; o > 0; o >>= 1) {
#pragma unroll
        for (int k = 0; k < NC; ++k) acc[k] += __shfl_xor_sync(mask, acc[k], o);
        d += __shfl_xor_sync(mask, d, o);
    }
    if (diag) *diag = d;
}

// Row p of the implicit-MCF operator A = 2M + dt L with its weights
// recomputed from the positions on every call (the matrix-free matvec of
// apps/MCF/mcf_kernels.cuh:101-193; cotangent mode as mcf_A_setup, uniform
// mode: weight 1 per neighbour and the valence as the vertex weight):
// acc += sum_j A_pj x_j over the row, diag (may be null) = A_pp.  rp/col
// is the [diagonal, oriented ring] pattern; the arithmetic and its order
// are k_mcf_assemble's, so a product equals the assembled matrix's.  PT:
// the positions' type, double, or float (the FP64 positions rounded once per
// call or solve, the same values the FP32 arithmetic would convert them to)
// when T is float, so that no conversion runs on the FP64 pipe per row.
template <typename T, typename G, int NC, typename PT>
__device__ __forceinline__ void mcf_row(const int32_t* __restrict__ row_ptr, const int32_t* __restrict__ col,
                                        const int8_t* __restrict__ bnd, const PT* __restrict__ xyz,
                                        T dt, bool uniform, int64_t p, const T* x, T* acc, T* diag)
{
    static_assert(std::is_same<G, Geo<T>>::value, "the matrix-free row uses the exact-type geometry");
    static_assert(std::is_same<PT, double>::value || std::is_same<PT, T>::value, "positions: FP64 or T");
    const int32_t  rp   = __ldg(row_ptr + p);
    const int32_t  k    = __ldg(row_ptr + p + 1) - rp - 1;
    const int32_t* rg   = col + rp + 1;
    const bool     wrap = __ldg(bnd + p) == 0;
    T              area = T(0), sumw = T(0);
    if (uniform) {
        for (int32_t i = 0; i < k; ++i) {
            const int32_t r = __ldg(rg + i);
            sumw += dt;
#pragma unroll
            for (int c = 0; c < NC; ++c) acc[c] -= dt * x[(int64_t)r * NC + c];
        }
        area = T(0.5) * (T)k;  // 1 / v_weight = valence
    } else if (k > 0 && k <= 8) {
        // rings of up to 8 neighbours (nearly every row of a triangle mesh):
        // all ids, then all positions and x rows, in flight together; each
        // fan triangle evaluated once (fan_row, bit for bit the per-call
        // values of the general loop below)
        const V3<PT> P = ld3(xyz, (int32_t)p);
        int32_t      id[8];
        V3<PT>       X[8];
        T            xv[8][NC];
#pragma unroll
        for (int i = 0; i < 8; ++i) id[i] = i < k ? __ldg(rg + i) : (int32_t)p;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            X[i] = ld3(xyz, id[i]);
#pragma unroll
            for (int c = 0; c < NC; ++c) xv[i][c] = x[(int64_t)id[i] * NC + c];
        }
        area = fan_row8<T, T>(
            P, k, wrap, dt, X,
            [&](int32_t i, T w) {
                sumw += w;
#pragma unroll
                for (int j = 0; j < 8; ++j)
                    if (j == i)
#pragma unroll
                        for (int c = 0; c < NC; ++c) acc[c] -= w * xv[j][c];
            });
    } else if (k > 0) {
        const V3<PT> P = ld3(xyz, (int32_t)p);
        area           = fan_row<T, T>(
            P, k, wrap, dt, [&](int32_t i) { return ld3(xyz, __ldg(rg + i)); },
            [&](int32_t i, T w) {
                sumw += w;
                const int32_t r = __ldg(rg + i);
#pragma unroll
                for (int c = 0; c < NC; ++c) acc[c] -= w * x[(int64_t)r * NC + c];
            });
    }
    const T vw = T(0.5) / area;
    const T iv = T(1) / vw;
    const T dg = iv + sumw;
#pragma unroll
    for (int c = 0; c < NC; ++c) acc[c] += dg * x[p * NC + c];
    if (diag) *diag = dg;
}

// scalar recurrence of k_cgm, in shared memory, touched by thread 0 only
struct CGMScalars
{
    double delta0, delta, beta;
    int    it;
    bool   conv;
};

// per-thread partial -> grid sum: FP32 partials reduce in FP32 per warp,
// FP64 ones are staged and summed by warp 0 (rxg_gridsum.cuh)
template <int BT, typename Post>
__device__ __forceinline__ bool cgm_sum(float v, double*, GridSum& g, RedSmem& r, Post post)
{
    return grid_sum<BT>(v, g, r, post);
}
template <int BT, typename Post>
__device__ __forceinline__ bool cgm_sum(double v, double* s_part, GridSum& g, RedSmem& r, Post post)
{
    return grid_sum_staged<BT>(v, s_part, g, r, post);
}

// positions of the matrix-free operator: FP64, or their FP32 rounding for T = float
template <typename T>
struct MfPos
{
    __device__ static const double* get(const CGArgs<T>& a) { return a.mf_xyz; }
};
template <>
struct MfPos<float>
{
    __device__ static const float* get(const CGArgs<float>& a) { return a.mf_xyzf; }
};

// L: lanes per matrix row in the two SpMV passes (1, or 4 for long rows).
// MF: the operator is the matrix-free implicit-MCF one (mcf_row; a.rp and
// a.col are the mesh's pattern, a.val is unused).
template <typename T, int NC, bool PC, int kCGT, int L, bool MF = false>
__global__ void __launch_bounds__(kCGT) k_cg(CGArgs<T> a)
{
    __shared__ RedSmem    red;
    __shared__ double     s_part[sizeof(T) == 8 ? kCGT : 1];
    __shared__ CGMScalars c;
    __shared__ T          s_al, s_bt;
    __shared__ int        s_first, s_done;
    const int64_t chunk = (a.n + gridDim.x - 1) / gridDim.x;
    const int64_t r0    = blockIdx.x * chunk;
    const int64_t r1    = min(a.n, r0 + chunk);
    T* const      src   = PC ? a.Z : a.R;  // vector the direction is built from
    GridSum       g{a.bar, a.part, a.err, gridDim.x, 0u, blockIdx.x};
    auto          conv = [&](double d) { return d < a.abs_tol || d / c.delta0 < a.rel_tol; };
    // Per-thread partial dot products stay in T over the thread's few rows;
    // the block and grid reductions are in FP64, and the scalar recurrence
    // runs on thread 0 (rxg_gridsum.cuh).

    // ---- pre_solve: S = A X, R = B - S, Z = D^-1 R, delta = R.Z (or R.R)
    const int lane = (int)threadIdx.x & (L - 1);
    T         tpart = T(0);
    for (int64_t i = r0 + threadIdx.x / L; i < r1; i += kCGT / L) {
        T acc[NC];
#pragma unroll
        for (int k = 0; k < NC; ++k) acc[k] = T(0);
        T diag = T(0);
        if constexpr (MF)
            mcf_row<T, Geo<T>, NC>(a.rp, a.col, a.mf_bnd, MfPos<T>::get(a), (T)a.mf_dt, a.mf_uniform != 0, i,
                                   a.X, acc, &diag);
        else if (L == 1) row_spmv<T, NC>(a.rp, a.col, a.val, i, a.X, acc, &diag);
        else row_spmv_group<T, NC, (L > 1 ? L : 2)>(a.rp, a.col, a.val, i, a.X, acc, &diag, lane);
        if (lane != 0) continue;
        const T di = T(1) / (diag + (sizeof(T) == 4 ? (T)FLT_EPSILON : (T)DBL_EPSILON));
        if (PC) a.dinv[i] = di;
#pragma unroll
        for (int k = 0; k < NC; ++k) {
            const T r       = a.B[i * NC + k] - acc[k];
            a.R[i * NC + k] = r;
            if (PC) {
                const T z       = di * r;
                a.Z[i * NC + k] = z;
                tpart += r * z;
            } else {
                tpart += r * r;
            }
        }
    }
    if (!cgm_sum<kCGT>(tpart, s_part, g, red, [&](double t) {
            c.delta0 = c.delta = t;
            c.beta             = 0.0;
            c.it               = 0;
            c.conv             = conv(t);
            s_bt               = T(0);
            s_first            = 1;
            s_done             = c.conv || a.max_iter <= 0;
        }))
        return;
    T* const P = a.P0;
    while (!s_done) {
        const T    bt    = s_bt;
        const bool first = s_first != 0;
        // ---- phase A: S = A src + beta S (= A p by linearity), p = src + beta p,
        //      S.p.  Only own rows of S and p are read back, so the p update
        //      needs neither extra work per non-zero nor another barrier.
        tpart = T(0);
        for (int64_t i = r0 + threadIdx.x / L; i < r1; i += kCGT / L) {
            T acc[NC];
#pragma unroll
            for (int k = 0; k < NC; ++k) acc[k] = T(0);
            if constexpr (MF)
                mcf_row<T, Geo<T>, NC>(a.rp, a.col, a.mf_bnd, MfPos<T>::get(a), (T)a.mf_dt, a.mf_uniform != 0,
                                       i, src, acc, (T*)nullptr);
            else if (L == 1) row_spmv<T, NC>(a.rp, a.col, a.val, i, src, acc, (T*)nullptr);
            else row_spmv_group<T, NC, (L > 1 ? L : 2)>(a.rp, a.col, a.val, i, src, acc, (T*)nullptr, lane);
            if (lane != 0) continue;
#pragma unroll
            for (int k = 0; k < NC; ++k) {
                const T si = first ? acc[k] : acc[k] + bt * a.S[i * NC + k];
                const T pi = first ? src[i * NC + k] : src[i * NC + k] + bt * P[i * NC + k];
                P[i * NC + k]   = pi;
                a.S[i * NC + k] = si;
                tpart += si * pi;
            }
        }
        if (!cgm_sum<kCGT>(tpart, s_part, g, red, [&](double sp) { s_al = (T)(c.delta / sp); })) return;
        const T al = s_al;
        // ---- phase B: X += alpha p, R -= alpha S, Z = D^-1 R, delta' = R.Z
        tpart = T(0);
        for (int64_t i = r0 + threadIdx.x; i < r1; i += kCGT) {
            const T di = PC ? a.dinv[i] : T(1);
#pragma unroll
            for (int k = 0; k < NC; ++k) {
                a.X[i * NC + k] += al * P[i * NC + k];
                const T r       = a.R[i * NC + k] - al * a.S[i * NC + k];
                a.R[i * NC + k] = r;
                if (PC) {
                    const T z       = di * r;
                    a.Z[i * NC + k] = z;
                    tpart += r * z;
                } else {
                    tpart += r * r;
                }
            }
        }
        if (!cgm_sum<kCGT>(tpart, s_part, g, red, [&](double dn) {
                if (conv(dn)) {
                    c.delta = dn;
                    c.conv  = true;
                    s_done  = 1;
                    return;
                }
                c.beta  = dn / c.delta;
                c.delta = dn;
                ++c.it;
                s_bt    = (T)c.beta;
                s_first = 0;
                s_done  = c.it >= a.max_iter;
            }))
            return;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.dstat[0] = c.delta0;
        a.dstat[1] = c.delta;
        a.istat[0] = c.it;
        a.istat[1] = c.conv ? 1 : 0;
    }
}

// ---------------------------------------------------------------------
// host side: CG launch
// ---------------------------------------------------------------------

static int num_sms() { return device_sm_count(); }

// CTA size of the persistent CG kernel: RXG_CG_THREADS=256|512|1024 (default 512)
static int cg_threads()
{
    static int t = 0;
    if (!t) {
        const char* e = getenv("RXG_CG_THREADS");
        t             = e ? atoi(e) : 512;
        if (t != 256 && t != 512 && t != 1024) t = 512;
    }
    return t;
}

template <typename T, int NC, bool PC, int BT, bool MF = false>
static int cg_grid_bt(int64_t n)
{
    // resident CTAs per SM, per device (0: not looked up yet)
    static int per_sm_dev[kMaxDevices] = {0};
    int&       per_sm = per_sm_dev[current_device()];
    if (per_sm <= 0) {
        // the grid must fit whichever variant runs (cooperative launch)
        int p1 = 0, p4 = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&p1, k_cg<T, NC, PC, BT, 1, MF>, BT, 0) !=
            cudaSuccess)
            p1 = 1;
        p4 = p1;
        if constexpr (NC == 1 && !MF)
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&p4, k_cg<T, NC, PC, BT, 4>, BT, 0) !=
                cudaSuccess)
                p4 = 1;
        per_sm = std::min(p1, p4);
        int cap = 4;
        if (const char* e = getenv("RXG_CG_BLOCKS_PER_SM")) cap = std::max(1, atoi(e));
        per_sm = std::max(1, std::min(per_sm, cap));
    }
    int64_t g = (int64_t)num_sms() * per_sm;
    g         = std::min<int64_t>(g, std::max<int64_t>(1, (n + 31) / 32));
    return (int)g;
}

template <typename T, int NC, bool PC, bool MF = false>
static int cg_grid(int64_t n)
{
    switch (cg_threads()) {
        case 256: return cg_grid_bt<T, NC, PC, 256, MF>(n);
        case 1024: return cg_grid_bt<T, NC, PC, 1024, MF>(n);
        default: return cg_grid_bt<T, NC, PC, 512, MF>(n);
    }
}

static size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

template <typename T>
static size_t cg_scratch_bytes(int64_t n, int nc, int G)
{
    return 5 * align256(sizeof(T) * n * nc) + align256(sizeof(T) * n) +
           align256(sizeof(double) * 2 * G) + 3 * 256;
}

// matrix-free operator of the MF launches (unused otherwise)
struct MatFreeOp
{
    const int8_t* bnd     = nullptr;
    const double* xyz     = nullptr;
    const float*  xyzf    = nullptr;  // FP32 rounding of xyz (T = float)
    double        dt      = 0.0;
    int           uniform = 0;
};

template <typename T, int NC, bool PC, bool MF = false>
static rxg_status cg_launch(int64_t n, int64_t nnz, const int32_t* rp, const int32_t* col,
                            const T* val, const T* B, T* X, const rxg_solver_opts& o,
                            rxg_solver_stats* st, uint8_t* scratch, cudaStream_t s,
                            const MatFreeOp& mf = MatFreeOp())
{
    const int  G = cg_grid<T, NC, PC, MF>(n);
    CGArgs<T>  a;
    a.mf_bnd     = mf.bnd;
    a.mf_xyz     = mf.xyz;
    a.mf_xyzf    = mf.xyzf;
    a.mf_dt      = mf.dt;
    a.mf_uniform = mf.uniform;
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
    RXG_CUDA_TRY(reset_grid_sum(a.bar, s));
    void* args[] = {&a};
    // rows of 12 or more entries on average (a Hessian's scalar form): four
    // lanes per row in the SpMV passes, so adjacent lanes read adjacent entries
    const bool  l4 = n > 0 && nnz >= 12 * n;
    const int   bt = cg_threads();
    const void* kern;
    if constexpr (MF) {
        (void)l4;
        kern = bt == 256    ? (const void*)k_cg<T, NC, PC, 256, 1, true>
               : bt == 1024 ? (const void*)k_cg<T, NC, PC, 1024, 1, true>
                            : (const void*)k_cg<T, NC, PC, 512, 1, true>;
    } else if constexpr (NC == 1) {
        if (l4)
            kern = bt == 256    ? (const void*)k_cg<T, NC, PC, 256, 4>
                   : bt == 1024 ? (const void*)k_cg<T, NC, PC, 1024, 4>
                                : (const void*)k_cg<T, NC, PC, 512, 4>;
        else
            kern = bt == 256    ? (const void*)k_cg<T, NC, PC, 256, 1>
                   : bt == 1024 ? (const void*)k_cg<T, NC, PC, 1024, 1>
                                : (const void*)k_cg<T, NC, PC, 512, 1>;
    } else {
        (void)l4;
        kern = bt == 256    ? (const void*)k_cg<T, NC, PC, 256, 1>
               : bt == 1024 ? (const void*)k_cg<T, NC, PC, 1024, 1>
                            : (const void*)k_cg<T, NC, PC, 512, 1>;
    }
    RXG_CUDA_TRY(cudaLaunchCooperativeKernel(kern, dim3(G), dim3(cg_threads()), args, 0, s));
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
static rxg_status cg_dispatch(int nc, int64_t n, int64_t nnz, const int32_t* rp,
                              const int32_t* col, const T* val, const T* B, T* X,
                              const rxg_solver_opts& o, rxg_solver_stats* st, uint8_t* scratch,
                              cudaStream_t s)
{
#define RXG_CG_CASE(NCV)                                                                          \
    case NCV:                                                                                     \
        return o.precond ? cg_launch<T, NCV, true>(n, nnz, rp, col, val, B, X, o, st, scratch, s) \
                         : cg_launch<T, NCV, false>(n, nnz, rp, col, val, B, X, o, st, scratch, s);
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

// Grid of a grid-stride kernel rounded down to whole waves (SMs x resident
// CTAs of `kern`) once it exceeds one: the grid-stride loop spreads the rest
// over all threads instead of running a short last wave (9% faster for the
// level-8 FP32 SpMM, 2,561 -> 2,432 CTAs).
template <typename K>
static int whole_wave_grid(K kern, int64_t n, int threads)
{
    int64_t blocks = (n + threads - 1) / threads;
    int     per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, 0) != cudaSuccess) {
        cudaGetLastError();
        per_sm = 0;
    }
    const int64_t wave = (int64_t)std::max(1, per_sm) * device_sm_count();
    if (per_sm > 0 && blocks > wave) blocks = (blocks / wave) * wave;
    return (int)std::max<int64_t>(1, std::min<int64_t>(blocks, 152 * 32));
}

template <typename TA, typename TX, typename TACC>
static rxg_status spmm_launch(int nc, int64_t n, const int32_t* rp, const int32_t* col,
                              const TA* val, const TX* x, const TACC* b, TACC* y, cudaStream_t s)
{
#define RXG_SPMM_CASE(NCV)                                                                     \
    case NCV:                                                                                  \
        if (b)                                                                                 \
            k_spmm<TA, TX, TACC, NCV, true>                                                    \
                <<<whole_wave_grid(k_spmm<TA, TX, TACC, NCV, true>, n, 256), 256, 0, s>>>(     \
                    n, rp, col, val, x, b, y);                                                 \
        else                                                                                   \
            k_spmm<TA, TX, TACC, NCV, false>                                                   \
                <<<whole_wave_grid(k_spmm<TA, TX, TACC, NCV, false>, n, 256), 256, 0, s>>>(    \
                    n, rp, col, val, x, b, y);                                                 \
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
        w = std::max(w, (size_t)pad4i(h.nEl) + few + pad4i(h.nVl - h.nVo) + pad4i(h.nFl - h.nFo) +
                            2 * pad4i(h.nVo + 1) + 3 * (size_t)h.nFl);
    }
    return w * 4;
}

static rxg_status launch_oriented(const Mesh* m, int32_t* off, int32_t* val, int8_t* bnd,
                                  int32_t* rface, cudaStream_t s)
{
    const size_t smem = oriented_smem_bytes(m);
    if (smem > 227 * 1024) {
        set_error("oriented VV: a patch needs %zu bytes of shared memory", smem);
        return RXG_ERR_PATCH_LIMIT;
    }
    if (smem > 48 * 1024)
        RXG_CUDA_TRY(cudaFuncSetAttribute(k_oriented_vv, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem));
    k_oriented_vv<<<m->num_patches, kQT2, smem, s>>>(m->d.hdr, m->d.arena, off, val, bnd, rface,
                                                      device_error_word());
    RXG_CUDA_TRY(cudaGetLastError());
    return RXG_OK;
}

rxg_status ensure_pattern(const Mesh* m, cudaStream_t s, Lazy** out)
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
    RXG_CUDA_TRY(cudaMalloc(&z->ring_face, 4 * std::max<int64_t>(1, 2 * ne)));
    rxg_status st = launch_oriented(m, z->ring_off, z->ring, z->bnd, z->ring_face, s);
    if (st) return st;
    k_pattern<<<grid_for(nv + 1), 256, 0, s>>>(nv, z->ring_off, z->ring, z->row_ptr, z->col);
    RXG_CUDA_TRY(cudaGetLastError());
    st = check_device_error(s);
    if (st) return st;
    z->ring_ready = true;
    return RXG_OK;
}

// ---------------------------------------------------------------------
// Persistent Jacobi-PCG on the packed MCF layout: the same iteration as
// k_cg (fused barrier-reductions, S carried as A z + beta S) on 4-wide row
// vectors and (column, value) entries, so a row, a neighbour or a non-zero
// is one wide access.  Used by the MCF step for both precisions.
// ---------------------------------------------------------------------

template <typename T>
struct CGMArgs
{
    int64_t        n;
    const int32_t* rp;
    const Ent<T>*  ent;
    const R4<T>*   B;
    R4<T>*         X;
    R4<T>*         R;
    R4<T>*         P;
    R4<T>*         S;
    R4<T>*         Z;
    T*             dinv;
    double*        part;
    unsigned*      bar;
    double*        dstat;
    int*           istat;
    int            max_iter;
    double         abs_tol, rel_tol;
    int*           err;
};

template <typename T, int kBT>
__global__ void __launch_bounds__(kBT) k_cgm(CGMArgs<T> a)
{
    __shared__ RedSmem    red;
    __shared__ double     s_part[sizeof(T) == 8 ? kBT : 1];
    __shared__ CGMScalars c;
    __shared__ T          s_al, s_bt;
    __shared__ int        s_first, s_done;
    const int64_t chunk = (a.n + gridDim.x - 1) / gridDim.x;
    const int64_t r0    = blockIdx.x * chunk;
    const int64_t r1    = min(a.n, r0 + chunk);
    const T       eps   = sizeof(T) == 4 ? (T)FLT_EPSILON : (T)DBL_EPSILON;
    GridSum       g{a.bar, a.part, a.err, gridDim.x, 0u, blockIdx.x};
    auto          conv = [&](double d) { return d < a.abs_tol || d / c.delta0 < a.rel_tol; };

    // ---- pre_solve: R = B - A X, Z = D^-1 R, delta = R.Z
    T tpart = T(0);
    for (int64_t i = r0 + threadIdx.x; i < r1; i += kBT) {
        T ax = 0, ay = 0, az = 0, diag = 0;
        row_spmv4<T>(a.rp, a.ent, i, a.X, ax, ay, az, &diag);
        const T     di = T(1) / (diag + eps);
        const R4<T> b  = a.B[i];
        R4<T>       r, z;
        r.x = b.x - ax, r.y = b.y - ay, r.z = b.z - az, r.w = T(0);
        z.x = di * r.x, z.y = di * r.y, z.z = di * r.z, z.w = T(0);
        a.dinv[i] = di;
        a.R[i]    = r;
        a.Z[i]    = z;
        tpart += r.x * z.x + r.y * z.y + r.z * z.z;
    }
    if (!cgm_sum<kBT>(tpart, s_part, g, red, [&](double t) {
            c.delta0 = c.delta = t;
            c.beta             = 0.0;
            c.it               = 0;
            c.conv             = conv(t);
            s_bt               = T(0);
            s_first            = 1;
            s_done             = c.conv || a.max_iter <= 0;
        }))
        return;
    while (!s_done) {
        const T    bt    = s_bt;
        const bool first = s_first != 0;
        // ---- phase A: S = A z + beta S, p = z + beta p, S.p
        tpart = T(0);
        for (int64_t i = r0 + threadIdx.x; i < r1; i += kBT) {
            T ax = 0, ay = 0, az = 0;
            row_spmv4<T>(a.rp, a.ent, i, a.Z, ax, ay, az, (T*)nullptr);
            const R4<T> zi = a.Z[i];
            R4<T>       si, pi;
            if (first) {
                si.x = ax, si.y = ay, si.z = az;
                pi = zi;
            } else {
                const R4<T> so = a.S[i], po = a.P[i];
                si.x = ax + bt * so.x, si.y = ay + bt * so.y, si.z = az + bt * so.z;
                pi.x = zi.x + bt * po.x, pi.y = zi.y + bt * po.y, pi.z = zi.z + bt * po.z;
            }
            si.w = pi.w = T(0);
            a.S[i] = si;
            a.P[i] = pi;
            tpart += si.x * pi.x + si.y * pi.y + si.z * pi.z;
        }
        if (!cgm_sum<kBT>(tpart, s_part, g, red, [&](double sp) { s_al = (T)(c.delta / sp); })) return;
        const T al = s_al;
        // ---- phase B: X += alpha p, R -= alpha S, Z = D^-1 R, R.Z
        tpart = T(0);
        for (int64_t i = r0 + threadIdx.x; i < r1; i += kBT) {
            const T     di = a.dinv[i];
            R4<T>       x  = a.X[i], r = a.R[i];
            const R4<T> pi = a.P[i], si = a.S[i];
            x.x += al * pi.x, x.y += al * pi.y, x.z += al * pi.z;
            r.x -= al * si.x, r.y -= al * si.y, r.z -= al * si.z;
            R4<T> z;
            z.x = di * r.x, z.y = di * r.y, z.z = di * r.z, z.w = T(0);
            a.X[i] = x;
            a.R[i] = r;
            a.Z[i] = z;
            tpart += r.x * z.x + r.y * z.y + r.z * z.z;
        }
        if (!cgm_sum<kBT>(tpart, s_part, g, red, [&](double dn) {
                if (conv(dn)) {
                    c.delta = dn;
                    c.conv  = true;
                    s_done  = 1;
                    return;
                }
                c.beta  = dn / c.delta;
                c.delta = dn;
                ++c.it;
                s_bt    = (T)c.beta;
                s_first = 0;
                s_done  = c.it >= a.max_iter;
            }))
            return;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.dstat[0] = c.delta0;
        a.dstat[1] = c.delta;
        a.istat[0] = c.it;
        a.istat[1] = c.conv ? 1 : 0;
    }
}

// CTA size of the packed MCF solver: RXG_MCF_CG_THREADS=256|512|1024 (default 1024)
static int cgm_threads()
{
    static int t = 0;
    if (!t) {
        const char* e = getenv("RXG_MCF_CG_THREADS");
        t             = e ? atoi(e) : 1024;
        if (t != 256 && t != 512 && t != 1024) t = 1024;
    }
    return t;
}

template <typename T, int BT>
static int cgm_grid_bt(int64_t n)
{
    static int per_sm_dev[kMaxDevices] = {0};
    int&       per_sm = per_sm_dev[current_device()];
    if (per_sm <= 0) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cgm<T, BT>, BT, 0) != cudaSuccess)
            per_sm = 1;
        per_sm = std::max(1, std::min(per_sm, 2048 / BT));
    }
    int64_t g = (int64_t)num_sms() * per_sm;
    return (int)std::min<int64_t>(g, std::max<int64_t>(1, (n + 31) / 32));
}

template <typename T>
static int cgm_grid(int64_t n)
{
    switch (cgm_threads()) {
        case 256: return cgm_grid_bt<T, 256>(n);
        case 512: return cgm_grid_bt<T, 512>(n);
        default: return cgm_grid_bt<T, 1024>(n);
    }
}

template <typename T>
static size_t cgm_scratch_bytes(int64_t n, int G)
{
    return 4 * align256(sizeof(R4<T>) * n) + align256(sizeof(T) * n) +
           align256(sizeof(double) * 2 * G) + 3 * 256;
}

template <typename T>
static rxg_status cgm_launch(int64_t n, const int32_t* rp, const Ent<T>* ent, const R4<T>* B,
                             R4<T>* X, const rxg_solver_opts& o, rxg_solver_stats* st,
                             uint8_t* scratch, cudaStream_t s)
{
    const int    G  = cgm_grid<T>(n);
    const size_t vb = align256(sizeof(R4<T>) * n);
    CGMArgs<T>   a;
    uint8_t*     q = scratch;
    a.n   = n;
    a.rp  = rp;
    a.ent = ent;
    a.B   = B;
    a.X   = X;
    a.R = (R4<T>*)q, q += vb;
    a.P = (R4<T>*)q, q += vb;
    a.S = (R4<T>*)q, q += vb;
    a.Z = (R4<T>*)q, q += vb;
    a.dinv  = (T*)q, q += align256(sizeof(T) * n);
    a.part  = (double*)q, q += align256(sizeof(double) * 2 * G);
    a.bar   = (unsigned*)q, q += 256;
    a.dstat = (double*)q, q += 256;
    a.istat = (int*)q, q += 256;
    a.max_iter = o.max_iter;
    a.abs_tol  = o.abs_tol;
    a.rel_tol  = o.rel_tol;
    a.err      = device_error_word();
    RXG_CUDA_TRY(reset_grid_sum(a.bar, s));
    void*       args[] = {&a};
    const void* kern   = cgm_threads() == 256   ? (const void*)k_cgm<T, 256>
                         : cgm_threads() == 512 ? (const void*)k_cgm<T, 512>
                                                : (const void*)k_cgm<T, 1024>;
    RXG_CUDA_TRY(cudaLaunchCooperativeKernel(kern, dim3(G), dim3(cgm_threads()), args, 0, s));
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
    return RXG_OK;
}

// RXG_MCF_VERBOSE=1 prints one line per refinement sweep to stderr
static bool mcf_verbose()
{
    static int v = -1;
    if (v < 0) {
        const char* e = getenv("RXG_MCF_VERBOSE");
        v             = (e && e[0] == '1') ? 1 : 0;
    }
    return v == 1;
}

// positions n x 3 (caller layout) <-> 4-wide
__global__ void k_pack3(int64_t n, const double* __restrict__ x, R4<double>* __restrict__ y)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        R4<double> v;
        v.x = x[3 * i], v.y = x[3 * i + 1], v.z = x[3 * i + 2], v.w = 0.0;
        y[i] = v;
    }
}
__global__ void k_unpack3(int64_t n, const R4<double>* __restrict__ y, double* __restrict__ x)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const R4<double> v = y[i];
        x[3 * i] = v.x, x[3 * i + 1] = v.y, x[3 * i + 2] = v.z;
    }
}

// x += d (FP64 += FP32 correction)
__global__ void k_add_correction4(int64_t n, R4<double>* __restrict__ x, const R4<float>* __restrict__ d)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        R4<double>      v = x[i];
        const R4<float> c = d[i];
        v.x += (double)c.x, v.y += (double)c.y, v.z += (double)c.z;
        x[i] = v;
    }
}

// r = B - A x accumulated in FP64 from the FP32 off-diagonal entries and the
// FP64 diagonal (2*area + the sum of the FP32 weights); r32 = (float) r;
// per-block r . D^-1 r (the Jacobi-weighted norm the plain PCG stops on)
__global__ void __launch_bounds__(256) k_resid_mixed4(int64_t n, const int32_t* __restrict__ rp,
                                                      const Ent<float>* __restrict__ ent,
                                                      const double* __restrict__ diag,
                                                      const R4<double>* __restrict__ x,
                                                      const R4<double>* __restrict__ B,
                                                      R4<float>* __restrict__ r32,
                                                      double* __restrict__ part)
{
    __shared__ double s_red[256 / 32 + 2];
    double            acc2 = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const R4<double> xi = x[i];
        const double     d  = diag[i];
        double           a0 = d * xi.x, a1 = d * xi.y, a2 = d * xi.z;
        const int32_t    e  = rp[i + 1];
        // the off-diagonal entries, six per round (a valence-6 row in one
        // round with no padded FP64 multiply-add)
        for (int32_t j0 = rp[i] + 1; j0 < e; j0 += 6) {
            Ent<float> q[6];
#pragma unroll
            for (int u = 0; u < 6; ++u) {
                if (j0 + u < e) {
                    q[u] = ent[j0 + u];
                } else {
                    q[u].col = (int32_t)i;
                    q[u].val = 0.f;
                }
            }
#pragma unroll
            for (int u = 0; u < 6; ++u) {
                const double     v  = (double)q[u].val;
                const R4<double> xv = x[q[u].col];
                a0 += v * xv.x, a1 += v * xv.y, a2 += v * xv.z;
            }
        }
        const R4<double> b  = B[i];
        const double     e0 = b.x - a0, e1 = b.y - a1, e2 = b.z - a2;
        R4<float>        r;
        r.x = (float)e0, r.y = (float)e1, r.z = (float)e2, r.w = 0.f;
        r32[i] = r;
        acc2 += (e0 * e0 + e1 * e1 + e2 * e2) / d;
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
    if (!b) RXG_CUDA_TRY(scratch_alloc((void**)&b, std::max<int64_t>(16, h->m.nv), S_(stream)));
    rxg_status st = launch_oriented(&h->m, offsets, values, b, nullptr, S_(stream));
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
            nv, z->row_ptr, z->col, z->bnd, xyz, dt, CsrOut<double, double>{(double*)A->val, (double*)B});
    else
        k_mcf_assemble<float, GeoMixed, float><<<g, 256, 0, s>>>(
            nv, z->row_ptr, z->col, z->bnd, xyz, (float)dt, CsrOut<float, float>{(float*)A->val, (float*)B});
    RXG_CUDA_TRY(cudaGetLastError());
    return RXG_OK;
}

rxg_status rxg_spmm(const rxg_csr* A, int32_t nc, const void* X, void* Y, void* stream)
{
    if (!A || !X || !Y || nc < 1 || nc > 4) {
        set_error("rxg_spmm: bad argument");
        return RXG_ERR_INVALID;
    }
    if (!is_device_ptr(X) || !is_device_ptr(Y) || !is_device_ptr(A->val) ||
        !is_device_ptr(A->row_ptr) || !is_device_ptr(A->col)) {
        set_error("rxg_spmm: A (row_ptr, col, val), X and Y must be device arrays");
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
    if (!is_device_ptr(B) || !is_device_ptr(X) || !is_device_ptr(A->val) ||
        !is_device_ptr(A->row_ptr) || !is_device_ptr(A->col)) {
        set_error("rxg_cg_solve: A (row_ptr, col, val), B and X must be device arrays");
        return RXG_ERR_INVALID;
    }
    cudaStream_t s  = S_(stream);
    const bool   pc = opts->precond != 0;
    rxg_solver_stats local;
    rxg_status       st;
    uint8_t*         scratch = nullptr;
    if (A->dtype == RXG_F64) {
        const size_t bytes = cg_scratch_bytes<double>(A->n, nc, cg_grid_any<double>(nc, pc, A->n));
        RXG_CUDA_TRY(scratch_alloc((void**)&scratch, bytes, s));
        st = cg_dispatch<double>(nc, A->n, A->nnz, A->row_ptr, A->col, (const double*)A->val,
                                 (const double*)B, (double*)X, *opts, &local, scratch, s);
    } else {
        const size_t bytes = cg_scratch_bytes<float>(A->n, nc, cg_grid_any<float>(nc, pc, A->n));
        RXG_CUDA_TRY(scratch_alloc((void**)&scratch, bytes, s));
        st = cg_dispatch<float>(nc, A->n, A->nnz, A->row_ptr, A->col, (const float*)A->val,
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
    const int     Gr = grid_for(n);
    // buffers: X4 (FP64 positions), B4 (FP64 RHS), packed A, then per precision
    const size_t x4b = align256(sizeof(R4<double>) * n);
    const size_t plain = 2 * x4b + align256(sizeof(Ent<double>) * nnz) +
                         cgm_scratch_bytes<double>(n, cgm_grid<double>(n));
    const int64_t max_row = h->m.max_valence + 1;  // diagonal + one-ring
    const size_t mixed = 2 * x4b + align256(sizeof(Ent<float>) * nnz) +
                         2 * align256(sizeof(R4<float>) * n) + align256(8 * Gr) + align256(8 * n) +
                         std::max(cgm_scratch_bytes<float>(n, cgm_grid<float>(n)),
                                  mcf_onchip_scratch_bytes(n, max_row));
    {
        std::lock_guard<std::mutex> g(z->mu);
        if ((st = mcf_buffers(z, std::max(plain, mixed), s))) return st;
    }
    // positions: device, or staged from host
    double* X      = xyz;
    bool    staged = false;
    if (!is_device_ptr(xyz)) {
        RXG_CUDA_TRY(scratch_alloc((void**)&X, 24 * n, s));
        RXG_CUDA_TRY(cudaMemcpyAsync(X, xyz, 24 * n, cudaMemcpyHostToDevice, s));
        staged = true;
    }
    uint8_t*    q  = (uint8_t*)z->buf;
    R4<double>* X4 = (R4<double>*)q;
    R4<double>* B4 = (R4<double>*)(q + x4b);
    uint8_t*    p  = q + 2 * x4b;
    rxg_solver_stats last   = {0, 1, 0.0, 0.0};
    const int        ga     = grid_for(n);
    const bool       onchip = precision == RXG_F32 && mcf_onchip_fits(n, max_row);
    k_pack3<<<ga, 256, 0, s>>>(n, X, X4);
    for (int step = 0; step < nsteps && st == RXG_OK; ++step) {
        // the assembly reads the caller-layout positions of this step
        if (step > 0) k_unpack3<<<ga, 256, 0, s>>>(n, X4, X);
        if (precision == RXG_F64) {
            Ent<double>* ent = (Ent<double>*)p;
            uint8_t*     scr = p + align256(sizeof(Ent<double>) * nnz);
            const auto ka = k_mcf_assemble<double, Geo<double>, double, PackedOut<double, double>>;
            ka<<<whole_wave_grid(ka, n, 256), 256, 0, s>>>(n, z->row_ptr, z->col, z->bnd, X, dt,
                                                         PackedOut<double, double>{ent, B4, nullptr});
            RXG_CUDA_TRY(cudaGetLastError());
            rxg_solver_opts o = {max_iter, 0.0, tol * tol, 1};
            st = cgm_launch<double>(n, z->row_ptr, ent, B4, X4, o, &last, scr, s);
        } else {
            Ent<float>* ent = (Ent<float>*)p;
            uint8_t*    w   = p + align256(sizeof(Ent<float>) * nnz);
            R4<float>*  r32 = (R4<float>*)w;
            w += align256(sizeof(R4<float>) * n);
            R4<float>* d32 = (R4<float>*)w;
            w += align256(sizeof(R4<float>) * n);
            double* part = (double*)w;
            w += align256(8 * Gr);
            double* D64 = (double*)w;
            w += align256(8 * n);
            uint8_t* scr = w;
            const auto ka = k_mcf_assemble<float, GeoMixed, double, PackedOut<float, double>>;
            ka<<<whole_wave_grid(ka, n, 256), 256, 0, s>>>(n, z->row_ptr, z->col, z->bnd, X, (float)dt,
                                                         PackedOut<float, double>{ent, B4, D64});
            RXG_CUDA_TRY(cudaGetLastError());
            if (onchip) {
                // whole refinement in one launch; statistics read after the last step
                st = mcf_onchip_solve(z, n, max_row, ent, D64, B4, X4, r32, scr, tol, max_iter, s);
                if (st == RXG_OK && step == nsteps - 1) st = mcf_onchip_stats(scr, &last, s);
                continue;
            }
            k_resid_mixed4<<<Gr, 256, 0, s>>>(n, z->row_ptr, ent, D64, X4, B4, r32, part);
            double rr0;
            if ((st = reduce_partials(part, Gr, s, &rr0))) break;
            double rr       = rr0;
            int    total_it = 0;
            bool   conv     = rr0 == 0.0;
            for (int sweep = 0; sweep < 16 && !conv && total_it < max_iter; ++sweep) {
                // solve only as far as this sweep needs, but not below FP32's reach
                const double need  = tol * std::sqrt(rr0 / rr);
                const double inner = std::max(1e-4, 0.3 * need);
                RXG_CUDA_TRY(cudaMemsetAsync(d32, 0, sizeof(R4<float>) * n, s));
                rxg_solver_opts  o = {max_iter - total_it, 0.0, inner * inner, 1};
                rxg_solver_stats si;
                st = cgm_launch<float>(n, z->row_ptr, ent, r32, d32, o, &si, scr, s);
                if (st) break;
                total_it += si.iters + 1;
                k_add_correction4<<<ga, 256, 0, s>>>(n, X4, d32);
                k_resid_mixed4<<<Gr, 256, 0, s>>>(n, z->row_ptr, ent, D64, X4, B4, r32, part);
                if ((st = reduce_partials(part, Gr, s, &rr))) break;
                conv = rr < tol * tol * rr0;
                if (mcf_verbose())
                    fprintf(stderr, "rxg mcf mixed: sweep %d inner_tol %.3g iters %d conv %d "
                                    "gamma %.3g -> %.3g |r|^2/|r0|^2 %.3g\n",
                            sweep, inner, si.iters, si.converged, si.start_res, si.final_res,
                            rr / rr0);
            }
            last.iters     = total_it;
            last.converged = conv ? 1 : 0;
            last.start_res = rr0;
            last.final_res = rr;
        }
    }
    if (st == RXG_OK) {
        k_unpack3<<<ga, 256, 0, s>>>(n, X4, X);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) st = cuda_status(e, "rxg_mcf_step");
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

namespace rxg {

// ---------------------------------------------------------------------
// Matrix-free implicit MCF (init_B / matvec / precond_matvec of
// apps/MCF/mcf_kernels.cuh:58-299, CGMatFreeAttrSolver of
// matrix/cg_mat_free_attr_solver.h:45-115): the operator's weights are
// recomputed from the positions on every product (mcf_row), nothing is
// assembled.  The pattern is the mesh's cached [diagonal, oriented ring].
// ---------------------------------------------------------------------

// CTAs per SM the FP32 product is compiled for: its rows hold eight ring
// positions and x rows in registers, and at one CTA-pair per SM (116
// registers) too few warps hide the latency of its divisions and square roots
template <typename T>
constexpr int matvec_min_ctas()
{
    return sizeof(T) == 4 ? 3 : 1;
}

// out = A in (JACOBI: out = D^-1 in, D = diag(A)), row-major nv x 3
template <typename T, bool JACOBI, typename PT>
__global__ void __launch_bounds__(256, matvec_min_ctas<T>()) k_mcf_matvec(int64_t nv, const int32_t* __restrict__ rp,
                                                    const int32_t* __restrict__ col,
                                                    const int8_t* __restrict__ bnd,
                                                    const PT* __restrict__ xyz, T dt, int uniform,
                                                    const T* __restrict__ in, T* __restrict__ out)
{
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nv;
         p += (int64_t)gridDim.x * blockDim.x) {
        T acc[3] = {T(0), T(0), T(0)};
        T dg     = T(0);
        mcf_row<T, Geo<T>, 3, PT>(rp, col, bnd, xyz, dt, uniform != 0, p, in, acc, &dg);
#pragma unroll
        for (int c = 0; c < 3; ++c) out[3 * p + c] = JACOBI ? in[3 * p + c] / dg : acc[c];
    }
}

// the FP32 rounding of n FP64 position triples
__global__ void __launch_bounds__(256) k_round_f32(int64_t n3, const double* __restrict__ x, float* __restrict__ y)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n3; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = (float)__ldg(x + i);
}

// B = (1 / v_weight) x: 2 x (clamped Voronoi area) x in cotangent mode, the
// valence x in uniform mode (init_B, mcf_kernels.cuh:58-98)
template <typename T>
__global__ void __launch_bounds__(256) k_mcf_init_b(int64_t nv, const int32_t* __restrict__ rp,
                                                    const int32_t* __restrict__ col,
                                                    const int8_t* __restrict__ bnd,
                                                    const double* __restrict__ xyz, int uniform,
                                                    T* __restrict__ B)
{
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nv;
         p += (int64_t)gridDim.x * blockDim.x) {
        const int32_t  r0   = rp[p];
        const int32_t  k    = rp[p + 1] - r0 - 1;
        const int32_t* rg   = col + r0 + 1;
        const bool     wrap = bnd[p] == 0;
        T              area = T(0);
        if (uniform) {
            area = T(0.5) * (T)k;
        } else if (k > 0) {
            const V3<double> P = ld3(xyz, (int32_t)p);
            V3<double>       Q = ld3(xyz, rg[k - 1]);
            for (int32_t i = 0; i < k; ++i) {
                const V3<double> R = ld3(xyz, rg[i]);
                if (wrap || i > 0) {
                    const T a = Geo<T>::va(P, Q, R);
                    area += a > T(0) ? a : T(0);
                }
                Q = R;
            }
        }
        const T vw = T(0.5) / area;
        const T iv = T(1) / vw;
        const V3<double> P = ld3(xyz, (int32_t)p);
        B[3 * p + 0] = iv * (T)P.x;
        B[3 * p + 1] = iv * (T)P.y;
        B[3 * p + 2] = iv * (T)P.z;
    }
}

}  // namespace rxg

using namespace rxg;

extern "C" {

rxg_status rxg_mcf_matvec(const rxg_mesh* h, double dt, int32_t flags, int32_t dtype,
                          const double* xyz, const void* in, void* out, void* stream)
{
    if (!h || !xyz || !in || !out || (dtype != RXG_F32 && dtype != RXG_F64) ||
        (flags & ~(RXG_MCF_UNIFORM_LAPLACE | RXG_MCF_JACOBI))) {
        set_error("rxg_mcf_matvec: bad argument");
        return RXG_ERR_INVALID;
    }
    if (!is_device_ptr(xyz) || !is_device_ptr(in) || !is_device_ptr(out)) {
        set_error("rxg_mcf_matvec: xyz, in and out must be device arrays");
        return RXG_ERR_INVALID;
    }
    Lazy*        z;
    cudaStream_t s  = S_(stream);
    rxg_status   st = ensure_pattern(&h->m, s, &z);
    if (st) return st;
    const int64_t nv = h->m.nv;
    const int     u  = (flags & RXG_MCF_UNIFORM_LAPLACE) ? 1 : 0;
    const bool    jc = (flags & RXG_MCF_JACOBI) != 0;
    if (dtype == RXG_F64) {
        if (jc)
            k_mcf_matvec<double, true, double><<<whole_wave_grid(k_mcf_matvec<double, true, double>, nv, 256), 256, 0, s>>>(nv, z->row_ptr, z->col, z->bnd, xyz, dt, u,
                                                                 (const double*)in, (double*)out);
        else
            k_mcf_matvec<double, false, double><<<whole_wave_grid(k_mcf_matvec<double, false, double>, nv, 256), 256, 0, s>>>(nv, z->row_ptr, z->col, z->bnd, xyz, dt, u,
                                                                  (const double*)in, (double*)out);
        RXG_CUDA_TRY(cudaGetLastError());
        return RXG_OK;
    }
    // FP32: the positions rounded once (k_round_f32), not per row
    float* xf = nullptr;
    if (!u) {
        RXG_CUDA_TRY(scratch_alloc((void**)&xf, sizeof(float) * 3 * (size_t)nv, s));
        k_round_f32<<<grid_for(3 * nv), 256, 0, s>>>(3 * nv, xyz, xf);
    }
    if (jc)
        k_mcf_matvec<float, true, float><<<whole_wave_grid(k_mcf_matvec<float, true, float>, nv, 256), 256, 0, s>>>(nv, z->row_ptr, z->col, z->bnd, xf, (float)dt, u,
                                                           (const float*)in, (float*)out);
    else
        k_mcf_matvec<float, false, float><<<whole_wave_grid(k_mcf_matvec<float, false, float>, nv, 256), 256, 0, s>>>(nv, z->row_ptr, z->col, z->bnd, xf, (float)dt, u,
                                                            (const float*)in, (float*)out);
    const cudaError_t e = cudaGetLastError();
    if (xf) cudaFreeAsync(xf, s);
    RXG_CUDA_TRY(e);
    return RXG_OK;
}

rxg_status rxg_mcf_init_b(const rxg_mesh* h, int32_t flags, int32_t dtype, const double* xyz, void* B,
                          void* stream)
{
    if (!h || !xyz || !B || (dtype != RXG_F32 && dtype != RXG_F64) ||
        (flags & ~(RXG_MCF_UNIFORM_LAPLACE | RXG_MCF_JACOBI))) {
        set_error("rxg_mcf_init_b: bad argument");
        return RXG_ERR_INVALID;
    }
    if (!is_device_ptr(xyz) || !is_device_ptr(B)) {
        set_error("rxg_mcf_init_b: xyz and B must be device arrays");
        return RXG_ERR_INVALID;
    }
    Lazy*        z;
    cudaStream_t s  = S_(stream);
    rxg_status   st = ensure_pattern(&h->m, s, &z);
    if (st) return st;
    const int64_t nv = h->m.nv;
    const int     u  = (flags & RXG_MCF_UNIFORM_LAPLACE) ? 1 : 0;
    if (dtype == RXG_F64)
        k_mcf_init_b<double><<<grid_for(nv), 256, 0, s>>>(nv, z->row_ptr, z->col, z->bnd, xyz, u, (double*)B);
    else
        k_mcf_init_b<float><<<grid_for(nv), 256, 0, s>>>(nv, z->row_ptr, z->col, z->bnd, xyz, u, (float*)B);
    RXG_CUDA_TRY(cudaGetLastError());
    return RXG_OK;
}

rxg_status rxg_mcf_solve_matfree(const rxg_mesh* h, double dt, int32_t flags, int32_t dtype,
                                 const double* xyz, const void* B, void* X,
                                 const rxg_solver_opts* opts, rxg_solver_stats* stats, void* stream)
{
    if (!h || !xyz || !B || !X || !opts || opts->max_iter < 0 ||
        (dtype != RXG_F32 && dtype != RXG_F64) || (flags & ~RXG_MCF_UNIFORM_LAPLACE)) {
        set_error("rxg_mcf_solve_matfree: bad argument");
        return RXG_ERR_INVALID;
    }
    if (!is_device_ptr(xyz) || !is_device_ptr(B) || !is_device_ptr(X)) {
        set_error("rxg_mcf_solve_matfree: xyz, B and X must be device arrays");
        return RXG_ERR_INVALID;
    }
    Lazy*        z;
    cudaStream_t s  = S_(stream);
    rxg_status   st = ensure_pattern(&h->m, s, &z);
    if (st) return st;
    const int64_t    n  = h->m.nv;
    const bool       pc = opts->precond != 0;
    MatFreeOp        mf;
    mf.bnd     = z->bnd;
    mf.xyz     = xyz;
    mf.dt      = dt;
    mf.uniform = (flags & RXG_MCF_UNIFORM_LAPLACE) ? 1 : 0;
    rxg_solver_stats local;
    uint8_t*         scratch = nullptr;
    if (dtype == RXG_F64) {
        const int G = pc ? cg_grid<double, 3, true, true>(n) : cg_grid<double, 3, false, true>(n);
        RXG_CUDA_TRY(scratch_alloc((void**)&scratch, cg_scratch_bytes<double>(n, 3, G), s));
        st = pc ? cg_launch<double, 3, true, true>(n, z->nnz, z->row_ptr, z->col, nullptr, (const double*)B,
                                                   (double*)X, *opts, &local, scratch, s, mf)
                : cg_launch<double, 3, false, true>(n, z->nnz, z->row_ptr, z->col, nullptr, (const double*)B,
                                                    (double*)X, *opts, &local, scratch, s, mf);
    } else {
        const int    G  = pc ? cg_grid<float, 3, true, true>(n) : cg_grid<float, 3, false, true>(n);
        const size_t sb = cg_scratch_bytes<float>(n, 3, G);
        // the CG scratch, then the positions rounded to FP32 once per solve
        RXG_CUDA_TRY(scratch_alloc((void**)&scratch, sb + sizeof(float) * 3 * (size_t)n, s));
        float* xf = reinterpret_cast<float*>(scratch + sb);
        k_round_f32<<<grid_for(3 * n), 256, 0, s>>>(3 * n, xyz, xf);
        RXG_CUDA_TRY(cudaGetLastError());
        mf.xyzf = xf;
        st = pc ? cg_launch<float, 3, true, true>(n, z->nnz, z->row_ptr, z->col, nullptr, (const float*)B,
                                                  (float*)X, *opts, &local, scratch, s, mf)
                : cg_launch<float, 3, false, true>(n, z->nnz, z->row_ptr, z->col, nullptr, (const float*)B,
                                                   (float*)X, *opts, &local, scratch, s, mf);
    }
    cudaFreeAsync(scratch, s);
    if (st) return st;
    if (stats) *stats = local;
    return local.converged ? RXG_OK : RXG_ERR_NOT_CONVERGED;
}

rxg_status rxg_mcf_step_matfree(const rxg_mesh* h, double dt, int32_t nsteps, int32_t flags, double tol,
                                int32_t max_iter, double* xyz, rxg_solver_stats* stats, void* stream)
{
    if (!h || !xyz || nsteps < 0 || max_iter <= 0 || !(tol > 0) || (flags & ~RXG_MCF_UNIFORM_LAPLACE)) {
        set_error("rxg_mcf_step_matfree: bad argument");
        return RXG_ERR_INVALID;
    }
    if (!is_device_ptr(xyz)) {
        set_error("rxg_mcf_step_matfree: xyz must be a device array");
        return RXG_ERR_INVALID;
    }
    cudaStream_t  s  = S_(stream);
    const int64_t n  = h->m.nv;
    double*       xb = nullptr;  // positions of the step's operator, then B
    RXG_CUDA_TRY(scratch_alloc((void**)&xb, 2 * sizeof(double) * 3 * n, s));
    double*         Bv = xb + 3 * n;
    rxg_solver_opts o;
    o.max_iter = max_iter;
    o.abs_tol  = 0.0;
    o.rel_tol  = tol * tol;  // on r.D^-1 r, as rxg_mcf_step
    o.precond  = 1;
    rxg_status       st = RXG_OK;
    rxg_solver_stats local{};
    for (int32_t k = 0; k < nsteps && st == RXG_OK; ++k) {
        if (cudaMemcpyAsync(xb, xyz, sizeof(double) * 3 * n, cudaMemcpyDeviceToDevice, s) != cudaSuccess) {
            st = cuda_status(cudaGetLastError(), "cudaMemcpyAsync");
            break;
        }
        if ((st = rxg_mcf_init_b(h, flags, RXG_F64, xb, Bv, s))) break;
        st = rxg_mcf_solve_matfree(h, dt, flags, RXG_F64, xb, Bv, xyz, &o, &local, s);
    }
    cudaFreeAsync(xb, s);
    if (stats) *stats = local;
    return st;
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
    if (!is_device_ptr(B) || !is_device_ptr(X) || !is_device_ptr(A->val) ||
        !is_device_ptr(A->row_ptr) || !is_device_ptr(A->col)) {
        set_error("rxg_cg_solve_noalloc: A (row_ptr, col, val), B and X must be device arrays");
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
        st = cg_dispatch<double>(nc, A->n, A->nnz, A->row_ptr, A->col, (const double*)A->val,
                                 (const double*)B, (double*)X, *opts, &local, scratch, s);
    else
        st = cg_dispatch<float>(nc, A->n, A->nnz, A->row_ptr, A->col, (const float*)A->val,
                                (const float*)B, (float*)X, *opts, &local, scratch, s);
    if (st) return st;
    if (stats) *stats = local;
    return local.converged ? RXG_OK : RXG_ERR_NOT_CONVERGED;
}

// ---------------------------------------------------------------------
// Adjoint of one implicit MCF step.
//
// Forward: A(x) x1 = B(x), A = 2 diag(area) + dt L(w), B = 2 diag(area) x
// (mcf_A_setup / mcf_B_setup).  For a loss l with gbar = dl/dx1:
//   lambda = A^{-T} gbar = A^{-1} gbar          (A is symmetric: one more PCG)
//   dl/dA_ij = -lambda_i . x1_j,  dl/dB_i = lambda_i
// and with row p's area a_p and weights w_pr:
//   dl/da_p  = 2 lambda_p . (x_p - x1_p)
//   dl/dw_pr = dt lambda_p . (x1_r - x1_p)      (times the max(w,0) gate)
//   dl/dx_p += 2 a_p lambda_p                   (B's explicit x)
// The weight and area derivatives come from forward-mode duals run through
// the same half_cot / voronoi code as the assembly, so clamps and obtuse
// branches are differentiated exactly as evaluated.
// ---------------------------------------------------------------------

namespace rxg {

struct Dual9
{
    double v;
    double d[9];
    __device__ Dual9() : v(0)
    {
#pragma unroll
        for (int i = 0; i < 9; ++i) d[i] = 0;
    }
    __device__ Dual9(double x) : v(x)
    {
#pragma unroll
        for (int i = 0; i < 9; ++i) d[i] = 0;
    }
};
__device__ __forceinline__ Dual9 operator+(const Dual9& a, const Dual9& b)
{
    Dual9 r(a.v + b.v);
#pragma unroll
    for (int i = 0; i < 9; ++i) r.d[i] = a.d[i] + b.d[i];
    return r;
}
__device__ __forceinline__ Dual9 operator-(const Dual9& a, const Dual9& b)
{
    Dual9 r(a.v - b.v);
#pragma unroll
    for (int i = 0; i < 9; ++i) r.d[i] = a.d[i] - b.d[i];
    return r;
}
__device__ __forceinline__ Dual9 operator-(const Dual9& a)
{
    Dual9 r(-a.v);
#pragma unroll
    for (int i = 0; i < 9; ++i) r.d[i] = -a.d[i];
    return r;
}
__device__ __forceinline__ Dual9 operator*(const Dual9& a, const Dual9& b)
{
    Dual9 r(a.v * b.v);
#pragma unroll
    for (int i = 0; i < 9; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
    return r;
}
__device__ __forceinline__ Dual9 operator/(const Dual9& a, const Dual9& b)
{
    const double iv = 1.0 / b.v;
    Dual9        r(a.v * iv);
#pragma unroll
    for (int i = 0; i < 9; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * iv;
    return r;
}
__device__ __forceinline__ Dual9& operator+=(Dual9& a, const Dual9& b) { return a = a + b; }
__device__ __forceinline__ Dual9 sqrt(const Dual9& a)
{
    const double s = ::sqrt(a.v);
    Dual9        r(s);
    const double h = s > 0 ? 0.5 / s : 0.0;
#pragma unroll
    for (int i = 0; i < 9; ++i) r.d[i] = a.d[i] * h;
    return r;
}
// x^(-1/2), derivative -x^(-3/2) / 2
__device__ __forceinline__ Dual9 inv_sqrt(const Dual9& a)
{
    const double s = ::rsqrt(a.v);
    Dual9        r(s);
    const double h = -0.5 * s * s * s;
#pragma unroll
    for (int i = 0; i < 9; ++i) r.d[i] = a.d[i] * h;
    return r;
}
__device__ __forceinline__ bool operator<(const Dual9& a, const Dual9& b) { return a.v < b.v; }
__device__ __forceinline__ bool operator>(const Dual9& a, const Dual9& b) { return a.v > b.v; }
__device__ __forceinline__ bool operator<=(const Dual9& a, const Dual9& b) { return a.v <= b.v; }
__device__ __forceinline__ bool operator>=(const Dual9& a, const Dual9& b) { return a.v >= b.v; }
template <>
__device__ __forceinline__ Dual9 tmin<Dual9>()
{
    return Dual9(DBL_MIN);
}

// seeded dual vertex: tangent slots 3*slot .. 3*slot+2
__device__ __forceinline__ V3<Dual9> seed3(V3<double> a, int slot)
{
    V3<Dual9> r{Dual9(a.x), Dual9(a.y), Dual9(a.z)};
    r.x.d[3 * slot]     = 1.0;
    r.y.d[3 * slot + 1] = 1.0;
    r.z.d[3 * slot + 2] = 1.0;
    return r;
}

// add c * (derivative slots 3*slot .. 3*slot+2 of f) to a 3-vector
__device__ __forceinline__ void axpy3(double* acc, const Dual9& f, int slot, double c)
{
    acc[0] += c * f.d[3 * slot + 0];
    acc[1] += c * f.d[3 * slot + 1];
    acc[2] += c * f.d[3 * slot + 2];
}

// Per vertex p, the derivative of  lam_p . ((A x1 - B)_p)  with respect to
// the positions x (A, B assembled from x): each fan triangle T_t = (p, r_t,
// r_t+1) is evaluated once with 9 dual tangents (tri_terms: its two
// half-cotangents and its Voronoi term, bit for bit the values of the
// separate per-entry calls), and its three derivative rows are combined with
// their coefficients -- dt lam_p . (x1_r - x1_p) for the half-cotangent of
// each edge whose (unclamped) weight is >= 0, 2 lam_p . (x_p - x1_p) for a
// positive Voronoi term -- before one scatter to r_t and r_t+1; p's own
// share is summed in registers.  g_in must be zero on entry.
__global__ void __launch_bounds__(128) k_mcf_backward(int64_t nv, const int32_t* __restrict__ row_ptr,
                                                      const int32_t* __restrict__ col,
                                                      const int8_t* __restrict__ bnd,
                                                      const double* __restrict__ x,
                                                      const double* __restrict__ x1,
                                                      const double* __restrict__ lam, double dt,
                                                      double* __restrict__ g_in)
{
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nv;
         p += (int64_t)gridDim.x * blockDim.x) {
        const int32_t    rp   = row_ptr[p];
        const int32_t    k    = row_ptr[p + 1] - rp - 1;
        const int32_t*   rg   = col + rp + 1;
        const bool       wrap = bnd[p] == 0;
        const V3<double> P    = ld3(x, (int32_t)p);
        const V3<double> L    = ld3(lam, (int32_t)p);
        const V3<double> Y    = ld3(x1, (int32_t)p);
        const double     ap   = 2.0 * (L.x * (P.x - Y.x) + L.y * (P.y - Y.y) + L.z * (P.z - Y.z));
        double           area = 0.0, gp[3] = {0.0, 0.0, 0.0};
        // fan triangles: t = 0 .. nt-1, T_t = (p, r_t, r_(t+1) mod k); an
        // open fan has no T_(k-1)
        const int32_t nt   = k <= 0 ? 0 : (wrap ? k : k - 1);
        auto          beta = [&](int32_t i) {
            const V3<double> Yr = ld3(x1, rg[i]);
            return dt * (L.x * (Yr.x - Y.x) + L.y * (Yr.y - Y.y) + L.z * (Yr.z - Y.z));
        };
        auto tv = [&](int32_t t) {  // value-only terms of T_t
            return tri_terms<double>(P, ld3(x, rg[t]), ld3(x, rg[t + 1 < k ? t + 1 : 0]));
        };
        if (nt > 0) {
            // weight of edge p - r_0: hb of the closing triangle (closed
            // fans) + ha of T_0
            const TriTerms<double> t0 = tv(0);
            double       hb_prev = wrap ? tv(k - 1).hb : 0.0;
            double       w_cur   = hb_prev + t0.ha;
            double       b_cur   = beta(0);
            const double w0 = w_cur, b0 = b_cur;
            double       ha_next = t0.ha;
            for (int32_t t = 0; t < nt; ++t) {
                const int32_t  a = rg[t], bi = t + 1 < k ? t + 1 : 0, b = rg[bi];
                const TriTerms<Dual9> D =
                    tri_terms<Dual9>(seed3(P, 0), seed3(ld3(x, a), 1), seed3(ld3(x, b), 2));
                // the next edge's weight and coefficient
                double w_next, b_next;
                if (t + 1 < k) {
                    ha_next = (t + 1 < nt) ? tv(t + 1).ha : 0.0;
                    w_next  = D.hb.v + ha_next;
                    b_next  = beta(t + 1);
                } else {  // closing triangle: the next edge is p - r_0
                    w_next = w0;
                    b_next = b0;
                }
                const double c_ha = (w_cur >= 0.0 && b_cur != 0.0) ? b_cur : 0.0;
                const double c_hb = (w_next >= 0.0 && b_next != 0.0) ? b_next : 0.0;
                const double c_va = D.va.v > 0.0 ? ap : 0.0;
                if (D.va.v > 0.0) area += D.va.v;
                double gr[3] = {0.0, 0.0, 0.0}, gs[3] = {0.0, 0.0, 0.0};
                axpy3(gp, D.ha, 0, c_ha), axpy3(gp, D.hb, 0, c_hb), axpy3(gp, D.va, 0, c_va);
                axpy3(gr, D.ha, 1, c_ha), axpy3(gr, D.hb, 1, c_hb), axpy3(gr, D.va, 1, c_va);
                axpy3(gs, D.ha, 2, c_ha), axpy3(gs, D.hb, 2, c_hb), axpy3(gs, D.va, 2, c_va);
                if (c_ha != 0.0 || c_hb != 0.0 || c_va != 0.0) {
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        atomicAdd(g_in + 3 * (int64_t)a + c, gr[c]);
                        atomicAdd(g_in + 3 * (int64_t)b + c, gs[c]);
                    }
                }
                w_cur = w_next;
                b_cur = b_next;
            }
        }
        atomicAdd(g_in + 3 * p + 0, gp[0] + 2.0 * area * L.x);
        atomicAdd(g_in + 3 * p + 1, gp[1] + 2.0 * area * L.y);
        atomicAdd(g_in + 3 * p + 2, gp[2] + 2.0 * area * L.z);
    }
}

}  // namespace rxg

extern "C" rxg_status rxg_mcf_step_backward(const rxg_mesh* h, double dt, const double* x_in,
                                            const double* x_out, const double* g_out,
                                            double* g_in, double tol, int32_t max_iter,
                                            rxg_solver_stats* stats, void* stream)
{
    using namespace rxg;
    if (!h || !x_in || !x_out || !g_out || !g_in || !(tol > 0) || max_iter <= 0) {
        set_error("rxg_mcf_step_backward: bad argument");
        return RXG_ERR_INVALID;
    }
    if (!is_device_ptr(x_in) || !is_device_ptr(x_out) || !is_device_ptr(g_out) || !is_device_ptr(g_in)) {
        set_error("rxg_mcf_step_backward: all arrays must be device arrays");
        return RXG_ERR_INVALID;
    }
    cudaStream_t s = (cudaStream_t)stream;
    Lazy*        z;
    rxg_status   st = ensure_pattern(&h->m, s, &z);
    if (st) return st;
    const int64_t n = h->m.nv, nnz = z->nnz;
    // the adjoint system is the forward step's (A symmetric): the same packed
    // assembly and persistent FP64 Jacobi-PCG (k_cgm) as rxg_mcf_step
    const size_t x4b  = align256(sizeof(R4<double>) * n);
    const size_t entb = align256(sizeof(Ent<double>) * nnz);
    const size_t need = entb + 2 * x4b + align256(24 * n) + cgm_scratch_bytes<double>(n, cgm_grid<double>(n));
    {
        std::lock_guard<std::mutex> g(z->mu);
        if ((st = mcf_buffers(z, need, s))) return st;
    }
    uint8_t*     q   = (uint8_t*)z->buf;
    Ent<double>* ent = (Ent<double>*)q;
    R4<double>*  B4  = (R4<double>*)(q + entb);
    R4<double>*  L4  = (R4<double>*)(q + entb + x4b);
    double*      lam = (double*)(q + entb + 2 * x4b);
    uint8_t*     scr = q + entb + 2 * x4b + align256(24 * n);
    const int    ga  = grid_for(n);
    const auto   ka  = k_mcf_assemble<double, Geo<double>, double, PackedOut<double, double>>;
    // (the assembly's right-hand side lands in B4 and is replaced by g_out)
    ka<<<whole_wave_grid(ka, n, 256), 256, 0, s>>>(n, z->row_ptr, z->col, z->bnd, x_in, dt,
                                                 PackedOut<double, double>{ent, B4, nullptr});
    RXG_CUDA_TRY(cudaGetLastError());
    k_pack3<<<ga, 256, 0, s>>>(n, g_out, B4);
    RXG_CUDA_TRY(cudaMemsetAsync(L4, 0, sizeof(R4<double>) * n, s));
    rxg_solver_opts  o = {max_iter, 0.0, tol * tol, 1};
    rxg_solver_stats local;
    st = cgm_launch<double>(n, z->row_ptr, ent, B4, L4, o, &local, scr, s);
    if (st) return st;
    k_unpack3<<<ga, 256, 0, s>>>(n, L4, lam);
    RXG_CUDA_TRY(cudaMemsetAsync(g_in, 0, 24 * n, s));
    k_mcf_backward<<<grid_for(n, 128), 128, 0, s>>>(n, z->row_ptr, z->col, z->bnd, x_in, x_out, lam,
                                                     dt, g_in);
    RXG_CUDA_TRY(cudaGetLastError());
    if (stats) *stats = local;
    return local.converged ? RXG_OK : RXG_ERR_NOT_CONVERGED;
}
