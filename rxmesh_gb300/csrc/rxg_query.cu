// Patch-parallel query kernels: VV, VE, VF, FV, EV and vertex normals.
//
// One CTA per patch (RXMesh's launch shape, rxmesh_static.inl:443-496).  The
// CTA stages its patch's EV / FE slices and ribbon tables into shared memory
// with TMA bulk copies (cp.async.bulk + mbarrier), builds the vertex-centred
// transposes there (the counting sort of block_mat_transpose,
// kernels/rxmesh_queries.cuh:17-107), resolves not-owned elements through the
// dense ribbon table (in place of the LP hashtable lookup of
// iterator.cuh:117-143) and writes its owned rows as one contiguous chunk of
// the global CSR with 16-byte stores.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <mutex>

#include "rxg_device.cuh"

namespace rxg {


__device__ int g_err_word;

// The error word's device address on the current device.  Every GPU that
// loads the library has its own copy of g_err_word, so the address is looked
// up once per device ordinal (with that device current) and cached.
int* device_error_word()
{
    static std::mutex mu;
    static int*       addr[kMaxDevices] = {nullptr};
    int               dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return nullptr;
    std::lock_guard<std::mutex> g(mu);
    if (!addr[dev] && cudaGetSymbolAddress((void**)&addr[dev], g_err_word) != cudaSuccess) {
        cudaGetLastError();
        addr[dev] = nullptr;
    }
    return addr[dev];
}

int device_sm_count()
{
    static std::mutex mu;
    static int        sms[kMaxDevices] = {0};
    int               dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return 1;
    std::lock_guard<std::mutex> g(mu);
    if (!sms[dev]) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
            cudaGetLastError();
            n = 0;
        }
        sms[dev] = n > 0 ? n : 1;
    }
    return sms[dev];
}

int current_device()
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return 0;
    return dev;
}

rxg_status check_device_error(cudaStream_t s)
{
    int* d = device_error_word();
    int  h = 0;
    if (!d) {
        set_error("device error word: no current CUDA device (or ordinal beyond %d)", kMaxDevices - 1);
        return RXG_ERR_NO_DEVICE;
    }
    RXG_CUDA_TRY(cudaMemcpyAsync(&h, d, sizeof(int), cudaMemcpyDeviceToHost, s));
    RXG_CUDA_TRY(cudaStreamSynchronize(s));
    if (h) {
        int zero = 0;
        cudaMemcpy(d, &zero, sizeof(int), cudaMemcpyHostToDevice);
        if (h & DEVERR_MBAR_TIMEOUT) {
            set_error("a bounded mbarrier wait timed out on the device (code %d)", h);
            return RXG_ERR_DEVICE_TIMEOUT;
        }
        if (h & DEVERR_GRID_TIMEOUT) {
            set_error("a bounded grid barrier timed out on the device (code %d)", h);
            return RXG_ERR_DEVICE_TIMEOUT;
        }
        if (h & DEVERR_NONMANIFOLD) {
            set_error("a vertex fan is not a disk or half-disk (non-manifold vertex)");
            return RXG_ERR_NONMANIFOLD;
        }
        set_error("device error word %d", h);
        return RXG_ERR_CUDA;
    }
    return RXG_OK;
}

// ---------------------------------------------------------------------
// staging
// ---------------------------------------------------------------------

// Warp 0 waits on the barrier phase (bounded); the other warps wait at the
// CTA barrier and so spend no issue slots.  The CTA barrier orders the
// completed bulk copies before every thread's reads.
__device__ __forceinline__ bool wait_stage(uint64_t* bar, int* err)
{
    __shared__ int s_ok;
    if (threadIdx.x < 32) {
        bool ok = mbar_wait_hinted(bar, 0, err);
        if (threadIdx.x == 0) s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

struct Slice
{
    const uint32_t* src;
    uint32_t        bytes;
};

// thread 0 arms the barrier and issues up to 4 bulk copies; everybody waits.
// Shared destinations must be 16-byte aligned.
template <int N>
__device__ __forceinline__ bool stage(uint64_t* bar, uint32_t* const (&dst)[N],
                                      const Slice (&sl)[N], int* err)
{
    if (threadIdx.x == 0) {
        uint32_t total = 0;
#pragma unroll
        for (int i = 0; i < N; ++i) total += sl[i].bytes;
        mbar_arrive_expect_tx(bar, total);
#pragma unroll
        for (int i = 0; i < N; ++i)
            if (sl[i].bytes) bulk_g2s(dst[i], sl[i].src, sl[i].bytes, bar);
    }
    return wait_stage(bar, err);
}

__device__ __forceinline__ PatchHdr load_hdr(const PatchHdr* __restrict__ hdrs)
{
    const int4* p = reinterpret_cast<const int4*>(hdrs + blockIdx.x);
    PatchHdr    h;
    int4*       q = reinterpret_cast<int4*>(&h);
#pragma unroll
    for (int i = 0; i < 4; ++i) q[i] = __ldg(p + i);
    return h;
}

__host__ __device__ __forceinline__ uint32_t fe_words(int32_t nF) { return (uint32_t)((3 * nF + 1) / 2); }

// vertex k (0..2) of local face f from FE (edge<<1|dir) and EV (a | b<<16)
__device__ __forceinline__ uint32_t face_vertex(const uint16_t* s_fe, const uint32_t* s_ev, int f,
                                                int k)
{
    uint32_t fe = s_fe[3 * f + k];
    uint32_t ev = s_ev[fe >> 1];
    return (fe & 1u) ? (ev >> 16) : (ev & 0xffffu);
}

// ---------------------------------------------------------------------
// VV / VE  (OP 0 / 1) and VF (OP 2): vertex-centred transposes
// ---------------------------------------------------------------------

// EF (OP 5) is the same transpose with rows = owned edges: every local
// face adds itself to the rows of its owned edges.  qb: first EF value of
// each patch's rows (indexed like hdrs; unused by the other ops).
//
// The count and scatter passes are branch-free: an incidence of an element
// the patch does not own goes to one of 32 spill counters behind the rows
// (one per lane, so a warp's spills do not contend), whose positions are
// never stored; the row offsets are written by the scan's last pass.  This
// form issued 11% fewer instructions than one with a branch per incidence.
constexpr int kSpill = 32;

// words of VF's first shared region: the EV slice, later the staged rows
// (3 u16 per local face + 4 words of alignment slack)
__host__ __device__ __forceinline__ int32_t vf_ev_words(const PatchHdr& h)
{
    const int32_t out_w = (3 * h.nFl + 1) / 2 + 4;
    return pad4i(h.nEl > out_w ? h.nEl : out_w);
}
template <int OP, int kQT>
__global__ void __launch_bounds__(kQT) k_query_vertex(const PatchHdr* __restrict__ hdrs,
                                                      const uint32_t* __restrict__ arena,
                                                      int32_t* __restrict__ out_off,
                                                      int32_t* __restrict__ out_val, int* err,
                                                      const int32_t* __restrict__ qb)
{
    extern __shared__ __align__(16) uint32_t smem[];
    __shared__ uint64_t bar;
    __shared__ int32_t  s_warp[kQT / 32];

    constexpr bool EF  = OP == RXG_OP_EF;
    constexpr bool FCE = OP == 2 || EF;  // walks the local faces
    const PatchHdr h   = load_hdr(hdrs);
    const int32_t  nVo = h.nVo;
    const int32_t  nRows = EF ? h.nEo : nVo;
    const int32_t  nRib = OP == 0 ? h.nVl - h.nVo : (OP == 1 ? h.nEl - h.nEo : h.nFl - h.nFo);
    const int32_t  ribOff = OP == 0 ? h.rv_off : (OP == 1 ? h.re_off : h.rf_off);

    // shared layout (all 16-byte aligned); the patch's rows are staged as
    // 16-bit local ids and mapped to linear ids on the way out
    // VF: the staged rows overlay the EV slice, which only the count pass
    // reads (it leaves each face's corners in place of its FE entries), so
    // the region is the larger of the two
    constexpr bool VF = OP == 2;
    const int32_t  ev_w  = EF ? 0 : (VF ? vf_ev_words(h) : pad4i(h.nEl));
    uint32_t*      s_ev  = smem;
    uint32_t*      s_fe  = s_ev + ev_w;
    uint32_t*      s_rib = s_fe + (FCE ? pad4i((int32_t)fe_words(h.nFl)) : 0);
    int32_t*       s_cnt = reinterpret_cast<int32_t*>(s_rib + pad4i(nRib));
    uint16_t*      s_out = VF ? reinterpret_cast<uint16_t*>(smem)
                              : reinterpret_cast<uint16_t*>(s_cnt + pad4i(nRows + 1 + kSpill));
    const int32_t spill = nRows + 1 + (int32_t)(threadIdx.x & 31);
    // counter of row r, or this lane's spill counter for r >= nRows
    auto slot = [&](uint32_t r) -> int32_t* { return &s_cnt[(int32_t)r < nRows ? (int32_t)r : spill]; };

    if (threadIdx.x == 0) mbar_init(&bar, 1);
    for (int i = threadIdx.x; i < nRows + 1 + kSpill; i += kQT) s_cnt[i] = 0;
    __syncthreads();

    bool ok;
    if (EF) {
        uint32_t* const dst[2] = {s_fe, s_rib};
        const Slice     sl[2]  = {{arena + h.fe_off, pad16_bytes((int32_t)fe_words(h.nFl))},
                                  {arena + ribOff, pad16_bytes(nRib)}};
        ok = stage(&bar, dst, sl, err);
    } else if (OP == 2) {
        uint32_t* const dst[3] = {s_ev, s_fe, s_rib};
        const Slice     sl[3]  = {{arena + h.ev_off, pad16_bytes(h.nEl)},
                                  {arena + h.fe_off, pad16_bytes((int32_t)fe_words(h.nFl))},
                                  {arena + ribOff, pad16_bytes(nRib)}};
        ok = stage(&bar, dst, sl, err);
    } else {
        uint32_t* const dst[2] = {s_ev, s_rib};
        const Slice     sl[2]  = {{arena + h.ev_off, pad16_bytes(h.nEl)},
                                  {arena + ribOff, pad16_bytes(nRib)}};
        ok = stage(&bar, dst, sl, err);
    }
    if (!ok) return;

    const uint16_t* fe16 = reinterpret_cast<const uint16_t*>(s_fe);
    const uint2*    ev2  = reinterpret_cast<const uint2*>(s_ev);  // two edges per load
    const int32_t   nE2  = (h.nEl + 1) >> 1;

    // 1. count owned-vertex (EF: owned-edge) incidences (nRows = nVo for
    // the vertex ops)
    if (EF) {
        for (int f = threadIdx.x; f < h.nFl; f += kQT) {
#pragma unroll
            for (int k = 0; k < 3; ++k) atomicAdd(slot((uint32_t)fe16[3 * f + k] >> 1), 1);
        }
    } else if (OP == 2) {
        // each thread resolves its faces' corners once and leaves them in
        // place of the faces' FE entries (the local FV the scatter reads)
        uint16_t* fv16 = reinterpret_cast<uint16_t*>(s_fe);
        for (int f = threadIdx.x; f < h.nFl; f += kQT) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const uint32_t v = face_vertex(fe16, s_ev, f, k);
                fv16[3 * f + k]  = (uint16_t)v;
                atomicAdd(slot(v), 1);
            }
        }
    } else {
        for (int e2 = threadIdx.x; e2 < nE2; e2 += kQT) {
            const uint2    w  = ev2[e2];
            const bool     hi = 2 * e2 + 1 < h.nEl;
            const uint32_t a0 = w.x & 0xffffu, b0 = w.x >> 16;
            const uint32_t a1 = hi ? w.y & 0xffffu : 0xffffu, b1 = hi ? w.y >> 16 : 0xffffu;
            atomicAdd(slot(a0), 1);
            atomicAdd(slot(b0), 1);
            atomicAdd(slot(a1), 1);
            atomicAdd(slot(b1), 1);
        }
    }
    __syncthreads();

    // 2. exclusive scan -> row offsets of the patch's owned rows, written
    // to the global offsets by the scan's last pass
    const int32_t vbase   = EF ? __ldg(qb + blockIdx.x) : (OP == 2 ? h.vf_base : h.vv_base);
    const int32_t rowbase = EF ? h.e_base : h.v_base;
    const int32_t total   = block_exclusive_scan<kQT>(s_cnt, nRows + 1, s_warp, out_off + rowbase, vbase);

    // 3. scatter 16-bit local ids into the staged chunk
    uint16_t* sbuf = s_out + (vbase & 3);  // element g lives at s_out[g - (vbase & ~3)]
    if (EF) {
        for (int f = threadIdx.x; f < h.nFl; f += kQT) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const uint32_t e = (uint32_t)fe16[3 * f + k] >> 1;
                const int32_t  q = atomicAdd(slot(e), 1);
                if ((int32_t)e < nRows) sbuf[q] = (uint16_t)f;
            }
        }
    } else if (OP == 2) {
        for (int f = threadIdx.x; f < h.nFl; f += kQT) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const uint32_t v = fe16[3 * f + k];  // local FV, written by the count
                const int32_t  q = atomicAdd(slot(v), 1);
                if ((int32_t)v < nVo) sbuf[q] = (uint16_t)f;
            }
        }
    } else {
        for (int e2 = threadIdx.x; e2 < nE2; e2 += kQT) {
            const uint2    w  = ev2[e2];
            const bool     hi = 2 * e2 + 1 < h.nEl;
            const uint32_t a0 = w.x & 0xffffu, b0 = w.x >> 16;
            const uint32_t a1 = hi ? w.y & 0xffffu : 0xffffu, b1 = hi ? w.y >> 16 : 0xffffu;
            const uint16_t e0 = (uint16_t)(2 * e2), e1 = (uint16_t)(2 * e2 + 1);
            const int32_t  q0 = atomicAdd(slot(a0), 1), q1 = atomicAdd(slot(b0), 1);
            const int32_t  q2 = atomicAdd(slot(a1), 1), q3 = atomicAdd(slot(b1), 1);
            if ((int32_t)a0 < nVo) sbuf[q0] = OP == 0 ? (uint16_t)b0 : e0;
            if ((int32_t)b0 < nVo) sbuf[q1] = OP == 0 ? (uint16_t)a0 : e0;
            if ((int32_t)a1 < nVo) sbuf[q2] = OP == 0 ? (uint16_t)b1 : e1;
            if ((int32_t)b1 < nVo) sbuf[q3] = OP == 0 ? (uint16_t)a1 : e1;
        }
    }
    __syncthreads();

    // 4. contiguous, vectorised write-out, local -> linear ids
    const int32_t   nOwn = OP == 0 ? nVo : (OP == 1 ? h.nEo : h.nFo);
    const int32_t   base = OP == 0 ? h.v_base : (OP == 1 ? h.e_base : h.f_base);  // VF, EF: faces
    const uint32_t* rib  = s_rib;
    store_u16_mapped<kQT>(out_val, vbase, s_out, total, [=](uint32_t loc) -> int32_t {
        return (int32_t)loc < nOwn ? base + (int32_t)loc : (int32_t)rib[loc - nOwn];
    });
}

// ---------------------------------------------------------------------
// FV (OP 3) and EV (OP 4): owned-element rows, one output word per thread
// ---------------------------------------------------------------------

template <int OP, int kQT>
__global__ void __launch_bounds__(kQT) k_query_elem(const PatchHdr* __restrict__ hdrs,
                                                    const uint32_t* __restrict__ arena,
                                                    int32_t* __restrict__ out_val, int* err)
{
    extern __shared__ __align__(16) uint32_t smem[];
    __shared__ uint64_t bar;

    constexpr bool FE = OP == RXG_OP_FE, EVD = OP == RXG_OP_EVD, EE = OP == RXG_OP_EE;
    const PatchHdr h   = load_hdr(hdrs);
    const int32_t  nVo = h.nVo;
    const int32_t  nVr = h.nVl - h.nVo;
    // FV needs every local edge an owned face uses, i.e. the whole EV slice;
    // EV needs only the owned prefix; FE needs no EV; EVD needs the whole
    // EV slice and every local face (the faces of the owned edges); EE
    // needs every local face and no EV.
    const int32_t ev_words = (OP == 3 || EVD) ? h.nEl : ((FE || EE) ? 0 : h.nEo);
    const int32_t fe_w     = (EVD || EE) ? (int32_t)fe_words(h.nFl)
                                         : ((OP == 3 || FE) ? (int32_t)fe_words(h.nFo) : 0);
    // ribbon table of the output ids: vertices, or edges for FE and EE
    const int32_t rib_n   = (FE || EE) ? h.nEl - h.nEo : nVr;
    const int32_t rib_off = (FE || EE) ? h.re_off : h.rv_off;

    uint32_t* s_ev = smem;
    uint32_t* s_fe = s_ev + pad4i(ev_words);
    uint32_t* s_rv = s_fe + pad4i(fe_w);

    if (threadIdx.x == 0) mbar_init(&bar, 1);
    __syncthreads();
    uint32_t* const dst[3] = {s_ev, s_fe, s_rv};
    const Slice     sl[3]  = {{arena + h.ev_off, pad16_bytes(ev_words)},
                              {arena + h.fe_off, pad16_bytes(fe_w)},
                              {arena + rib_off, pad16_bytes(rib_n)}};
    if (!stage(&bar, dst, sl, err)) return;

    const uint16_t* fe16 = reinterpret_cast<const uint16_t*>(s_fe);
    if (FE) {
        // edge k of face f runs from corner k to corner k+1 (FE order)
        const int32_t n    = 3 * h.nFo;
        int32_t*      base = out_val + 3 * (int64_t)h.f_base;
        for (int i = threadIdx.x; i < n; i += kQT) {
            const uint32_t e = (uint32_t)fe16[i] >> 1;
            base[i] = (int32_t)e < h.nEo ? h.e_base + (int32_t)e : (int32_t)s_rv[e - h.nEo];
        }
    } else if (EVD) {
        // four 16-bit slots per owned edge: v0, opposite vertex in the face
        // traversing v0->v1, v1, opposite vertex in the face traversing
        // v1->v0 (0xffff: no such face).  Local ids fit 16 bits with 0xffff
        // to spare (at most 65,535 local vertices).
        uint2* slot = reinterpret_cast<uint2*>(s_rv + pad4i(nVr));  // one per owned edge
        for (int e = threadIdx.x; e < h.nEo; e += kQT) {
            const uint32_t ev = s_ev[e];
            slot[e]           = make_uint2((ev & 0xffffu) | 0xffff0000u, (ev >> 16) | 0xffff0000u);
        }
        __syncthreads();
        // every local face names the vertex opposite each of its edges
        // (corner k+2 for edge k); on an edge-manifold mesh the two faces of
        // an edge traverse it in opposite directions, so each slot has one writer
        uint16_t* s16 = reinterpret_cast<uint16_t*>(slot);
        for (int f = threadIdx.x; f < h.nFl; f += kQT) {
            const uint32_t c[3] = {fe16[3 * f], fe16[3 * f + 1], fe16[3 * f + 2]};
            uint32_t       v[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const uint32_t ev = s_ev[c[k] >> 1];
                v[k]              = (c[k] & 1u) ? (ev >> 16) : (ev & 0xffffu);
            }
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const uint32_t e = c[k] >> 1;
                if ((int32_t)e < h.nEo) s16[4 * e + 1 + 2 * (c[k] & 1u)] = (uint16_t)v[(k + 2) % 3];
            }
        }
        __syncthreads();
        // one owned edge per thread: its four slots as one 16-byte store
        const int32_t vb   = h.v_base;
        auto          lin  = [=](uint32_t l) -> int32_t {
            return l == 0xffffu ? -1 : ((int32_t)l < nVo ? vb + (int32_t)l : (int32_t)s_rv[l - nVo]);
        };
        int4* base = reinterpret_cast<int4*>(out_val + 4 * (int64_t)h.e_base);
        for (int e = threadIdx.x; e < h.nEo; e += kQT) {
            const uint2 w = slot[e];
            base[e]       = make_int4(lin(w.x & 0xffffu), lin(w.x >> 16), lin(w.y & 0xffffu), lin(w.y >> 16));
        }
    } else if (EE) {
        // per owned edge two 32-bit slots of two 16-bit local edge ids: slot
        // d for the face traversing the edge from its vertex d (FE's
        // direction bit), holding that face's next and previous edge
        // (0xffff: no such face).  On an edge-manifold, consistently
        // oriented mesh each slot has one writer.
        uint32_t* slot = s_rv + pad4i(rib_n);
        for (int i = threadIdx.x; i < 2 * h.nEo; i += kQT) slot[i] = 0xffffffffu;
        __syncthreads();
        for (int f = threadIdx.x; f < h.nFl; f += kQT) {
            const uint32_t c[3] = {fe16[3 * f], fe16[3 * f + 1], fe16[3 * f + 2]};
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const uint32_t e = c[k] >> 1;
                if ((int32_t)e < h.nEo) slot[2 * e + (c[k] & 1u)] = (c[(k + 1) % 3] >> 1) | ((c[(k + 2) % 3] >> 1) << 16);
            }
        }
        __syncthreads();
        // one owned edge per thread: its four slots as one 16-byte store
        const int32_t eb  = h.e_base, nEo = h.nEo;
        auto          lin = [=](uint32_t l) -> int32_t {
            return l == 0xffffu ? -1 : ((int32_t)l < nEo ? eb + (int32_t)l : (int32_t)s_rv[l - nEo]);
        };
        const uint2* s2   = reinterpret_cast<const uint2*>(slot);
        int4*        base = reinterpret_cast<int4*>(out_val + 4 * (int64_t)h.e_base);
        for (int e = threadIdx.x; e < h.nEo; e += kQT) {
            const uint2 w = s2[e];
            base[e]       = make_int4(lin(w.x & 0xffffu), lin(w.x >> 16), lin(w.y & 0xffffu), lin(w.y >> 16));
        }
    } else if (OP == 3) {
        const int32_t n    = 3 * h.nFo;
        int32_t*      base = out_val + 3 * (int64_t)h.f_base;
        for (int i = threadIdx.x; i < n; i += kQT) {
            uint32_t v = face_vertex(fe16, s_ev, i / 3, i % 3);
            base[i]    = (int32_t)v < nVo ? h.v_base + (int32_t)v : (int32_t)s_rv[v - nVo];
        }
    } else {
        const int32_t n    = 2 * h.nEo;
        int32_t*      base = out_val + 2 * (int64_t)h.e_base;
        for (int i = threadIdx.x; i < n; i += kQT) {
            uint32_t ev = s_ev[i >> 1];
            uint32_t v  = (i & 1) ? (ev >> 16) : (ev & 0xffffu);
            base[i]     = (int32_t)v < nVo ? h.v_base + (int32_t)v : (int32_t)s_rv[v - nVo];
        }
    }
}

// ---------------------------------------------------------------------
// FF (OP 7): faces sharing an edge with each owned face.  Per patch: the
// local EF lists of every local edge (counting sort over the local faces,
// which include every edge neighbour of an owned face), then one thread per
// owned face walks its three edges' lists.  qb: first FF value of each
// patch's rows (indexed like hdrs).  Ground truth of
// tests/RXMesh_test/rxmesh_test.h:290-330.
// ---------------------------------------------------------------------

// FF on an edge-manifold, consistently oriented mesh: every edge has at most
// one face per traversal direction, so two 16-bit face slots per local edge
// (no atomics, no scan) give each owned face its neighbour across edge k in
// the slot of the opposite direction; rows list the neighbours in edge order.
template <int kQT>
__global__ void __launch_bounds__(kQT) k_query_ff_oriented(const PatchHdr* __restrict__ hdrs,
                                                           const uint32_t* __restrict__ arena,
                                                           int32_t* __restrict__ out_off,
                                                           int32_t* __restrict__ out_val,
                                                           int* err,
                                                           const int32_t* __restrict__ qb)
{
    extern __shared__ __align__(16) uint32_t smem[];
    __shared__ uint64_t bar;
    __shared__ int32_t  s_warp[kQT / 32];

    const PatchHdr h   = load_hdr(hdrs);
    const int32_t  nFo = h.nFo, nFl = h.nFl, nEl = h.nEl;
    const int32_t  nFr = nFl - nFo;
    uint32_t* s_fe   = smem;
    uint32_t* s_rf   = s_fe + pad4i((int32_t)fe_words(nFl));
    uint32_t* s_slot = s_rf + pad4i(nFr);                                      // nEl words
    int32_t*  s_fc   = reinterpret_cast<int32_t*>(s_slot + pad4i(nEl));        // nFo+1
    uint16_t* s_out  = reinterpret_cast<uint16_t*>(s_fc + pad4i(nFo + 1));

    if (threadIdx.x == 0) mbar_init(&bar, 1);
    for (int i = threadIdx.x; i < nEl; i += kQT) s_slot[i] = 0xffffffffu;
    __syncthreads();
    uint32_t* const dst[2] = {s_fe, s_rf};
    const Slice     sl[2]  = {{arena + h.fe_off, pad16_bytes((int32_t)fe_words(nFl))},
                              {arena + h.rf_off, pad16_bytes(nFr)}};
    if (!stage(&bar, dst, sl, err)) return;
    const uint16_t* fe16 = reinterpret_cast<const uint16_t*>(s_fe);
    uint16_t*       slot = reinterpret_cast<uint16_t*>(s_slot);  // [2e + dir]

    for (int f = threadIdx.x; f < nFl; f += kQT) {
#pragma unroll
        for (int k = 0; k < 3; ++k) slot[fe16[3 * f + k]] = (uint16_t)f;
    }
    __syncthreads();
    for (int f = threadIdx.x; f < nFo; f += kQT) {
        int32_t c = 0;
#pragma unroll
        for (int k = 0; k < 3; ++k) c += slot[fe16[3 * f + k] ^ 1u] != 0xffffu;
        s_fc[f] = c;
    }
    if (threadIdx.x == 0) s_fc[nFo] = 0;
    __syncthreads();
    // row offsets written to the global offsets by the scan's last pass
    const int32_t vbase = __ldg(qb + blockIdx.x);
    const int32_t total = block_exclusive_scan<kQT>(s_fc, nFo + 1, s_warp, out_off + h.f_base, vbase);
    uint16_t* sbuf = s_out + (vbase & 3);
    for (int f = threadIdx.x; f < nFo; f += kQT) {
        int32_t pos = s_fc[f];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const uint16_t g = slot[fe16[3 * f + k] ^ 1u];
            if (g != 0xffffu) sbuf[pos++] = g;
        }
    }
    __syncthreads();
    const uint32_t* rf = s_rf;
    const int32_t   fb = h.f_base;
    store_u16_mapped<kQT>(out_val, vbase, s_out, total, [=](uint32_t loc) -> int32_t {
        return (int32_t)loc < nFo ? fb + (int32_t)loc : (int32_t)rf[loc - nFo];
    });
}

template <int kQT>
__global__ void __launch_bounds__(kQT) k_query_ff(const PatchHdr* __restrict__ hdrs,
                                                  const uint32_t* __restrict__ arena,
                                                  int32_t* __restrict__ out_off,
                                                  int32_t* __restrict__ out_val, int* err,
                                                  const int32_t* __restrict__ qb)
{
    extern __shared__ __align__(16) uint32_t smem[];
    __shared__ uint64_t bar;
    __shared__ int32_t  s_warp[kQT / 32];

    const PatchHdr h   = load_hdr(hdrs);
    const int32_t  nFo = h.nFo, nFl = h.nFl, nEl = h.nEl;
    const int32_t  nFr = nFl - nFo;
    uint32_t* s_fe  = smem;
    uint32_t* s_rf  = s_fe + pad4i((int32_t)fe_words(nFl));
    int32_t*  s_ec  = reinterpret_cast<int32_t*>(s_rf + pad4i(nFr));           // nEl+1
    uint16_t* s_ef  = reinterpret_cast<uint16_t*>(s_ec + pad4i(nEl + 1));       // 3 nFl
    int32_t*  s_fc  = reinterpret_cast<int32_t*>(s_ef) + pad4i((3 * nFl + 1) / 2);  // nFo+1
    uint16_t* s_out = reinterpret_cast<uint16_t*>(s_fc + pad4i(nFo + 1));

    if (threadIdx.x == 0) mbar_init(&bar, 1);
    for (int i = threadIdx.x; i <= nEl; i += kQT) s_ec[i] = 0;
    __syncthreads();
    uint32_t* const dst[2] = {s_fe, s_rf};
    const Slice     sl[2]  = {{arena + h.fe_off, pad16_bytes((int32_t)fe_words(nFl))},
                              {arena + h.rf_off, pad16_bytes(nFr)}};
    if (!stage(&bar, dst, sl, err)) return;
    const uint16_t* fe16 = reinterpret_cast<const uint16_t*>(s_fe);

    // 1. local EF: count, scan, scatter (afterwards s_ec[e] is the end of
    //    row e, so row e is [e ? s_ec[e-1] : 0, s_ec[e]))
    for (int i = threadIdx.x; i < 3 * nFl; i += kQT) atomicAdd(&s_ec[fe16[i] >> 1], 1);
    __syncthreads();
    block_exclusive_scan<kQT>(s_ec, nEl + 1, s_warp);
    for (int i = threadIdx.x; i < 3 * nFl; i += kQT)
        s_ef[atomicAdd(&s_ec[fe16[i] >> 1], 1)] = (uint16_t)(i / 3);
    __syncthreads();

    // 2. FF row lengths of the owned faces: sum over the edges of (faces - 1)
    for (int f = threadIdx.x; f < nFo; f += kQT) {
        int32_t c = 0;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const int32_t e = fe16[3 * f + k] >> 1;
            c += s_ec[e] - (e ? s_ec[e - 1] : 0) - 1;
        }
        s_fc[f] = c;
    }
    if (threadIdx.x == 0) s_fc[nFo] = 0;
    __syncthreads();
    const int32_t vbase = __ldg(qb + blockIdx.x);
    const int32_t total = block_exclusive_scan<kQT>(s_fc, nFo + 1, s_warp, out_off + h.f_base, vbase);

    // 3. rows: each owned face lists the other faces of its three edges
    uint16_t* sbuf = s_out + (vbase & 3);
    for (int f = threadIdx.x; f < nFo; f += kQT) {
        int32_t pos = s_fc[f];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const int32_t e = fe16[3 * f + k] >> 1;
            for (int32_t j = e ? s_ec[e - 1] : 0; j < s_ec[e]; ++j) {
                const uint16_t g = s_ef[j];
                if (g != (uint16_t)f) sbuf[pos++] = g;
            }
        }
    }
    __syncthreads();
    const uint32_t* rf = s_rf;
    const int32_t   fb = h.f_base;
    store_u16_mapped<kQT>(out_val, vbase, s_out, total, [=](uint32_t loc) -> int32_t {
        return (int32_t)loc < nFo ? fb + (int32_t)loc : (int32_t)rf[loc - nFo];
    });
}

// ---------------------------------------------------------------------
// Vertex normals: per patch, each owned vertex sums the normals of its
// incident faces (owned and ribbon) in input VF order, reading the patch's
// incidence block (static topology: per incident face the two other
// corners, in the face's cyclic order after the vertex): no atomics, a fixed
// summation order, so the result is deterministic.  Each face normal is
// formed with the vertex as the first corner, cross(a - v, b - v): the same
// vector as from the face's input corner order (a cyclic rotation), within
// FP32 rounding.  Max weights scale it by 1 / (|v - a|^2 + |b - v|^2), the
// two edges at the corner.  Formula of compute_vertex_normal
// (apps/VertexNormal/vertex_normal_kernel.cuh:10-43).
// ---------------------------------------------------------------------

template <int W, int kQT>
__global__ void __launch_bounds__(kQT) k_vertex_normals(const PatchHdr* __restrict__ hdrs,
                                                        const int32_t* __restrict__ nrm_off,
                                                        const uint32_t* __restrict__ nrm,
                                                        const uint32_t* __restrict__ arena,
                                                        const float* __restrict__ xyz,
                                                        float* __restrict__ out, int* err)
{
    extern __shared__ __align__(16) uint32_t smem[];
    __shared__ uint64_t bar;

    const PatchHdr h     = load_hdr(hdrs);
    const int32_t  nVo   = h.nVo, nVr = h.nVl - h.nVo;
    const int32_t  b0    = __ldg(nrm_off + blockIdx.x);
    const int32_t  words = __ldg(nrm_off + blockIdx.x + 1) - b0;  // > 0, multiple of 4
    const uint32_t* s_off = smem;
    const uint32_t* s_vis = smem + pad4i(nVo + 1);
    float4*         s_pos = reinterpret_cast<float4*>(smem + words);

    if (threadIdx.x == 0) mbar_init(&bar, 1);
    __syncthreads();
    // the incidence block comes in by TMA while the threads gather the
    // positions: owned ones from the patch's contiguous range, ribbon ones
    // through the ribbon table read straight from global memory
    if (threadIdx.x == 0) {
        mbar_arrive_expect_tx(&bar, 4u * (uint32_t)words);
        bulk_g2s(smem, nrm + b0, 4u * (uint32_t)words, &bar);
    }
    const float* xo = xyz + 3 * (int64_t)h.v_base;
    for (int i = threadIdx.x; i < nVo; i += kQT)
        s_pos[i] = make_float4(__ldg(xo + 3 * i), __ldg(xo + 3 * i + 1), __ldg(xo + 3 * i + 2), 0.f);
    for (int i = threadIdx.x; i < nVr; i += kQT) {
        const int64_t g = 3 * (int64_t)__ldg(arena + h.rv_off + i);
        s_pos[nVo + i]  = make_float4(__ldg(xyz + g), __ldg(xyz + g + 1), __ldg(xyz + g + 2), 0.f);
    }
    if (!wait_stage(&bar, err)) return;  // its CTA barrier also orders the position stores

    float* o = out + 3 * (int64_t)h.v_base;
    for (int v = threadIdx.x; v < nVo; v += kQT) {
        const float4   P  = s_pos[v];
        float          a0 = 0.f, a1 = 0.f, a2 = 0.f;
        const uint32_t j1 = s_off[v + 1];
#pragma unroll 2
        for (uint32_t j = s_off[v]; j < j1; ++j) {
            const uint32_t q = s_vis[j];
            const float4   A = s_pos[q & 0xffffu], B = s_pos[q >> 16];
            const float3   u = make_float3(A.x - P.x, A.y - P.y, A.z - P.z);
            const float3   w = make_float3(B.x - P.x, B.y - P.y, B.z - P.z);
            const float    n0 = u.y * w.z - w.y * u.z, n1 = u.z * w.x - w.z * u.x, n2 = u.x * w.y - w.x * u.y;
            if (W == RXG_NORMAL_MAX) {
                // n / (|v - a|^2 + |b - v|^2), one reciprocal for the three
                // components
                const float r = 1.f / ((u.x * u.x + u.y * u.y + u.z * u.z) + (w.x * w.x + w.y * w.y + w.z * w.z));
                a0 += n0 * r;
                a1 += n1 * r;
                a2 += n2 * r;
            } else {
                a0 += n0;
                a1 += n1;
                a2 += n2;
            }
        }
        o[3 * v]     = a0;
        o[3 * v + 1] = a1;
        o[3 * v + 2] = a2;
    }
}

// ---------------------------------------------------------------------
// The sweep in one launch (rxg_query_sweep): per patch, any of VV, VE, VF,
// FV, EV and vertex normals.  The patch's EV / FE slices, its three ribbon
// tables and (for normals) its incidence block are staged once; VV and VE
// share one counting sort (a row of VV and the same row of VE list the same
// incident edges: the offsets are identical, the values are the edge's other
// end and the edge); VF turns the FE slice into local FV in place.  Each
// output is the value its own kernel writes (normals, FV, EV, EVD-free
// rows bit for bit; CSR rows as the same sets, in shared-memory-atomic order).
// ---------------------------------------------------------------------

struct SweepArgs
{
    int32_t *vv_off, *vv_val, *ve_off, *ve_val, *vf_off, *vf_val, *fv_val, *ev_val;
    const float* xyz;
    float*       nrm_out;
    int          weighting;
};

// words of the sweep's reused region for one patch (normals block + float4
// positions, VV and VE rows, VF rows: the largest of the requested ones)
__host__ __device__ __forceinline__ int32_t sweep_big_words(const PatchHdr& h, int32_t nrm_words, bool nrm,
                                                             bool vvve, bool vf)
{
    int32_t w = 0;
    if (nrm) w = nrm_words + 4 * h.nVl;
    const int32_t vvw = pad4i(h.nEl + 4) + h.nEl + 4;  // VV rows, then VE rows 16-byte aligned
    if (vvve) w = w > vvw ? w : vvw;
    const int32_t vfw = (3 * h.nFl + 1) / 2 + 4;
    if (vf) w = w > vfw ? w : vfw;
    return pad4i(w);
}

template <int kQT>
__global__ void __launch_bounds__(kQT) k_query_sweep(const PatchHdr* __restrict__ hdrs,
                                                     const int32_t* __restrict__ nrm_off,
                                                     const uint32_t* __restrict__ nrm,
                                                     const uint32_t* __restrict__ arena, SweepArgs o,
                                                     int* err)
{
    extern __shared__ __align__(16) uint32_t smem[];
    __shared__ uint64_t bar;
    __shared__ int32_t  s_warp[kQT / 32];

    const PatchHdr h   = load_hdr(hdrs);
    const int32_t  nVo = h.nVo, nEo = h.nEo, nFo = h.nFo;
    const int32_t  nVr = h.nVl - nVo, nEr = h.nEl - nEo, nFr = h.nFl - nFo;
    const bool     NRM = o.nrm_out != nullptr, VVVE = o.vv_val || o.ve_val, VF = o.vf_val != nullptr;
    const int32_t  b0  = NRM ? __ldg(nrm_off + blockIdx.x) : 0;
    const int32_t  nw  = NRM ? __ldg(nrm_off + blockIdx.x + 1) - b0 : 0;

    // only the slices the requested outputs read are staged (the host sizes
    // shared memory for all of them)
    const bool    NEV = VVVE || VF || o.fv_val || o.ev_val, NFE = VF || o.fv_val;
    const bool    NRV = o.vv_val || o.fv_val || o.ev_val, NRE = o.ve_val != nullptr;
    const int32_t wev = NEV ? pad4i(h.nEl) : 0, wfe = NFE ? pad4i((int32_t)fe_words(h.nFl)) : 0;
    const int32_t wrv = NRV ? pad4i(nVr) : 0, wre = NRE ? pad4i(nEr) : 0, wrf = VF ? pad4i(nFr) : 0;
    uint32_t* s_ev  = smem;
    uint32_t* s_fe  = s_ev + wev;
    uint32_t* s_rv  = s_fe + wfe;
    uint32_t* s_re  = s_rv + wrv;
    uint32_t* s_rf  = s_re + wre;
    int32_t*  s_cnt = reinterpret_cast<int32_t*>(s_rf + wrf);
    uint32_t* s_big = reinterpret_cast<uint32_t*>(s_cnt + pad4i(nVo + 1 + kSpill));

    if (threadIdx.x == 0) mbar_init(&bar, 1);
    __syncthreads();
    {
        uint32_t* const dst[6] = {s_ev, s_fe, s_rv, s_re, s_rf, s_big};
        const Slice     sl[6]  = {{arena + h.ev_off, 4u * (uint32_t)wev}, {arena + h.fe_off, 4u * (uint32_t)wfe},
                                  {arena + h.rv_off, 4u * (uint32_t)wrv}, {arena + h.re_off, 4u * (uint32_t)wre},
                                  {arena + h.rf_off, 4u * (uint32_t)wrf}, {nrm + b0, 4u * (uint32_t)nw}};
        // positions for the normals come in while the slices do
        float4* s_pos = reinterpret_cast<float4*>(s_big + nw);
        if (threadIdx.x == 0) {
            uint32_t total = 0;
#pragma unroll
            for (int i = 0; i < 6; ++i) total += sl[i].bytes;
            mbar_arrive_expect_tx(&bar, total);
#pragma unroll
            for (int i = 0; i < 6; ++i)
                if (sl[i].bytes) bulk_g2s(dst[i], sl[i].src, sl[i].bytes, &bar);
        }
        if (NRM) {
            const float* xo = o.xyz + 3 * (int64_t)h.v_base;
            for (int i = threadIdx.x; i < nVo; i += kQT)
                s_pos[i] = make_float4(__ldg(xo + 3 * i), __ldg(xo + 3 * i + 1), __ldg(xo + 3 * i + 2), 0.f);
            for (int i = threadIdx.x; i < nVr; i += kQT) {
                const int64_t g = 3 * (int64_t)__ldg(arena + h.rv_off + i);
                s_pos[nVo + i]  = make_float4(__ldg(o.xyz + g), __ldg(o.xyz + g + 1), __ldg(o.xyz + g + 2), 0.f);
            }
        }
        if (!wait_stage(&bar, err)) return;
    }
    const uint16_t* fe16 = reinterpret_cast<const uint16_t*>(s_fe);
    const int32_t   vb = h.v_base, eb = h.e_base, fb = h.f_base;
    auto            vlin = [=](uint32_t l) -> int32_t { return (int32_t)l < nVo ? vb + (int32_t)l : (int32_t)s_rv[l - nVo]; };

    // ---- normals (the arithmetic and order of k_vertex_normals)
    if (NRM) {
        const uint32_t* s_off = s_big;
        const uint32_t* s_vis = s_big + pad4i(nVo + 1);
        const float4*   s_pos = reinterpret_cast<const float4*>(s_big + nw);
        float*          out   = o.nrm_out + 3 * (int64_t)vb;
        for (int v = threadIdx.x; v < nVo; v += kQT) {
            const float4   P  = s_pos[v];
            float          a0 = 0.f, a1 = 0.f, a2 = 0.f;
            const uint32_t j1 = s_off[v + 1];
            for (uint32_t j = s_off[v]; j < j1; ++j) {
                const uint32_t q = s_vis[j];
                const float4   A = s_pos[q & 0xffffu], B = s_pos[q >> 16];
                const float3   u = make_float3(A.x - P.x, A.y - P.y, A.z - P.z);
                const float3   w = make_float3(B.x - P.x, B.y - P.y, B.z - P.z);
                const float n0 = u.y * w.z - w.y * u.z, n1 = u.z * w.x - w.z * u.x, n2 = u.x * w.y - w.x * u.y;
                if (o.weighting == RXG_NORMAL_MAX) {
                    const float r = 1.f / ((u.x * u.x + u.y * u.y + u.z * u.z) + (w.x * w.x + w.y * w.y + w.z * w.z));
                    a0 += n0 * r;
                    a1 += n1 * r;
                    a2 += n2 * r;
                } else {
                    a0 += n0;
                    a1 += n1;
                    a2 += n2;
                }
            }
            out[3 * v]     = a0;
            out[3 * v + 1] = a1;
            out[3 * v + 2] = a2;
        }
    }
    // ---- EV and FV rows
    if (o.ev_val) {
        int32_t* base = o.ev_val + 2 * (int64_t)eb;
        for (int i = threadIdx.x; i < 2 * nEo; i += kQT) {
            const uint32_t ev = s_ev[i >> 1];
            base[i]           = vlin((i & 1) ? (ev >> 16) : (ev & 0xffffu));
        }
    }
    if (o.fv_val) {
        int32_t* base = o.fv_val + 3 * (int64_t)fb;
        for (int i = threadIdx.x; i < 3 * nFo; i += kQT) base[i] = vlin(face_vertex(fe16, s_ev, i / 3, i % 3));
    }
    if (!VVVE && !VF) return;
    const int32_t spill = nVo + 1 + (int32_t)(threadIdx.x & 31);
    auto          slot  = [&](uint32_t r) -> int32_t* { return &s_cnt[(int32_t)r < nVo ? (int32_t)r : spill]; };
    __syncthreads();  // the normals' use of the reused region is over

    // ---- VV and VE: one counting sort over the EV endpoints
    if (VVVE) {
        for (int i = threadIdx.x; i < nVo + 1 + kSpill; i += kQT) s_cnt[i] = 0;
        __syncthreads();
        const uint2*  ev2 = reinterpret_cast<const uint2*>(s_ev);
        const int32_t nE2 = (h.nEl + 1) >> 1;
        for (int e2 = threadIdx.x; e2 < nE2; e2 += kQT) {
            const uint2    w  = ev2[e2];
            const bool     hi = 2 * e2 + 1 < h.nEl;
            const uint32_t a0 = w.x & 0xffffu, b0 = w.x >> 16;
            const uint32_t a1 = hi ? w.y & 0xffffu : 0xffffu, b1 = hi ? w.y >> 16 : 0xffffu;
            atomicAdd(slot(a0), 1);
            atomicAdd(slot(b0), 1);
            atomicAdd(slot(a1), 1);
            atomicAdd(slot(b1), 1);
        }
        __syncthreads();
        const int32_t vbase = h.vv_base;
        const int32_t total = block_exclusive_scan<kQT>(s_cnt, nVo + 1, s_warp, o.vv_off ? o.vv_off + vb : nullptr, vbase);
        if (o.ve_off) {  // the same offsets, read before the scatter moves the counters
            for (int v = threadIdx.x; v <= nVo; v += kQT) o.ve_off[vb + v] = vbase + s_cnt[v];
            __syncthreads();
        }
        // rows of VV at s_big, of VE behind them (element g at [g - (vbase & ~3)])
        uint16_t* svv = reinterpret_cast<uint16_t*>(s_big);
        uint16_t* sve = reinterpret_cast<uint16_t*>(s_big + pad4i(h.nEl + 4));
        uint16_t* bvv = svv + (vbase & 3);
        uint16_t* bve = sve + (vbase & 3);
        for (int e2 = threadIdx.x; e2 < nE2; e2 += kQT) {
            const uint2    w  = ev2[e2];
            const bool     hi = 2 * e2 + 1 < h.nEl;
            const uint32_t a0 = w.x & 0xffffu, b0 = w.x >> 16;
            const uint32_t a1 = hi ? w.y & 0xffffu : 0xffffu, b1 = hi ? w.y >> 16 : 0xffffu;
            const uint16_t e0 = (uint16_t)(2 * e2), e1 = (uint16_t)(2 * e2 + 1);
            const int32_t  q0 = atomicAdd(slot(a0), 1), q1 = atomicAdd(slot(b0), 1);
            const int32_t  q2 = atomicAdd(slot(a1), 1), q3 = atomicAdd(slot(b1), 1);
            if ((int32_t)a0 < nVo) bvv[q0] = (uint16_t)b0, bve[q0] = e0;
            if ((int32_t)b0 < nVo) bvv[q1] = (uint16_t)a0, bve[q1] = e0;
            if ((int32_t)a1 < nVo) bvv[q2] = (uint16_t)b1, bve[q2] = e1;
            if ((int32_t)b1 < nVo) bvv[q3] = (uint16_t)a1, bve[q3] = e1;
        }
        __syncthreads();
        if (o.vv_val) store_u16_mapped<kQT>(o.vv_val, vbase, svv, total, vlin);
        if (o.ve_val)
            store_u16_mapped<kQT>(o.ve_val, vbase, sve, total, [=](uint32_t l) -> int32_t {
                return (int32_t)l < nEo ? eb + (int32_t)l : (int32_t)s_re[l - nEo];
            });
        if (VF) __syncthreads();  // VF reuses the counters and the region
    }

    // ---- VF: the FE slice becomes local FV in place (FV rows are written)
    if (VF) {
        for (int i = threadIdx.x; i < nVo + 1 + kSpill; i += kQT) s_cnt[i] = 0;
        __syncthreads();
        uint16_t* fv16 = reinterpret_cast<uint16_t*>(s_fe);
        for (int f = threadIdx.x; f < h.nFl; f += kQT) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const uint32_t v = face_vertex(fe16, s_ev, f, k);
                fv16[3 * f + k]  = (uint16_t)v;
                atomicAdd(slot(v), 1);
            }
        }
        __syncthreads();
        const int32_t vbase = h.vf_base;
        const int32_t total = block_exclusive_scan<kQT>(s_cnt, nVo + 1, s_warp, o.vf_off ? o.vf_off + vb : nullptr, vbase);
        uint16_t* svf = reinterpret_cast<uint16_t*>(s_big);
        uint16_t* bvf = svf + (vbase & 3);
        for (int f = threadIdx.x; f < h.nFl; f += kQT) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const uint32_t v = fv16[3 * f + k];
                const int32_t  q = atomicAdd(slot(v), 1);
                if ((int32_t)v < nVo) bvf[q] = (uint16_t)f;
            }
        }
        __syncthreads();
        store_u16_mapped<kQT>(o.vf_val, vbase, svf, total, [=](uint32_t l) -> int32_t {
            return (int32_t)l < nFo ? fb + (int32_t)l : (int32_t)s_rf[l - nFo];
        });
    }
}

// A wait that cannot complete (nothing arrives at the barrier), bounded by
// `attempts` tries of ~1 us each: it reports through the error word and the
// CTA returns, the path every bounded wait in the library takes.
__global__ void k_wait_selftest(int* err, int attempts)
{
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) mbar_init(&bar, 1);
    __syncthreads();
    if (threadIdx.x == 0) {
        bool ok = false;
        for (int i = 0; i < attempts && !ok; ++i) ok = mbar_try_wait_hint(&bar, 0, 1000);
        if (!ok) atomicOr(err, DEVERR_MBAR_TIMEOUT);
    }
}

// ---------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------

// shared-memory table kinds of the normal kernels (after the query ops)
constexpr int kNormalArea = 12, kNormalMax = 13;
// and of the oriented-mesh FF kernel
constexpr int kFFOriented = 11;

// dynamic shared memory (bytes) of one patch for a kernel kind
static size_t smem_words(const PatchHdr& h, int kind)
{
    const int32_t nVr = h.nVl - h.nVo, nEr = h.nEl - h.nEo, nFr = h.nFl - h.nFo;
    const int32_t few = pad4i((3 * h.nFl + 1) / 2);
    switch (kind) {
        case RXG_OP_VV:
        case RXG_OP_VE:
            return pad4i(h.nEl) + pad4i(kind == RXG_OP_VV ? nVr : nEr) + pad4i(h.nVo + 1 + kSpill) +
                   h.nEl + 4;
        case RXG_OP_VF: return vf_ev_words(h) + few + pad4i(nFr) + pad4i(h.nVo + 1 + kSpill);
        case RXG_OP_FV: return pad4i(h.nEl) + pad4i((3 * h.nFo + 1) / 2) + pad4i(nVr);
        case RXG_OP_EV: return pad4i(h.nEo) + pad4i(nVr);
        case RXG_OP_EF: return few + pad4i(nFr) + pad4i(h.nEo + 1 + kSpill) + (3 * h.nFl + 1) / 2 + 4;
        case RXG_OP_FE: return pad4i((3 * h.nFo + 1) / 2) + pad4i(nEr);
        case RXG_OP_FF:  // + the patch's FF values, added by compute_smem_table
            return few + pad4i(nFr) + pad4i(h.nEl + 1) + few + pad4i(h.nFo + 1) + 4;
        case RXG_OP_EVD: return pad4i(h.nEl) + few + pad4i(nVr) + 2 * (size_t)h.nEo;
        case RXG_OP_EE: return few + pad4i(nEr) + 2 * (size_t)h.nEo;
        case kFFOriented:  // + the patch's FF values, added by compute_smem_table
            return few + pad4i(nFr) + pad4i(h.nEl) + pad4i(h.nFo + 1) + 4;
        default:  // normals: positions as float4 behind the incidence block
            return 4 * (size_t)h.nVl;
    }
}

void compute_smem_table(Mesh& m)
{
    for (int kind = 0; kind <= kNormalMax; ++kind) {
        if (kind == 10) continue;  // unused
        size_t w = 0;
        for (size_t p = 0; p < m.hdr.size(); ++p) {
            size_t pw = smem_words(m.hdr[p], kind);
            if (kind == kNormalArea || kind == kNormalMax)
                pw += (size_t)(m.nrm_off[p + 1] - m.nrm_off[p]);
            if (kind == RXG_OP_FF || kind == kFFOriented)
                pw += (size_t)(m.ff_base[p + 1] - m.ff_base[p] + 1) / 2;
            w = std::max(w, pw);
        }
        m.smem_bytes[kind] = w * 4;
    }
    // the fused sweep: the slices each set of outputs stages (as
    // k_query_sweep lays them out) plus its counters and reused region
    for (int c = 0; c < 64; ++c) {
        const bool NRM = c & 1, VV = c & 2, VE = c & 4, VF = c & 8, FV = c & 16, EV = c & 32;
        const bool VVVE = VV || VE, NEV = VVVE || VF || FV || EV, NFE = VF || FV;
        const bool NRV = VV || FV || EV, NRE = VE;
        size_t     w = 0;
        for (size_t p = 0; p < m.hdr.size(); ++p) {
            const PatchHdr& h  = m.hdr[p];
            const int32_t   nw = NRM ? m.nrm_off[p + 1] - m.nrm_off[p] : 0;
            const size_t    pw = (size_t)(NEV ? pad4i(h.nEl) : 0) + (NFE ? pad4i((int32_t)fe_words(h.nFl)) : 0) +
                              (NRV ? pad4i(h.nVl - h.nVo) : 0) + (NRE ? pad4i(h.nEl - h.nEo) : 0) +
                              (VF ? pad4i(h.nFl - h.nFo) : 0) + pad4i(h.nVo + 1 + kSpill) +
                              sweep_big_words(h, nw, NRM, VVVE, VF);
            w = std::max(w, pw);
        }
        m.sweep_smem[c] = w * 4;
    }
}

size_t query_smem_bytes(const Mesh* m, int kind) { return m->smem_bytes[kind]; }

template <typename K>
static rxg_status launch_patch_kernel(K kern, const Mesh* m, size_t smem, cudaStream_t s,
                                      const char* name)
{
    (void)kern;
    if (smem > 227 * 1024) {
        set_error("%s: a patch needs %zu bytes of shared memory (> 227 KB); use smaller patches",
                  name, smem);
        return RXG_ERR_PATCH_LIMIT;
    }
    return RXG_OK;
}

// Patches [p0, p0 + np) of a patch kernel: CTA b works on patch p0 + b (its
// header pointer is offset; every other index in the headers is absolute).
struct PatchRange
{
    int32_t p0, np;
};

template <typename F, typename... Args>
static rxg_status launch(F* kern, int threads, const Mesh* m, size_t smem, cudaStream_t s,
                         const char* name, PatchRange r, const PatchHdr* hd, Args... args)
{
    rxg_status st = launch_patch_kernel(kern, m, smem, s, name);
    if (st) return st;
    if (r.np <= 0) return RXG_OK;
    if (smem > 48 * 1024)
        RXG_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem));
    kern<<<r.np, threads, smem, s>>>(hd + r.p0, args...);
    RXG_CUDA_TRY(cudaGetLastError());
    return RXG_OK;
}

// threads per query CTA: 128 by default (fastest on the 1024x1024 torus with
// 512-face patches), RXG_QUERY_THREADS=32|64|128|256 to tune
int query_threads()
{
    static int t = 0;
    if (!t) {
        const char* e = getenv("RXG_QUERY_THREADS");
        t             = e ? atoi(e) : 128;
        if (t != 32 && t != 64 && t != 128 && t != 256) t = 128;
    }
    return t;
}

template <int BT>
static rxg_status launch_query_bt(const Mesh* m, int op, int32_t* d_off, int32_t* d_val,
                                  cudaStream_t s, PatchRange r)
{
    const size_t    smem = query_smem_bytes(m, op);
    int*            err  = device_error_word();
    const PatchHdr* hd   = m->d.hdr;
    const uint32_t* ar   = m->d.arena;
    const int32_t*  ef_b = m->d.qbase + r.p0;                         // EF bases, indexed like hd
    const int32_t*  ff_b = m->d.qbase + (m->num_patches + 1) + r.p0;  // FF bases
    switch (op) {
        case RXG_OP_VV: return launch(k_query_vertex<0, BT>, BT, m, smem, s, "VV", r, hd, ar, d_off, d_val, err, ef_b);
        case RXG_OP_VE: return launch(k_query_vertex<1, BT>, BT, m, smem, s, "VE", r, hd, ar, d_off, d_val, err, ef_b);
        case RXG_OP_VF: return launch(k_query_vertex<2, BT>, BT, m, smem, s, "VF", r, hd, ar, d_off, d_val, err, ef_b);
        case RXG_OP_EF: return launch(k_query_vertex<RXG_OP_EF, BT>, BT, m, smem, s, "EF", r, hd, ar, d_off, d_val, err, ef_b);
        case RXG_OP_FF:
            if (m->edge_manifold && m->oriented)
                return launch(k_query_ff_oriented<BT>, BT, m, query_smem_bytes(m, kFFOriented), s,
                              "FF", r, hd, ar, d_off, d_val, err, ff_b);
            return launch(k_query_ff<BT>, BT, m, smem, s, "FF", r, hd, ar, d_off, d_val, err, ff_b);
        case RXG_OP_FV: return launch(k_query_elem<3, BT>, BT, m, smem, s, "FV", r, hd, ar, d_val, err);
        case RXG_OP_EV: return launch(k_query_elem<4, BT>, BT, m, smem, s, "EV", r, hd, ar, d_val, err);
        case RXG_OP_FE: return launch(k_query_elem<RXG_OP_FE, BT>, BT, m, smem, s, "FE", r, hd, ar, d_val, err);
        case RXG_OP_EVD: return launch(k_query_elem<RXG_OP_EVD, BT>, BT, m, smem, s, "EVD", r, hd, ar, d_val, err);
        case RXG_OP_EE: return launch(k_query_elem<RXG_OP_EE, BT>, BT, m, smem, s, "EE", r, hd, ar, d_val, err);
    }
    set_error("rxg_query: unknown op %d", op);
    return RXG_ERR_INVALID;
}

static rxg_status launch_query_range(const Mesh* m, int op, int32_t* d_off, int32_t* d_val,
                                     cudaStream_t s, PatchRange r)
{
    switch (query_threads()) {
        case 32: return launch_query_bt<32>(m, op, d_off, d_val, s, r);
        case 64: return launch_query_bt<64>(m, op, d_off, d_val, s, r);
        case 256: return launch_query_bt<256>(m, op, d_off, d_val, s, r);
        default: return launch_query_bt<128>(m, op, d_off, d_val, s, r);
    }
}

rxg_status launch_query(const Mesh* m, int op, int32_t* d_off, int32_t* d_val, cudaStream_t s)
{
    return launch_query_range(m, op, d_off, d_val, s, PatchRange{0, m->num_patches});
}

// threads per CTA of the fused sweep: 128 by default (faster than 256 on
// the 1024^2 torus), RXG_SWEEP_THREADS=256 to tune
static int sweep_threads()
{
    static int t = 0;
    if (!t) {
        const char* e = getenv("RXG_SWEEP_THREADS");
        t             = (e && atoi(e) == 256) ? 256 : 128;
    }
    return t;
}

template <int BT>
static rxg_status launch_normals_bt(const Mesh* m, int weighting, const float* xyz, float* out,
                                    cudaStream_t s, PatchRange r)
{
    // Max or area weights: the same shared-memory layout (table kinds kNormalMax / kNormalArea)
    const size_t    smem = query_smem_bytes(m, weighting == RXG_NORMAL_MAX ? kNormalMax : kNormalArea);
    int*            err  = device_error_word();
    const PatchHdr* hd   = m->d.hdr;
    const int32_t*  no   = m->d.nrm_off + r.p0;  // CTA b reads nrm_off[p0 + b], [p0 + b + 1]
    if (weighting == RXG_NORMAL_MAX)
        return launch(k_vertex_normals<RXG_NORMAL_MAX, BT>, BT, m, smem, s, "normals", r, hd, no,
                      (const uint32_t*)m->d.nrm, (const uint32_t*)m->d.arena, xyz, out, err);
    return launch(k_vertex_normals<RXG_NORMAL_AREA, BT>, BT, m, smem, s, "normals", r, hd, no,
                  (const uint32_t*)m->d.nrm, (const uint32_t*)m->d.arena, xyz, out, err);
}

static rxg_status launch_normals(const Mesh* m, int weighting, const float* xyz, float* out,
                                 cudaStream_t s, PatchRange r)
{
    switch (query_threads()) {
        case 32: return launch_normals_bt<32>(m, weighting, xyz, out, s, r);
        case 64: return launch_normals_bt<64>(m, weighting, xyz, out, s, r);
        case 256: return launch_normals_bt<256>(m, weighting, xyz, out, s, r);
        default: return launch_normals_bt<128>(m, weighting, xyz, out, s, r);
    }
}

// scratch helper: device copy of a possibly-host array
struct Staged
{
    void*        d    = nullptr;
    bool         owns = false;
    cudaStream_t s    = nullptr;
    ~Staged()
    {
        if (owns) cudaFreeAsync(d, s);
    }
};

static rxg_status stage_out(void* user, size_t bytes, cudaStream_t s, Staged& st)
{
    st.s = s;
    if (user == nullptr || is_device_ptr(user)) {
        st.d = user;
        return RXG_OK;
    }
    RXG_CUDA_TRY(scratch_alloc(&st.d, bytes ? bytes : 16, s));
    st.owns = true;
    return RXG_OK;
}

// page-locked (or registered) host memory: a stream-ordered copy can target it
static bool is_pinned_host(const void* p)
{
    if (!p) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

// the device address of page-locked host memory (nullptr otherwise)
static void* host_mapped(void* p)
{
    if (!is_pinned_host(p)) return nullptr;
    void* d = nullptr;
    if (cudaHostGetDevicePointer(&d, p, 0) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return d;
}

static rxg_status stage_in(const void* user, size_t bytes, cudaStream_t s, Staged& st)
{
    st.s = s;
    if (user == nullptr || is_device_ptr(user)) {
        st.d = const_cast<void*>(user);
        return RXG_OK;
    }
    RXG_CUDA_TRY(scratch_alloc(&st.d, bytes ? bytes : 16, s));
    st.owns = true;
    RXG_CUDA_TRY(cudaMemcpyAsync(st.d, user, bytes, cudaMemcpyHostToDevice, s));
    return RXG_OK;
}

// One output array of a host-array call: element e of the device copy goes
// to element e of the host array; eb[k] is the first element slice k writes.
struct HostPiece
{
    char*                host;
    const char*          dev;
    size_t               esz;
    std::vector<int64_t> eb;  // kSlices + 1 element bounds
};

constexpr int kSlices = 4;

// Host arrays: the kernel runs over kSlices slices of patches on stream s;
// as each slice finishes (an event), its output ranges are copied to the host
// on the mesh's copy stream, so the copies overlap the following slices.
// Every patch writes a contiguous range of each output (linear ids are
// patch-ordered), so the slices' ranges are disjoint.  Returns after the
// copies have landed.
template <typename Run>
static rxg_status run_to_host(const Mesh& M, cudaStream_t s, const int32_t* pb, Run run,
                              std::vector<HostPiece>& pieces)
{
    std::lock_guard<std::mutex> lk(M.stage_mu);
    if (!M.copy_stream) {
        RXG_CUDA_TRY(cudaStreamCreateWithFlags(&M.copy_stream, cudaStreamNonBlocking));
        for (cudaEvent_t& e : M.copy_ev) RXG_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    for (int k = 0; k < kSlices; ++k) {
        rxg_status st = run(PatchRange{pb[k], pb[k + 1] - pb[k]});
        if (st) return st;
        RXG_CUDA_TRY(cudaEventRecord(M.copy_ev[k], s));
        RXG_CUDA_TRY(cudaStreamWaitEvent(M.copy_stream, M.copy_ev[k], 0));
        for (HostPiece& q : pieces) {
            const size_t off = (size_t)q.eb[k] * q.esz, bytes = (size_t)(q.eb[k + 1] - q.eb[k]) * q.esz;
            if (bytes)
                RXG_CUDA_TRY(cudaMemcpyAsync(q.host + off, q.dev + off, bytes, cudaMemcpyDeviceToHost,
                                             M.copy_stream));
        }
    }
    RXG_CUDA_TRY(cudaStreamSynchronize(M.copy_stream));
    return RXG_OK;
}

// patch bounds of the slices
static void slice_patches(const Mesh& M, int32_t* pb)
{
    for (int k = 0; k <= kSlices; ++k) pb[k] = (int32_t)((int64_t)M.num_patches * k / kSlices);
}

// first linear vertex / edge / face of patch p (the total for p = num_patches)
static int64_t v_first(const Mesh& M, int32_t p) { return p < M.num_patches ? M.hdr[p].v_base : M.nv; }
static int64_t e_first(const Mesh& M, int32_t p) { return p < M.num_patches ? M.hdr[p].e_base : M.ne; }
static int64_t f_first(const Mesh& M, int32_t p) { return p < M.num_patches ? M.hdr[p].f_base : M.nf; }

}  // namespace rxg

using namespace rxg;

extern "C" {

rxg_status rxg_query_size(const rxg_mesh* h, int32_t op, int64_t* n_rows, int64_t* n_values)
{
    if (!h || !n_rows || !n_values) {
        set_error("rxg_query_size: NULL argument");
        return RXG_ERR_INVALID;
    }
    const Mesh& M = h->m;
    switch (op) {
        case RXG_OP_VV:
        case RXG_OP_VE: *n_rows = M.nv; *n_values = 2 * M.ne; return RXG_OK;
        case RXG_OP_VF: *n_rows = M.nv; *n_values = 3 * M.nf; return RXG_OK;
        case RXG_OP_FV: *n_rows = M.nf; *n_values = 3 * M.nf; return RXG_OK;
        case RXG_OP_EV: *n_rows = M.ne; *n_values = 2 * M.ne; return RXG_OK;
        case RXG_OP_EF: *n_rows = M.ne; *n_values = 3 * M.nf; return RXG_OK;
        case RXG_OP_FE: *n_rows = M.nf; *n_values = 3 * M.nf; return RXG_OK;
        case RXG_OP_FF: *n_rows = M.nf; *n_values = M.ff_base.empty() ? 0 : M.ff_base.back(); return RXG_OK;
        case RXG_OP_EVD:
        case RXG_OP_EE: *n_rows = M.ne; *n_values = 4 * M.ne; return RXG_OK;
    }
    set_error("rxg_query_size: unknown op %d", op);
    return RXG_ERR_INVALID;
}

rxg_status rxg_query(const rxg_mesh* h, int32_t op, int32_t* offsets, int32_t* values,
                     void* stream)
{
    int64_t rows, nval;
    rxg_status st = rxg_query_size(h, op, &rows, &nval);
    if (st) return st;
    const bool csr = op <= RXG_OP_VF || op == RXG_OP_EF || op == RXG_OP_FF;
    if ((op == RXG_OP_EVD || op == RXG_OP_EE) && (!h->m.edge_manifold || !h->m.oriented)) {
        set_error("rxg_query: %s needs an edge-manifold, consistently oriented mesh "
                  "(each edge's two faces traverse it in opposite directions)",
                  op == RXG_OP_EE ? "EE" : "EVDiamond");
        return RXG_ERR_NONMANIFOLD;
    }
    if (!values || (csr && !offsets)) {
        set_error("rxg_query: values%s must not be NULL", csr ? " and offsets" : "");
        return RXG_ERR_INVALID;
    }
    if (((uintptr_t)values & 15u) != 0) {
        set_error("rxg_query: values must be 16-byte aligned (vectorised row stores)");
        return RXG_ERR_INVALID;
    }
    cudaStream_t s = (cudaStream_t)stream;
    Staged       so, sv;
    const size_t off_bytes = csr ? (size_t)(rows + 1) * 4 : 0, val_bytes = (size_t)nval * 4;
    if ((st = stage_out(csr ? offsets : nullptr, off_bytes, s, so))) return st;
    if ((st = stage_out(values, val_bytes, s, sv))) return st;
    const Mesh& M = h->m;
    if (!so.owns && !sv.owns) return launch_query(&M, op, (int32_t*)so.d, (int32_t*)sv.d, s);
    // host outputs: sliced launch, each slice's rows copied while the next runs
    int32_t pb[kSlices + 1];
    slice_patches(M, pb);
    std::vector<HostPiece> pieces;
    if (csr && so.owns) {
        HostPiece q{(char*)offsets, (const char*)so.d, 4, {}};
        // the offsets (4 bytes a row) go back in one copy after the last
        // slice: the link carries the same bytes with fewer copies, each of
        // which costs a few microseconds of gap
        for (int k = 0; k <= kSlices; ++k) q.eb.push_back(k == kSlices ? rows + 1 : 0);
        pieces.push_back(q);
    }
    if (sv.owns) {
        HostPiece q{(char*)values, (const char*)sv.d, 4, {}};
        for (int k = 0; k <= kSlices; ++k) {
            const int32_t p = pb[k];
            int64_t       e;
            if (op == RXG_OP_FV || op == RXG_OP_FE) e = 3 * f_first(M, p);
            else if (op == RXG_OP_EV) e = 2 * e_first(M, p);
            else if (op == RXG_OP_EVD || op == RXG_OP_EE) e = 4 * e_first(M, p);
            else if (op == RXG_OP_EF) e = M.ef_base[p];
            else if (op == RXG_OP_FF) e = M.ff_base[p];
            else if (p == M.num_patches) e = nval;
            else e = op == RXG_OP_VF ? M.hdr[p].vf_base : M.hdr[p].vv_base;
            q.eb.push_back(e);
        }
        pieces.push_back(q);
    }
    st = run_to_host(M, s, pb,
                     [&](PatchRange r) {
                         return launch_query_range(&M, op, (int32_t*)so.d, (int32_t*)sv.d, s, r);
                     },
                     pieces);
    return st;
}

rxg_status rxg_vertex_normals(const rxg_mesh* h, int32_t weighting, const float* xyz, float* out,
                              void* stream)
{
    if (!h || !xyz || !out || (weighting != RXG_NORMAL_MAX && weighting != RXG_NORMAL_AREA)) {
        set_error("rxg_vertex_normals: bad argument");
        return RXG_ERR_INVALID;
    }
    cudaStream_t s     = (cudaStream_t)stream;
    const size_t bytes = (size_t)h->m.nv * 12;
    Staged       si, so;
    rxg_status   st;
    if ((st = stage_in(xyz, bytes, s, si))) return st;
    if ((st = stage_out(out, bytes, s, so))) return st;
    const Mesh& M = h->m;
    if (!so.owns) {
        st = launch_normals(&M, weighting, (const float*)si.d, (float*)so.d, s,
                            PatchRange{0, M.num_patches});
        if (st == RXG_OK && si.owns) RXG_CUDA_TRY(cudaStreamSynchronize(s));
        return st;
    }
    int32_t pb[kSlices + 1];
    slice_patches(M, pb);
    std::vector<HostPiece> pieces(1, HostPiece{(char*)out, (const char*)so.d, 12, {}});
    for (int k = 0; k <= kSlices; ++k) pieces[0].eb.push_back(v_first(M, pb[k]));
    return run_to_host(M, s, pb,
                       [&](PatchRange r) {
                           return launch_normals(&M, weighting, (const float*)si.d, (float*)so.d, s, r);
                       },
                       pieces);
}

rxg_status rxg_query_ex(const rxg_mesh* h, int32_t op, int32_t* offsets, int32_t* values, int32_t flags,
                        void* stream)
{
    if (flags & ~(RXG_HOST_ASYNC | RXG_HOST_DIRECT)) {
        set_error("rxg_query_ex: unknown flags %d", flags);
        return RXG_ERR_INVALID;
    }
    const bool csr = op <= RXG_OP_VF || op == RXG_OP_EF || op == RXG_OP_FF;
    int64_t    rows, nval;
    rxg_status st = rxg_query_size(h, op, &rows, &nval);
    if (st) return st;
    // argument errors, device outputs and non-manifold EVDiamond: rxg_query
    if (!flags || !values || (csr && !offsets) || is_device_ptr(values) ||
        ((op == RXG_OP_EVD || op == RXG_OP_EE) && (!h->m.edge_manifold || !h->m.oriented)))
        return rxg_query(h, op, offsets, values, stream);
    cudaStream_t s = (cudaStream_t)stream;
    if (flags & RXG_HOST_DIRECT) {
        int32_t* dv = (int32_t*)host_mapped(values);
        int32_t* dof = !csr ? nullptr : is_device_ptr(offsets) ? offsets : (int32_t*)host_mapped(offsets);
        if (dv && (!csr || dof)) {
            if (((uintptr_t)dv & 15u) != 0) {
                set_error("rxg_query_ex: values must be 16-byte aligned (vectorised row stores)");
                return RXG_ERR_INVALID;
            }
            return launch_query(&h->m, op, dof, dv, s);
        }
    }
    // stream-ordered staging: every host output page-locked, else rxg_query
    if (!is_pinned_host(values) || (csr && !is_device_ptr(offsets) && !is_pinned_host(offsets)))
        return rxg_query(h, op, offsets, values, stream);
    if (((uintptr_t)values & 15u) != 0) {
        set_error("rxg_query_ex: values must be 16-byte aligned (vectorised row stores)");
        return RXG_ERR_INVALID;
    }
    Staged       so, sv;
    const size_t off_bytes = csr ? (size_t)(rows + 1) * 4 : 0, val_bytes = (size_t)nval * 4;
    if ((st = stage_out(csr ? offsets : nullptr, off_bytes, s, so))) return st;
    if ((st = stage_out(values, val_bytes, s, sv))) return st;
    // kernel, then the copies, all on `stream`; the scratch is freed in
    // stream order after the copies (Staged's destructor)
    if ((st = launch_query(&h->m, op, (int32_t*)so.d, (int32_t*)sv.d, s))) return st;
    if (so.owns) RXG_CUDA_TRY(cudaMemcpyAsync(offsets, so.d, off_bytes, cudaMemcpyDeviceToHost, s));
    RXG_CUDA_TRY(cudaMemcpyAsync(values, sv.d, val_bytes, cudaMemcpyDeviceToHost, s));
    return RXG_OK;
}

rxg_status rxg_vertex_normals_ex(const rxg_mesh* h, int32_t weighting, const float* xyz, float* out,
                                 int32_t flags, void* stream)
{
    if (flags & ~(RXG_HOST_ASYNC | RXG_HOST_DIRECT)) {
        set_error("rxg_vertex_normals_ex: unknown flags %d", flags);
        return RXG_ERR_INVALID;
    }
    if (!flags || !h || !xyz || !out || (weighting != RXG_NORMAL_MAX && weighting != RXG_NORMAL_AREA) ||
        is_device_ptr(out))
        return rxg_vertex_normals(h, weighting, xyz, out, stream);
    cudaStream_t s     = (cudaStream_t)stream;
    const size_t bytes = (size_t)h->m.nv * 12;
    if (flags & RXG_HOST_DIRECT) {
        const float* dx = is_device_ptr(xyz) ? xyz : (const float*)host_mapped(const_cast<float*>(xyz));
        float*       dn = (float*)host_mapped(out);
        if (dx && dn) return launch_normals(&h->m, weighting, dx, dn, s, PatchRange{0, h->m.num_patches});
    }
    if (!is_pinned_host(out) || !(is_device_ptr(xyz) || is_pinned_host(xyz)))
        return rxg_vertex_normals(h, weighting, xyz, out, stream);
    Staged     si, so;
    rxg_status st;
    if ((st = stage_in(xyz, bytes, s, si))) return st;  // stream-ordered upload
    if ((st = stage_out(out, bytes, s, so))) return st;
    if ((st = launch_normals(&h->m, weighting, (const float*)si.d, (float*)so.d, s,
                             PatchRange{0, h->m.num_patches})))
        return st;
    RXG_CUDA_TRY(cudaMemcpyAsync(out, so.d, bytes, cudaMemcpyDeviceToHost, s));
    return RXG_OK;
}

// Syncs `stream`, reads and clears the device error word set by bounded waits.
rxg_status rxg_query_sweep(const rxg_mesh* h, const rxg_sweep_out* o, void* stream)
{
    if (!h || !o) {
        set_error("rxg_query_sweep: NULL argument");
        return RXG_ERR_INVALID;
    }
    const Mesh& M = h->m;
    // CSR outputs come as pairs; every array given must be device memory;
    // value arrays 16-byte aligned (vectorised row stores)
    const struct { const void* off; const void* val; const char* name; bool csr; } outs[] = {
        {o->vv_offsets, o->vv_values, "VV", true}, {o->ve_offsets, o->ve_values, "VE", true},
        {o->vf_offsets, o->vf_values, "VF", true}, {nullptr, o->fv_values, "FV", false},
        {nullptr, o->ev_values, "EV", false}};
    for (const auto& q : outs) {
        if (q.csr && ((q.off == nullptr) != (q.val == nullptr))) {
            set_error("rxg_query_sweep: %s needs both offsets and values (or neither)", q.name);
            return RXG_ERR_INVALID;
        }
        if ((q.off && !is_device_ptr(q.off)) || (q.val && !is_device_ptr(q.val))) {
            set_error("rxg_query_sweep: the %s arrays must be device arrays", q.name);
            return RXG_ERR_INVALID;
        }
        if (q.val && ((uintptr_t)q.val & 15u) != 0) {
            set_error("rxg_query_sweep: the %s values must be 16-byte aligned", q.name);
            return RXG_ERR_INVALID;
        }
    }
    if (o->normals) {
        if (!o->xyz || !is_device_ptr(o->xyz) || !is_device_ptr(o->normals) ||
            (o->weighting != RXG_NORMAL_MAX && o->weighting != RXG_NORMAL_AREA)) {
            set_error("rxg_query_sweep: normals need device xyz and out arrays and a valid weighting");
            return RXG_ERR_INVALID;
        }
    }
    SweepArgs a;
    a.vv_off = o->vv_offsets, a.vv_val = o->vv_values, a.ve_off = o->ve_offsets, a.ve_val = o->ve_values;
    a.vf_off = o->vf_offsets, a.vf_val = o->vf_values, a.fv_val = o->fv_values, a.ev_val = o->ev_values;
    a.xyz = o->xyz, a.nrm_out = o->normals, a.weighting = o->weighting;
    const int c = (o->normals ? 1 : 0) | (a.vv_val ? 2 : 0) | (a.ve_val ? 4 : 0) | (a.vf_val ? 8 : 0) |
                  (a.fv_val ? 16 : 0) | (a.ev_val ? 32 : 0);
    if (!c) return RXG_OK;
    cudaStream_t    s    = (cudaStream_t)stream;
    const size_t    smem = M.sweep_smem[c];
    int*            err  = device_error_word();
    const PatchHdr* hd   = M.d.hdr;
    const PatchRange r{0, M.num_patches};
    const uint32_t *nb = (const uint32_t*)M.d.nrm, *ar = (const uint32_t*)M.d.arena;
    if (sweep_threads() == 128)
        return launch(k_query_sweep<128>, 128, &M, smem, s, "sweep", r, hd, (const int32_t*)M.d.nrm_off, nb, ar,
                      a, err);
    return launch(k_query_sweep<256>, 256, &M, smem, s, "sweep", r, hd, (const int32_t*)M.d.nrm_off, nb, ar, a,
                  err);
}

// The sweep's outputs in page-locked host memory (or device memory), stream
// ordered: the six kernels run concurrently on the mesh's sweep streams,
// the fastest first and at the highest priority, each writing into one
// device scratch block; the mesh's copy stream moves each result to the
// host as soon as its kernel is done, in that order, so the host link (the
// bound of a sweep to host memory) starts early and stays busy.  Host
// positions for the normals come in on their kernel's stream.  `stream`
// waits for all of it; the call itself returns at once.
rxg_status rxg_query_sweep_ex(const rxg_mesh* h, const rxg_sweep_out* o, int32_t flags, void* stream)
{
    if (!h || !o) {
        set_error("rxg_query_sweep_ex: NULL argument");
        return RXG_ERR_INVALID;
    }
    if (flags & ~RXG_HOST_ASYNC) {
        set_error("rxg_query_sweep_ex: unknown flags %d", flags);
        return RXG_ERR_INVALID;
    }
    if (!flags) return rxg_query_sweep(h, o, stream);
    const Mesh& M = h->m;
    // the outputs in launch order: the quickest kernels first
    struct Out
    {
        int         op;
        void*       off;
        void*       val;
        const char* name;
    };
    const Out outs[5] = {{RXG_OP_EV, nullptr, o->ev_values, "EV"},
                         {RXG_OP_FV, nullptr, o->fv_values, "FV"},
                         {RXG_OP_VV, o->vv_offsets, o->vv_values, "VV"},
                         {RXG_OP_VE, o->ve_offsets, o->ve_values, "VE"},
                         {RXG_OP_VF, o->vf_offsets, o->vf_values, "VF"}};
    // every array device or page-locked host memory; CSR outputs as pairs;
    // device value arrays 16-byte aligned (the kernels' vectorised stores)
    auto kind_ok = [](const void* p) { return p == nullptr || is_device_ptr(p) || is_pinned_host(p); };
    size_t off_b[5] = {}, val_b[5] = {};
    for (int k = 0; k < 5; ++k) {
        const Out& q   = outs[k];
        const bool csr = q.op <= RXG_OP_VF;
        if (csr && ((q.off == nullptr) != (q.val == nullptr))) {
            set_error("rxg_query_sweep_ex: %s needs both offsets and values (or neither)", q.name);
            return RXG_ERR_INVALID;
        }
        if (!kind_ok(q.off) || !kind_ok(q.val)) {
            set_error("rxg_query_sweep_ex: the %s arrays must be device or page-locked host memory", q.name);
            return RXG_ERR_INVALID;
        }
        if (q.val && is_device_ptr(q.val) && ((uintptr_t)q.val & 15u) != 0) {
            set_error("rxg_query_sweep_ex: the %s values must be 16-byte aligned", q.name);
            return RXG_ERR_INVALID;
        }
        int64_t rows = 0, nval = 0;
        rxg_status st = rxg_query_size(h, q.op, &rows, &nval);
        if (st) return st;
        off_b[k] = csr ? (size_t)(rows + 1) * 4 : 0;
        val_b[k] = (size_t)nval * 4;
    }
    if (o->normals && (!o->xyz || !kind_ok(o->xyz) || !kind_ok(o->normals) ||
                       (o->weighting != RXG_NORMAL_MAX && o->weighting != RXG_NORMAL_AREA))) {
        set_error("rxg_query_sweep_ex: normals need xyz and out arrays (device or page-locked host) and a "
                  "valid weighting");
        return RXG_ERR_INVALID;
    }
    // scratch: every host output and host xyz, 256-byte aligned pieces
    auto   up     = [](size_t b) { return (b + 255) & ~(size_t)255; };
    auto   host   = [](const void* p) { return p != nullptr && !is_device_ptr(p); };
    size_t scr    = 0;
    size_t so[5], sv[5];
    for (int k = 0; k < 5; ++k) {
        so[k] = scr, scr += host(outs[k].off) ? up(off_b[k]) : 0;
        sv[k] = scr, scr += host(outs[k].val) ? up(val_b[k]) : 0;
    }
    const size_t nb = (size_t)M.nv * 3 * sizeof(float);
    const size_t sx = scr;
    scr += (o->normals && host(o->xyz)) ? up(nb) : 0;
    const size_t sn = scr;
    scr += (o->normals && host(o->normals)) ? up(nb) : 0;

    cudaStream_t                s = (cudaStream_t)stream;
    std::lock_guard<std::mutex> lk(M.stage_mu);
    if (!M.sweep_streams[0]) {
        int least = 0, greatest = 0;
        RXG_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        for (int k = 0; k < 6; ++k) {
            // greatest is the numerically lowest; step towards least
            const int pr = greatest + k < least ? greatest + k : least;
            RXG_CUDA_TRY(cudaStreamCreateWithPriority(&M.sweep_streams[k], cudaStreamNonBlocking, pr));
        }
        for (cudaEvent_t& e : M.sweep_ev) RXG_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    if (!M.copy_stream) {
        RXG_CUDA_TRY(cudaStreamCreateWithFlags(&M.copy_stream, cudaStreamNonBlocking));
        for (cudaEvent_t& e : M.copy_ev) RXG_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    char* base = nullptr;
    if (scr) RXG_CUDA_TRY(scratch_alloc((void**)&base, scr, s));
    cudaEvent_t fork = M.sweep_ev[6], join = M.sweep_ev[7];
    // the enqueue; whatever it returns, `stream` then joins the copy stream
    // and frees the scratch in its order (nothing leaks on an error)
    auto enqueue = [&]() -> rxg_status {
        RXG_CUDA_TRY(cudaEventRecord(fork, s));
        RXG_CUDA_TRY(cudaStreamWaitEvent(M.copy_stream, fork, 0));
        for (int k = 0; k < 5; ++k) {
            const Out& q = outs[k];
            if (!q.val) continue;
            cudaStream_t ks = M.sweep_streams[k];
            RXG_CUDA_TRY(cudaStreamWaitEvent(ks, fork, 0));
            int32_t*   dof = !q.off ? nullptr : host(q.off) ? (int32_t*)(base + so[k]) : (int32_t*)q.off;
            int32_t*   dv  = host(q.val) ? (int32_t*)(base + sv[k]) : (int32_t*)q.val;
            rxg_status st  = launch_query(&M, q.op, dof, dv, ks);
            if (st) return st;
            RXG_CUDA_TRY(cudaEventRecord(M.sweep_ev[k], ks));
            RXG_CUDA_TRY(cudaStreamWaitEvent(s, M.sweep_ev[k], 0));
            RXG_CUDA_TRY(cudaStreamWaitEvent(M.copy_stream, M.sweep_ev[k], 0));
            if (host(q.off))
                RXG_CUDA_TRY(cudaMemcpyAsync(q.off, dof, off_b[k], cudaMemcpyDeviceToHost, M.copy_stream));
            if (host(q.val))
                RXG_CUDA_TRY(cudaMemcpyAsync(q.val, dv, val_b[k], cudaMemcpyDeviceToHost, M.copy_stream));
        }
        if (o->normals) {
            cudaStream_t ks = M.sweep_streams[5];
            RXG_CUDA_TRY(cudaStreamWaitEvent(ks, fork, 0));
            const float* dx = o->xyz;
            if (host(o->xyz)) {
                RXG_CUDA_TRY(cudaMemcpyAsync(base + sx, o->xyz, nb, cudaMemcpyHostToDevice, ks));
                dx = (const float*)(base + sx);
            }
            float*     dn = host(o->normals) ? (float*)(base + sn) : o->normals;
            rxg_status st = launch_normals(&M, o->weighting, dx, dn, ks, PatchRange{0, M.num_patches});
            if (st) return st;
            RXG_CUDA_TRY(cudaEventRecord(M.sweep_ev[5], ks));
            RXG_CUDA_TRY(cudaStreamWaitEvent(s, M.sweep_ev[5], 0));
            RXG_CUDA_TRY(cudaStreamWaitEvent(M.copy_stream, M.sweep_ev[5], 0));
            if (host(o->normals))
                RXG_CUDA_TRY(cudaMemcpyAsync(o->normals, dn, nb, cudaMemcpyDeviceToHost, M.copy_stream));
        }
        return RXG_OK;
    };
    const rxg_status st = enqueue();
    // `stream` waits for the copies; the scratch is freed in its order
    cudaError_t e = cudaEventRecord(join, M.copy_stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, join, 0);
    if (base && e == cudaSuccess) e = cudaFreeAsync(base, s);
    if (st) return st;
    return e == cudaSuccess ? RXG_OK : cuda_status(e, "rxg_query_sweep_ex join");
}

rxg_status rxg_device_check(void* stream) { return check_device_error((cudaStream_t)stream); }

rxg_status rxg_selftest_bounded_wait(void* stream)
{
    int* err = device_error_word();
    if (!err) {
        set_error("rxg_selftest_bounded_wait: no current CUDA device");
        return RXG_ERR_NO_DEVICE;
    }
    k_wait_selftest<<<1, 32, 0, (cudaStream_t)stream>>>(err, 100);
    RXG_CUDA_TRY(cudaGetLastError());
    return RXG_OK;
}

}  // extern "C"
