// rxg/query.cuh -- device-side queries over a mesh's patches (nvcc only).
//
// The generic query engine RXMesh applications are written against, over
// the patch layout librxg.so builds (rxg_mesh_device_context):
//   Query<blockThreads>     include/rxmesh/query.h:16-137, query.inl:106-260
//                           (dispatch / prologue / run_compute / epilogue,
//                           get_iterator, compute_vertex_valence)
//   Iterator<HandleT>       include/rxmesh/iterator.cuh:50-194 (size,
//                           operator[], local, front, back)
//   ShmemAllocator          include/rxmesh/kernels/shmem_allocator.cuh
//   for_each / run_kernel / prepare_launch_box / for_each_vertex ...
//                           include/rxmesh/rxmesh_static.h:205-594
//                           (members of RXMeshStatic in rxg/rxmesh.hpp)
// One CTA per patch.  The CTA copies its patch's EV and FE slices from the
// arena into shared memory (16-byte loads; every slice is 16-byte aligned
// and padded), builds the requested relation there (the transposes by a
// counting sort: shared-memory counts, a block scan, a scatter), and then
// calls the user's function for each source element with an iterator over
// that element's row.  An iterator entry is a 16-bit local index; operator[]
// turns it into a handle carrying the element's linear id: owned elements
// are the patch's base id plus the local index, ribbon (not-owned) elements
// are looked up in the patch's dense ribbon table, where RXMesh probes its
// LP hashtable (iterator.cuh:117-143, lp_hashtable.h:222-284).
//
// Rows of owned source elements are complete (every face, edge and vertex
// adjacent to an owned element is local to its patch).  With
// allow_not_owned, ribbon sources are visited too and their rows hold only
// the patch's part of their neighbourhood, as in RXMesh.
#pragma once

#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <tuple>
#include <type_traits>

#include "rxmesh.hpp"

namespace rxg {

constexpr uint16_t INVALID16 = 0xFFFFu;

namespace detail {

// one patch record (rxg_mesh_patches' layout, 64 bytes)
struct PatchRec
{
    int32_t nVo, nVl, nEo, nEl, nFo, nFl;
    int32_t v_base, e_base, f_base, vv_base, vf_base;
    int32_t ev_off, fe_off, rv_off, re_off, rf_off;
};

__device__ __forceinline__ PatchRec load_patch(const Context& ctx, uint32_t p)
{
    const int4* src = reinterpret_cast<const int4*>(ctx.c.patch_hdr + 16 * (size_t)p);
    PatchRec    r;
    int4*       d = reinterpret_cast<int4*>(&r);
#pragma unroll
    for (int i = 0; i < 4; ++i) d[i] = __ldg(src + i);
    return r;
}

// local index -> linear id for one element type of one patch
struct Resolver
{
    int32_t         n_owned = 0, n_local = 0, base = 0;
    const uint32_t* rib     = nullptr;
    __device__ __forceinline__ int32_t operator()(uint32_t l) const
    {
        if ((int32_t)l < n_owned) return base + (int32_t)l;
        if ((int32_t)l < n_local) return (int32_t)__ldg(rib + (l - (uint32_t)n_owned));
        return -1;
    }
};

__device__ __forceinline__ Resolver resolver(const uint32_t* arena, const PatchRec& h, int elem)
{
    Resolver r;
    if (elem == RXG_ELEM_VERTEX) {
        r.n_owned = h.nVo, r.n_local = h.nVl, r.base = h.v_base, r.rib = arena + h.rv_off;
    } else if (elem == RXG_ELEM_EDGE) {
        r.n_owned = h.nEo, r.n_local = h.nEl, r.base = h.e_base, r.rib = arena + h.re_off;
    } else {
        r.n_owned = h.nFo, r.n_local = h.nFl, r.base = h.f_base, r.rib = arena + h.rf_off;
    }
    return r;
}

// argument types of a (non-generic) lambda or functor (the reference's
// FunctionTraits, util/meta.h): compute_op(handle, iterator)
template <typename T>
struct FunctionTraits : FunctionTraits<decltype(&T::operator())>
{
};
template <typename C, typename R, typename... A>
struct FunctionTraits<R (C::*)(A...) const>
{
    template <size_t i>
    using arg = std::decay_t<std::tuple_element_t<i, std::tuple<A...>>>;
};
template <typename C, typename R, typename... A>
struct FunctionTraits<R (C::*)(A...)>
{
    template <size_t i>
    using arg = std::decay_t<std::tuple_element_t<i, std::tuple<A...>>>;
};

// source / output element types of each query (InputHandle / OutputIterator)
template <Op op>
struct OpTraits;
template <>
struct OpTraits<Op::VV> { static constexpr int src = RXG_ELEM_VERTEX, out = RXG_ELEM_VERTEX; };
template <>
struct OpTraits<Op::VE> { static constexpr int src = RXG_ELEM_VERTEX, out = RXG_ELEM_EDGE; };
template <>
struct OpTraits<Op::VF> { static constexpr int src = RXG_ELEM_VERTEX, out = RXG_ELEM_FACE; };
template <>
struct OpTraits<Op::FV> { static constexpr int src = RXG_ELEM_FACE, out = RXG_ELEM_VERTEX; };
template <>
struct OpTraits<Op::FE> { static constexpr int src = RXG_ELEM_FACE, out = RXG_ELEM_EDGE; };
template <>
struct OpTraits<Op::FF> { static constexpr int src = RXG_ELEM_FACE, out = RXG_ELEM_FACE; };
template <>
struct OpTraits<Op::EV> { static constexpr int src = RXG_ELEM_EDGE, out = RXG_ELEM_VERTEX; };
template <>
struct OpTraits<Op::EF> { static constexpr int src = RXG_ELEM_EDGE, out = RXG_ELEM_FACE; };
template <>
struct OpTraits<Op::EVDiamond> { static constexpr int src = RXG_ELEM_EDGE, out = RXG_ELEM_VERTEX; };
template <>
struct OpTraits<Op::EE> { static constexpr int src = RXG_ELEM_EDGE, out = RXG_ELEM_EDGE; };

// Exclusive scan of s[0..n) in place (any n), returns the total.
template <uint32_t BT>
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t* s, int n)
{
    __shared__ uint32_t s_warp[32];
    const int      tid   = (int)threadIdx.x;
    const int      chunk = (n + (int)BT - 1) / (int)BT;
    const int      beg = min(n, tid * chunk), end = min(n, beg + chunk);
    uint32_t       sum = 0;
    for (int i = beg; i < end; ++i) sum += s[i];
    uint32_t  x    = sum;
    const int lane = tid & 31, warp = tid >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < (int)(BT / 32) ? s_warp[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < (int)(BT / 32)) s_warp[lane] = w;
    }
    __syncthreads();
    uint32_t       run   = x - sum + (warp > 0 ? s_warp[warp - 1] : 0u);
    const uint32_t total = s_warp[BT / 32 - 1];
    for (int i = beg; i < end; ++i) {
        const uint32_t v = s[i];
        s[i]             = run;
        run += v;
    }
    __syncthreads();
    return total;
}

template <int ELEM>
struct HandleOf;
template <>
struct HandleOf<RXG_ELEM_VERTEX> { using type = VertexHandle; };
template <>
struct HandleOf<RXG_ELEM_EDGE> { using type = EdgeHandle; };
template <>
struct HandleOf<RXG_ELEM_FACE> { using type = FaceHandle; };

}  // namespace detail

// Iterator over one source element's row (Iterator<HandleT>,
// iterator.cuh:50-194): size(), operator[] (a handle with the neighbour's
// linear id; invalid past the end or for a missing EVDiamond vertex),
// local(i) (the 16-bit local index), front(), back().
template <typename HandleT>
struct Iterator
{
    using Handle = HandleT;
    __device__ __forceinline__ Iterator() {}
    __device__ __forceinline__ Iterator(uint16_t local_id, const uint16_t* vals, uint32_t begin,
                                        uint32_t end, const detail::Resolver& res)
        : m_local_id(local_id), m_vals(vals), m_begin(begin), m_end(end), m_res(res)
    {
    }
    __device__ __forceinline__ uint16_t size() const { return (uint16_t)(m_end - m_begin); }
    __device__ __forceinline__ HandleT  operator[](uint16_t i) const
    {
        if (m_begin + i >= m_end) return HandleT();
        const uint16_t l = m_vals[m_begin + i];
        if (l == INVALID16) return HandleT();
        const int32_t id = m_res(l);
        return id >= 0 ? HandleT(id) : HandleT();
    }
    __device__ __forceinline__ uint16_t local(uint16_t i) const
    {
        return m_begin + i < m_end ? m_vals[m_begin + i] : INVALID16;
    }
    __device__ __forceinline__ HandleT  front() const { return (*this)[0]; }
    __device__ __forceinline__ HandleT  back() const { return size() ? (*this)[size() - 1] : HandleT(); }
    // local index of the source element in its patch
    __device__ __forceinline__ uint16_t local_id() const { return m_local_id; }

   private:
    uint16_t         m_local_id = INVALID16;
    const uint16_t*  m_vals     = nullptr;
    uint32_t         m_begin = 0, m_end = 0;
    detail::Resolver m_res;
};
using VertexIterator = Iterator<VertexHandle>;
using EdgeIterator   = Iterator<EdgeHandle>;
using FaceIterator   = Iterator<FaceHandle>;

// Bump allocator over the kernel's dynamic shared memory (ShmemAllocator,
// kernels/shmem_allocator.cuh).  Every thread holds its own copy and makes
// the same calls, so all agree on the layout.  Allocations are 16-byte
// aligned; dealloc releases the most recent allocations (a stack).
struct ShmemAllocator
{
    __device__ __forceinline__ ShmemAllocator()
    {
        extern __shared__ __align__(16) char rxg_dyn_smem[];
        m_base = m_ptr = rxg_dyn_smem;
    }
    __device__ __forceinline__ char* alloc(uint32_t num_bytes)
    {
        char* r = m_ptr;
        m_ptr += (num_bytes + 15u) & ~15u;
        return r;
    }
    template <typename T>
    __device__ __forceinline__ T* alloc(uint32_t count)
    {
        return reinterpret_cast<T*>(alloc(count * (uint32_t)sizeof(T)));
    }
    __device__ __forceinline__ void dealloc(uint32_t num_bytes) { m_ptr -= (num_bytes + 15u) & ~15u; }
    template <typename T>
    __device__ __forceinline__ void dealloc(uint32_t count)
    {
        dealloc(count * (uint32_t)sizeof(T));
    }
    __device__ __forceinline__ uint32_t get_allocated_size_bytes() const
    {
        return (uint32_t)(m_ptr - m_base);
    }
    __device__ __forceinline__ void release_to(uint32_t bytes) { m_ptr = m_base + bytes; }

   private:
    char* m_base;
    char* m_ptr;
};

// Per-CTA query over one patch (Query<blockThreads>, query.h:16-137).
template <uint32_t blockThreads>
struct Query
{
    static_assert(blockThreads % 32 == 0 && blockThreads <= 1024, "blockThreads: 32..1024, whole warps");

    __device__ __forceinline__ Query(const Query&)            = delete;
    __device__ __forceinline__ Query& operator=(const Query&) = delete;

    __device__ __forceinline__ Query(const Context& context, const uint32_t pid = blockIdx.x)
        : m_arena(context.c.arena), m_pid(pid)
    {
        m_p = detail::load_patch(context, pid);
    }

    __device__ __forceinline__ int get_patch_id() const { return (int)m_pid; }
    __device__ __forceinline__ uint32_t num_owned_vertices() const { return (uint32_t)m_p.nVo; }
    __device__ __forceinline__ uint32_t num_owned_edges() const { return (uint32_t)m_p.nEo; }
    __device__ __forceinline__ uint32_t num_owned_faces() const { return (uint32_t)m_p.nFo; }

    // valence of every local vertex from the patch's edges (exact for
    // owned vertices, whose edges are all local); compute_vertex_valence /
    // vertex_valence of query.h:36-54
    __device__ void compute_vertex_valence(cooperative_groups::thread_block& block,
                                           ShmemAllocator&                   shrd_alloc)
    {
        m_s_valence = shrd_alloc.alloc<uint32_t>((uint32_t)m_p.nVl);
        for (int v = threadIdx.x; v < m_p.nVl; v += blockThreads) m_s_valence[v] = 0;
        block.sync();
        const uint32_t* ev = m_arena + m_p.ev_off;
        for (int e = threadIdx.x; e < m_p.nEl; e += blockThreads) {
            const uint32_t w = __ldg(ev + e);
            atomicAdd(&m_s_valence[w & 0xffffu], 1u);
            atomicAdd(&m_s_valence[w >> 16], 1u);
        }
        block.sync();
    }
    __device__ __forceinline__ uint16_t vertex_valence(uint16_t v) const
    {
        return (uint16_t)m_s_valence[v];
    }
    __device__ __forceinline__ uint16_t vertex_valence(VertexHandle vh) const
    {
        const int32_t l = vh.linear_id() - m_p.v_base;
        return (l >= 0 && l < m_p.nVo) ? (uint16_t)m_s_valence[l] : (uint16_t)0;
    }

    // The whole block calls dispatch: the query, then compute_op(handle,
    // iterator) for every owned source element (Query::dispatch,
    // query.h:56-63, query.inl:126-156).
    template <Op op, typename computeT>
    __device__ void dispatch(cooperative_groups::thread_block& block, ShmemAllocator& shrd_alloc,
                             computeT compute_op, const bool oriented = false)
    {
        prologue<op>(block, shrd_alloc, oriented, false);
        run_typed<typename detail::HandleOf<detail::OpTraits<op>::src>::type,
                  typename detail::HandleOf<detail::OpTraits<op>::out>::type>(compute_op);
        epilogue(block, shrd_alloc);
    }
    // With an active-set predicate (query.h:65-75): compute_op only for
    // sources with compute_active_set(handle) true; allow_not_owned lets
    // ribbon sources of the patch be active (their rows are the patch's
    // part of the neighbourhood).
    template <Op op, typename computeT, typename activeSetT>
    __device__ void dispatch(cooperative_groups::thread_block& block, ShmemAllocator& shrd_alloc,
                             computeT compute_op, activeSetT compute_active_set,
                             const bool oriented = false, const bool allow_not_owned = false)
    {
        prologue<op>(block, shrd_alloc, oriented, allow_not_owned);
        using SrcH = typename detail::HandleOf<detail::OpTraits<op>::src>::type;
        using OutH = typename detail::HandleOf<detail::OpTraits<op>::out>::type;
        for (uint32_t s = threadIdx.x; s < m_num_src; s += blockThreads) {
            const SrcH h = source_handle<SrcH>(s);
            if (!compute_active_set(h)) continue;
            Iterator<OutH> it = get_iterator<Iterator<OutH>>((uint16_t)s);
            compute_op(h, it);
        }
        epilogue(block, shrd_alloc);
    }

    // Run query `op` and keep its rows in shared memory (prologue,
    // query.h:78-98).  oriented applies to Op::VV: each owned vertex's row
    // lists its neighbours in the rotational order of its faces (a boundary
    // vertex's row runs from one boundary neighbour to the other), the
    // order orient_edges_around_vertices gives (rxmesh_queries.cuh:376-499).
    template <Op op>
    __device__ void prologue(cooperative_groups::thread_block& block, ShmemAllocator& shrd_alloc,
                             const bool oriented = false, const bool allow_not_owned = true)
    {
        constexpr int SRC = detail::OpTraits<op>::src;
        constexpr int OUT = detail::OpTraits<op>::out;
        m_shmem_before    = shrd_alloc.get_allocated_size_bytes();
        m_out             = OUT;
        m_src             = SRC;
        m_s_offset        = nullptr;
        m_stride          = 0;
        const detail::PatchRec& h = m_p;
        m_num_src = (uint32_t)(SRC == RXG_ELEM_VERTEX ? (allow_not_owned ? h.nVl : h.nVo)
                               : SRC == RXG_ELEM_EDGE ? (allow_not_owned ? h.nEl : h.nEo)
                                                      : (allow_not_owned ? h.nFl : h.nFo));
        // EV slice: every op but FE / EF / FF / EE; FE slice: every op but
        // EV, VE and (unoriented) VV
        constexpr bool need_ev = op != Op::FE && op != Op::EF && op != Op::FF && op != Op::EE;
        constexpr bool need_fe = op != Op::EV && op != Op::VV && op != Op::VE;
        const bool     want_fe = need_fe || (op == Op::VV && oriented);
        uint32_t*      s_ev    = need_ev ? shrd_alloc.alloc<uint32_t>((uint32_t)h.nEl) : nullptr;
        uint16_t*      s_fe    = want_fe ? shrd_alloc.alloc<uint16_t>((uint32_t)(3 * h.nFl + 1)) : nullptr;
        if (need_ev) copy16(s_ev, m_arena + h.ev_off, (uint32_t)h.nEl);
        if (want_fe) copy16(reinterpret_cast<uint32_t*>(s_fe), m_arena + h.fe_off,
                            (uint32_t)((3 * h.nFl + 1) / 2));
        block.sync();

        if constexpr (op == Op::EV) {
            m_s_value = reinterpret_cast<uint16_t*>(s_ev);  // (a, b) u16 pairs
            m_stride  = 2;
        } else if constexpr (op == Op::FE) {
            for (int i = threadIdx.x; i < 3 * h.nFl; i += blockThreads) s_fe[i] >>= 1;
            block.sync();
            m_s_value = s_fe;
            m_stride  = 3;
        } else if constexpr (op == Op::FV) {
            m_s_value = shrd_alloc.alloc<uint16_t>((uint32_t)(3 * h.nFl));
            for (int i = threadIdx.x; i < 3 * h.nFl; i += blockThreads)
                m_s_value[i] = face_vertex(s_fe, s_ev, i / 3, i % 3);
            block.sync();
            m_stride = 3;
        } else if constexpr (op == Op::EVDiamond) {
            m_s_value = shrd_alloc.alloc<uint16_t>((uint32_t)(4 * h.nEl));
            for (int e = threadIdx.x; e < h.nEl; e += blockThreads) {
                const uint32_t w     = s_ev[e];
                m_s_value[4 * e + 0] = (uint16_t)(w & 0xffffu);
                m_s_value[4 * e + 1] = INVALID16;
                m_s_value[4 * e + 2] = (uint16_t)(w >> 16);
                m_s_value[4 * e + 3] = INVALID16;
            }
            block.sync();
            // the vertex opposite edge k of a face is its corner k+2; a face
            // traversing the edge as stored (dir 0) fills slot 1, else slot 3
            for (int i = threadIdx.x; i < 3 * h.nFl; i += blockThreads) {
                const uint32_t fe = s_fe[i];
                const int      f = i / 3, k = i - 3 * (i / 3);
                m_s_value[4 * (fe >> 1) + 1 + 2 * (fe & 1u)] = face_vertex(s_fe, s_ev, f, (k + 2) % 3);
            }
            block.sync();
            m_stride = 4;
        } else if constexpr (op == Op::EE) {
            m_s_value = shrd_alloc.alloc<uint16_t>((uint32_t)(4 * h.nEl));
            for (int i = threadIdx.x; i < 4 * h.nEl; i += blockThreads) m_s_value[i] = INVALID16;
            block.sync();
            // beside edge k of a face lie the face's edges k+1 (next) and k+2
            // (previous); the face traversing the edge as stored (dir 0)
            // fills slots 0 and 1, the other one slots 2 and 3
            for (int i = threadIdx.x; i < 3 * h.nFl; i += blockThreads) {
                const uint32_t fe = s_fe[i];
                const int      f = i / 3, k = i - 3 * (i / 3);
                uint16_t*      q = m_s_value + 4 * (fe >> 1) + 2 * (fe & 1u);
                q[0]             = (uint16_t)(s_fe[3 * f + (k + 1) % 3] >> 1);
                q[1]             = (uint16_t)(s_fe[3 * f + (k + 2) % 3] >> 1);
            }
            block.sync();
            m_stride = 4;
        } else if constexpr (op == Op::VV || op == Op::VE) {
            build_vertex_edges<op == Op::VV>(block, shrd_alloc, s_ev);
            if (op == Op::VV && oriented) orient(block, shrd_alloc, s_ev, s_fe);
        } else if constexpr (op == Op::VF) {
            build_vertex_faces(block, shrd_alloc, s_ev, s_fe, m_s_offset, m_s_value);
        } else if constexpr (op == Op::EF || op == Op::FF) {
            uint32_t* ef_off = shrd_alloc.alloc<uint32_t>((uint32_t)h.nEl + 1);
            uint16_t* ef_val = shrd_alloc.alloc<uint16_t>((uint32_t)(3 * h.nFl));
            for (int e = threadIdx.x; e <= h.nEl; e += blockThreads) ef_off[e] = 0;
            block.sync();
            for (int i = threadIdx.x; i < 3 * h.nFl; i += blockThreads) atomicAdd(&ef_off[s_fe[i] >> 1], 1u);
            block.sync();
            detail::block_exclusive_scan<blockThreads>(ef_off, h.nEl + 1);
            uint32_t* pos = shrd_alloc.alloc<uint32_t>((uint32_t)h.nEl);
            for (int e = threadIdx.x; e < h.nEl; e += blockThreads) pos[e] = ef_off[e];
            block.sync();
            for (int i = threadIdx.x; i < 3 * h.nFl; i += blockThreads)
                ef_val[atomicAdd(&pos[s_fe[i] >> 1], 1u)] = (uint16_t)(i / 3);
            block.sync();
            shrd_alloc.dealloc<uint32_t>((uint32_t)h.nEl);
            if constexpr (op == Op::EF) {
                m_s_offset = ef_off;
                m_s_value  = ef_val;
            } else {
                // faces sharing an edge with f: every other face of f's edges
                uint32_t* ff_off = shrd_alloc.alloc<uint32_t>((uint32_t)h.nFl + 1);
                for (int f = threadIdx.x; f < h.nFl; f += blockThreads) {
                    uint32_t c = 0;
                    for (int k = 0; k < 3; ++k) {
                        const uint32_t e = s_fe[3 * f + k] >> 1;
                        c += ef_off[e + 1] - ef_off[e] - 1;
                    }
                    ff_off[f] = c;
                }
                if (threadIdx.x == 0) ff_off[h.nFl] = 0;
                block.sync();
                const uint32_t total = detail::block_exclusive_scan<blockThreads>(ff_off, h.nFl + 1);
                uint16_t*      ff_val = shrd_alloc.alloc<uint16_t>(total);
                for (int f = threadIdx.x; f < h.nFl; f += blockThreads) {
                    uint32_t p = ff_off[f];
                    for (int k = 0; k < 3; ++k) {
                        const uint32_t e = s_fe[3 * f + k] >> 1;
                        for (uint32_t j = ef_off[e]; j < ef_off[e + 1]; ++j)
                            if (ef_val[j] != (uint16_t)f) ff_val[p++] = ef_val[j];
                    }
                }
                block.sync();
                m_s_offset = ff_off;
                m_s_value  = ff_val;
            }
        }
    }

    // compute_op(handle, iterator) for every source element of the last
    // prologue (run_compute, query.h:100-106); the handle and iterator
    // types are compute_op's parameter types, which must match the query
    template <typename computeT>
    __device__ void run_compute(cooperative_groups::thread_block& block, computeT compute_op)
    {
        (void)block;
        using Tr   = detail::FunctionTraits<computeT>;
        using SrcH = typename Tr::template arg<0>;
        using OutH = typename Tr::template arg<1>::Handle;
        run_typed<SrcH, OutH>(compute_op);
    }

    // iterator over the row of source element local_id (get_iterator,
    // query.h:108-113); IteratorT must match the last prologue's output type
    template <typename IteratorT>
    __device__ __forceinline__ IteratorT get_iterator(uint16_t local_id) const
    {
        const uint32_t b = m_s_offset ? m_s_offset[local_id] : (uint32_t)local_id * m_stride;
        const uint32_t e = m_s_offset ? m_s_offset[local_id + 1] : b + m_stride;
        return IteratorT(local_id, m_s_value, b, e, detail::resolver(m_arena, m_p, m_out));
    }

    // release the query's shared memory (epilogue, query.h:115-120)
    __device__ void epilogue(cooperative_groups::thread_block& block, ShmemAllocator& shrd_alloc)
    {
        block.sync();
        shrd_alloc.release_to(m_shmem_before);
    }

   private:
    // 16-byte copy of `words` words (the arena slice is padded to 16 bytes)
    __device__ __forceinline__ static void copy16(uint32_t* dst, const uint32_t* src, uint32_t words)
    {
        const uint32_t n4 = (words + 3) / 4;
        const uint4*   s  = reinterpret_cast<const uint4*>(src);
        uint4*         d  = reinterpret_cast<uint4*>(dst);
        for (uint32_t i = threadIdx.x; i < n4; i += blockThreads) d[i] = __ldg(s + i);
    }
    // corner k of local face f (FE: edge<<1|dir; EV: a | b<<16)
    __device__ __forceinline__ static uint16_t face_vertex(const uint16_t* fe16, const uint32_t* ev,
                                                           int f, int k)
    {
        const uint32_t fe = fe16[3 * f + k];
        const uint32_t w  = ev[fe >> 1];
        return (uint16_t)((fe & 1u) ? (w >> 16) : (w & 0xffffu));
    }
    template <typename SrcH>
    __device__ __forceinline__ SrcH source_handle(uint32_t s) const
    {
        const int32_t id = detail::resolver(m_arena, m_p, m_src)(s);
        return id >= 0 ? SrcH(id) : SrcH();
    }
    template <typename SrcH, typename OutH, typename computeT>
    __device__ __forceinline__ void run_typed(computeT& compute_op)
    {
        for (uint32_t s = threadIdx.x; s < m_num_src; s += blockThreads) {
            Iterator<OutH> it = get_iterator<Iterator<OutH>>((uint16_t)s);
            compute_op(source_handle<SrcH>(s), it);
        }
    }
    // VV (VVAL: the other end) or VE (the edge) rows of every local vertex
    template <bool VVAL>
    __device__ void build_vertex_edges(cooperative_groups::thread_block& block,
                                       ShmemAllocator& shrd_alloc, const uint32_t* s_ev)
    {
        const int nV = m_p.nVl, nE = m_p.nEl;
        m_s_offset   = shrd_alloc.alloc<uint32_t>((uint32_t)nV + 1);
        m_s_value    = shrd_alloc.alloc<uint16_t>((uint32_t)(2 * nE));
        for (int v = threadIdx.x; v <= nV; v += blockThreads) m_s_offset[v] = 0;
        block.sync();
        for (int e = threadIdx.x; e < nE; e += blockThreads) {
            const uint32_t w = s_ev[e];
            atomicAdd(&m_s_offset[w & 0xffffu], 1u);
            atomicAdd(&m_s_offset[w >> 16], 1u);
        }
        block.sync();
        detail::block_exclusive_scan<blockThreads>(m_s_offset, nV + 1);
        uint32_t* pos = shrd_alloc.alloc<uint32_t>((uint32_t)nV);
        for (int v = threadIdx.x; v < nV; v += blockThreads) pos[v] = m_s_offset[v];
        block.sync();
        for (int e = threadIdx.x; e < nE; e += blockThreads) {
            const uint32_t w = s_ev[e], a = w & 0xffffu, b = w >> 16;
            m_s_value[atomicAdd(&pos[a], 1u)] = VVAL ? (uint16_t)b : (uint16_t)e;
            m_s_value[atomicAdd(&pos[b], 1u)] = VVAL ? (uint16_t)a : (uint16_t)e;
        }
        block.sync();
        shrd_alloc.dealloc<uint32_t>((uint32_t)nV);
    }
    // VF rows of every local vertex into (off, val), allocated here
    __device__ void build_vertex_faces(cooperative_groups::thread_block& block,
                                       ShmemAllocator& shrd_alloc, const uint32_t* s_ev,
                                       const uint16_t* s_fe, uint32_t*& off, uint16_t*& val)
    {
        const int nV = m_p.nVl, nF = m_p.nFl;
        off          = shrd_alloc.alloc<uint32_t>((uint32_t)nV + 1);
        val          = shrd_alloc.alloc<uint16_t>((uint32_t)(3 * nF));
        for (int v = threadIdx.x; v <= nV; v += blockThreads) off[v] = 0;
        block.sync();
        for (int i = threadIdx.x; i < 3 * nF; i += blockThreads)
            atomicAdd(&off[face_vertex(s_fe, s_ev, i / 3, i % 3)], 1u);
        block.sync();
        detail::block_exclusive_scan<blockThreads>(off, nV + 1);
        uint32_t* pos = shrd_alloc.alloc<uint32_t>((uint32_t)nV);
        for (int v = threadIdx.x; v < nV; v += blockThreads) pos[v] = off[v];
        block.sync();
        for (int i = threadIdx.x; i < 3 * nF; i += blockThreads)
            val[atomicAdd(&pos[face_vertex(s_fe, s_ev, i / 3, i % 3)], 1u)] = (uint16_t)(i / 3);
        block.sync();
        shrd_alloc.dealloc<uint32_t>((uint32_t)nV);
    }
    // Reorder each owned vertex's VV row into the rotational order of its
    // faces: face (v, a, b) is followed by the face (v, b, c).  An interior
    // row starts at the neighbour after v in its first-listed face, a
    // boundary row at the neighbour whose edge has a face on one side only.
    // Rows of non-manifold fans are left as they are.
    __device__ void orient(cooperative_groups::thread_block& block, ShmemAllocator& shrd_alloc,
                           const uint32_t* s_ev, const uint16_t* s_fe)
    {
        uint32_t* vf_off;
        uint16_t* vf_val;
        const uint32_t mark = shrd_alloc.get_allocated_size_bytes();
        build_vertex_faces(block, shrd_alloc, s_ev, s_fe, vf_off, vf_val);
        for (int v = threadIdx.x; v < m_p.nVo; v += blockThreads) {
            const uint32_t fb = vf_off[v], k = vf_off[v + 1] - fb;
            const uint32_t rb = m_s_offset[v], rl = m_s_offset[v + 1] - rb;
            if (k == 0 || (rl != k && rl != k + 1)) continue;
            // next (a) and previous (b) corner of v in each face
            auto ab = [&](uint32_t j, uint16_t& a, uint16_t& b) {
                const int f = vf_val[fb + j];
                const int c = face_vertex(s_fe, s_ev, f, 0) == v ? 0 : (face_vertex(s_fe, s_ev, f, 1) == v ? 1 : 2);
                a           = face_vertex(s_fe, s_ev, f, (c + 1) % 3);
                b           = face_vertex(s_fe, s_ev, f, (c + 2) % 3);
            };
            uint32_t start = k;  // boundary start: a face whose a is no face's b
            for (uint32_t i = 0; i < k && start == k; ++i) {
                uint16_t ai, bi;
                ab(i, ai, bi);
                bool found = false;
                for (uint32_t j = 0; j < k && !found; ++j) {
                    uint16_t aj, bj;
                    ab(j, aj, bj);
                    found = bj == ai;
                }
                if (!found) start = i;
            }
            const bool bnd = start < k;
            if (!bnd) start = 0;
            if (rl != k + (bnd ? 1u : 0u)) continue;
            // walk into registers first; write back only a complete fan
            uint32_t cur = start, n = 0;
            bool     ok  = true;
            uint16_t a0, b0;
            ab(cur, a0, b0);
            // the row is rewritten in place after the walk is known to close
            uint16_t* row = m_s_value + rb;
            uint16_t  first = a0;
            uint32_t  visited = 0;
            // first pass: check
            {
                uint32_t c = start;
                while (true) {
                    ++visited;
                    uint16_t a, b;
                    ab(c, a, b);
                    uint32_t nxt = k;
                    for (uint32_t j = 0; j < k; ++j) {
                        uint16_t aj, bj;
                        ab(j, aj, bj);
                        if (aj == b) {
                            nxt = j;
                            break;
                        }
                    }
                    if (nxt == k || nxt == start) break;
                    if (visited >= k) {
                        ok = false;
                        break;
                    }
                    c = nxt;
                }
                if (visited != k) ok = false;
            }
            if (!ok) continue;
            // second pass: write
            row[n++] = first;
            while (true) {
                uint16_t a, b;
                ab(cur, a, b);
                uint32_t nxt = k;
                for (uint32_t j = 0; j < k; ++j) {
                    uint16_t aj, bj;
                    ab(j, aj, bj);
                    if (aj == b) {
                        nxt = j;
                        break;
                    }
                }
                if (nxt == k || nxt == start) {
                    if (bnd) row[n++] = b;
                    break;
                }
                row[n++] = b;
                cur      = nxt;
            }
        }
        block.sync();
        shrd_alloc.release_to(mark);
    }

    const uint32_t*  m_arena;
    uint32_t         m_pid;
    detail::PatchRec m_p;
    uint32_t         m_shmem_before = 0;
    uint32_t         m_num_src      = 0;
    int              m_src = 0, m_out = 0;
    uint32_t         m_stride    = 0;
    uint32_t*        m_s_offset  = nullptr;
    uint16_t*        m_s_value   = nullptr;
    uint32_t*        m_s_valence = nullptr;
};

namespace detail {

inline size_t pad16(size_t b) { return (b + 15) & ~size_t(15); }

// dynamic shared memory of Query::prologue<op> for the largest patch
// (calc_shared_memory, rxmesh_static.inl:548-741, for this layout)
inline size_t query_smem_bytes(Op op, const rxg_device_context& c, bool oriented)
{
    const size_t V = (size_t)c.max_local_vertices, E = (size_t)c.max_local_edges,
                 F = (size_t)c.max_local_faces;
    const size_t ff   = (size_t)(c.max_face_adjacent_faces > 3 ? c.max_face_adjacent_faces : 3);
    const size_t ev   = pad16(4 * E), fe = pad16(2 * (3 * F + 1));
    const size_t offV = pad16(4 * (V + 1)), offE = pad16(4 * (E + 1)), offF = pad16(4 * (F + 1));
    const size_t posV = pad16(4 * V), posE = pad16(4 * E);
    const size_t vals3F = pad16(2 * 3 * F);
    switch (op) {
        case Op::VV:
            if (oriented) return ev + fe + offV + pad16(4 * E) + offV + vals3F + posV;
            return ev + offV + pad16(4 * E) + posV;
        case Op::VE: return ev + offV + pad16(4 * E) + posV;
        case Op::VF: return ev + fe + offV + vals3F + posV;
        case Op::FV: return ev + fe + vals3F;
        case Op::FE: return fe;
        case Op::EV: return ev;
        case Op::EF: return fe + offE + vals3F + posE;
        case Op::FF: {
            const size_t tail = offF + pad16(2 * F * ff);
            return fe + offE + vals3F + (tail > posE ? tail : posE);
        }
        case Op::EVDiamond: return ev + fe + pad16(8 * E);
        case Op::EE: return fe + pad16(8 * E);
    }
    return 0;
}

template <uint32_t blockThreads, Op op, typename LambdaT>
__global__ void __launch_bounds__(blockThreads)
    query_kernel(const Context context, const bool oriented, LambdaT user_lambda)
{
    auto           block = cooperative_groups::this_thread_block();
    ShmemAllocator shrd_alloc;
    Query<blockThreads> query(context);
    query.template dispatch<op>(block, shrd_alloc, user_lambda, oriented);
}

template <typename HandleT, typename LambdaT>
__global__ void __launch_bounds__(256) for_each_element_kernel(int64_t n, LambdaT apply)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        apply(HandleT((int32_t)i));
}

template <uint32_t blockThreads>
void prepare_launch_box_impl(const RXMeshStatic& rx, const std::vector<Op>& ops,
                             LaunchBox<blockThreads>& lb, const void* kernel, bool oriented,
                             bool with_vertex_valence, bool is_concurrent,
                             const std::function<size_t(uint32_t, uint32_t, uint32_t)>& user_shmem)
{
    const Context ctx = rx.get_context();
    size_t        q   = 0;
    for (Op op : ops) {
        const size_t b = query_smem_bytes(op, ctx.c, oriented);
        q              = is_concurrent ? q + b : (b > q ? b : q);
    }
    size_t smem = q + 256;  // + slack for the user's own small allocations
    if (with_vertex_valence) smem += pad16(4 * (size_t)ctx.c.max_local_vertices);
    if (user_shmem)
        smem += user_shmem((uint32_t)ctx.c.max_local_vertices, (uint32_t)ctx.c.max_local_edges,
                           (uint32_t)ctx.c.max_local_faces);
    int optin = 0;
    check_cuda(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx.c.device),
               "cudaDeviceGetAttribute");
    if (smem > (size_t)optin)
        throw Error(RXG_ERR_PATCH_LIMIT, "query needs more shared memory per patch than a CTA has");
    if (kernel && smem > 48 * 1024)
        check_cuda(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                   "cudaFuncSetAttribute");
    lb.blocks         = (uint32_t)ctx.c.num_patches;
    lb.num_threads    = blockThreads;
    lb.smem_bytes_dyn = (uint32_t)smem;
}

template <Op op, uint32_t blockThreads, typename LambdaT>
void for_each_impl(const RXMeshStatic& rx, const LaunchBox<blockThreads>* lb_in, const LambdaT& f,
                   bool oriented, cudaStream_t stream)
{
    const void*             kern = (const void*)query_kernel<blockThreads, op, LambdaT>;
    LaunchBox<blockThreads> lb;
    if (lb_in)
        lb = *lb_in;
    else
        prepare_launch_box_impl<blockThreads>(rx, {op}, lb, kern, oriented, false, false, nullptr);
    if (lb_in && lb.smem_bytes_dyn > 48 * 1024)
        check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)lb.smem_bytes_dyn),
                   "cudaFuncSetAttribute");
    if (lb.blocks == 0) return;
    query_kernel<blockThreads, op, LambdaT>
        <<<lb.blocks, lb.num_threads, lb.smem_bytes_dyn, stream>>>(rx.get_context(), oriented, f);
    check_cuda(cudaGetLastError(), "for_each launch");
}

template <typename HandleT, typename LambdaT>
void for_each_element_device(const RXMeshStatic& rx, const LambdaT& f, cudaStream_t stream)
{
    const int64_t n = HandleT::kElem == RXG_ELEM_VERTEX ? rx.get_num_vertices()
                      : HandleT::kElem == RXG_ELEM_EDGE ? rx.get_num_edges()
                                                        : rx.get_num_faces();
    if (n == 0) return;
    const int64_t blocks = (n + 255) / 256;
    for_each_element_kernel<HandleT, LambdaT>
        <<<(unsigned)(blocks < 152 * 16 ? blocks : 152 * 16), 256, 0, stream>>>(n, f);
    check_cuda(cudaGetLastError(), "for_each_vertex/edge/face launch");
}

}  // namespace detail
}  // namespace rxg
