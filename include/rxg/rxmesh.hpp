// rxg/rxmesh.hpp -- C++ host facade over the C ABI of librxg.so (rxg.h).
//
// Keeps the names and argument meaning of RXMesh's host API for the hot path
// so that C++ callers switch with few edits:
//   RXMeshStatic            include/rxmesh/rxmesh_static.h:61-112
//   Op                      include/rxmesh/types.h
//   DenseMatrix<T>          include/rxmesh/matrix/dense_matrix.h (device
//                           storage; row-major here, ColMajor by default there)
//   SparseMatrix<T>         include/rxmesh/matrix/sparse_matrix.h:77
//   CGSolver / PCGSolver    include/rxmesh/matrix/cg_solver.h:17-130,
//                           matrix/pcg_solver.h:14-213
//   DiffScalarProblem       include/rxmesh/diff/diff_scalar_problem.h:310-321
//                           (ARAP term only)
//   VertexHandle / EdgeHandle / FaceHandle   include/rxmesh/handle.h:19-144
//   VertexAttribute<T> ...  include/rxmesh/attribute.h (add_*_attribute,
//                           rxmesh_static.h:608-793)
//   Context, LaunchBox      include/rxmesh/context.h, launch_box.h
// Compiled by nvcc, this header also brings in rxg/query.cuh: Query<bt>,
// Iterator<H>, ShmemAllocator and the kernels behind RXMeshStatic::for_each,
// run_kernel and the device side of for_each_vertex/edge/face.
// Every call goes through librxg.so; errors throw rxg::Error carrying the
// rxg_status and rxg_last_error().  Header only; needs the CUDA runtime.
#ifndef RXG_RXMESH_HPP
#define RXG_RXMESH_HPP

#include <cuda_runtime_api.h>

#include <functional>
#include <typeinfo>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../rxg.h"
#if defined(__CUDACC__)
#include "diff.cuh"  // Scalar and face_term_kernel behind DiffScalarProblem::add_term
#endif

namespace rxg {

class Error : public std::runtime_error
{
   public:
    Error(rxg_status s, const std::string& what) : std::runtime_error(what), status(s) {}
    rxg_status status;
};

inline void check(rxg_status s)
{
    if (s != RXG_OK)
        throw Error(s, std::string(rxg_status_string(s)) + ": " + rxg_last_error());
}

// synchronise s and throw if a bounded device-side wait gave up
// (rxg_device_check)
inline void device_check(cudaStream_t s = nullptr) { check(rxg_device_check(s)); }

inline void check_cuda(cudaError_t e, const char* what)
{
    if (e != cudaSuccess)
        throw Error(RXG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// Query operations (RXMesh's Op)
enum class Op : int32_t {
    VV = RXG_OP_VV,
    VE = RXG_OP_VE,
    VF = RXG_OP_VF,
    FV = RXG_OP_FV,
    EV = RXG_OP_EV,
    EF = RXG_OP_EF,
    FE = RXG_OP_FE,
    FF = RXG_OP_FF,
    EVDiamond = RXG_OP_EVD,
    EE = RXG_OP_EE,
    // the elements themselves (per-element terms, add_term<Op::V>); not queries
    V = 100,
    E = 101,
    F = 102
};

// where a buffer lives (RXMesh's locationT)
enum locationT : uint32_t { LOCATION_NONE = 0, HOST = 1, DEVICE = 2, LOCATION_ALL = 3 };

template <typename T>
struct dtype_of;
template <>
struct dtype_of<float>
{
    static constexpr int32_t value = RXG_F32;
};
template <>
struct dtype_of<double>
{
    static constexpr int32_t value = RXG_F64;
};

// Owning device array.
template <typename T>
class DeviceArray
{
   public:
    DeviceArray() = default;
    explicit DeviceArray(size_t n) { resize(n); }
    DeviceArray(const DeviceArray&)            = delete;
    DeviceArray& operator=(const DeviceArray&) = delete;
    DeviceArray(DeviceArray&& o) noexcept : m_ptr(o.m_ptr), m_n(o.m_n)
    {
        o.m_ptr = nullptr;
        o.m_n   = 0;
    }
    DeviceArray& operator=(DeviceArray&& o) noexcept
    {
        std::swap(m_ptr, o.m_ptr);
        std::swap(m_n, o.m_n);
        return *this;
    }
    ~DeviceArray()
    {
        if (m_ptr) cudaFree(m_ptr);
    }
    void resize(size_t n)
    {
        if (m_ptr) cudaFree(m_ptr);
        m_ptr = nullptr;
        m_n   = n;
        if (n) check_cuda(cudaMalloc(reinterpret_cast<void**>(&m_ptr), n * sizeof(T)), "cudaMalloc");
    }
    T*       data() { return m_ptr; }
    const T* data() const { return m_ptr; }
    size_t   size() const { return m_n; }

    void upload(const T* h, size_t n, cudaStream_t s = nullptr)
    {
        if (n != m_n) resize(n);
        if (n) check_cuda(cudaMemcpyAsync(m_ptr, h, n * sizeof(T), cudaMemcpyHostToDevice, s),
                          "cudaMemcpyAsync");
        check_cuda(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    }
    std::vector<T> to_host(cudaStream_t s = nullptr) const
    {
        std::vector<T> h(m_n);
        if (m_n)
            check_cuda(cudaMemcpyAsync(h.data(), m_ptr, m_n * sizeof(T), cudaMemcpyDeviceToHost, s),
                       "cudaMemcpyAsync");
        check_cuda(cudaStreamSynchronize(s), "cudaStreamSynchronize");
        return h;
    }
    void fill_zero(cudaStream_t s = nullptr)
    {
        if (m_n) check_cuda(cudaMemsetAsync(m_ptr, 0, m_n * sizeof(T), s), "cudaMemsetAsync");
    }

   private:
    T*     m_ptr = nullptr;
    size_t m_n   = 0;
};

class RXMeshStatic;

#if defined(__CUDACC__)
#define RXG_HD __host__ __device__
#else
#define RXG_HD
#endif
// extended-lambda traits (nvcc --extended-lambda): a __device__-only lambda
// cannot run in the HOST branch of for_each_vertex and the like
// and a plain host lambda cannot run in the DEVICE branch (without
// --extended-lambda any functor is taken to be device-callable)
#if defined(__CUDACC__) && defined(__CUDACC_EXTENDED_LAMBDA__)
#define RXG_IS_D_LAMBDA(T) __nv_is_extended_device_lambda_closure_type(T)
#define RXG_DEVICE_CALLABLE(T) \
    (__nv_is_extended_device_lambda_closure_type(T) || __nv_is_extended_host_device_lambda_closure_type(T))
#else
#define RXG_IS_D_LAMBDA(T) false
#define RXG_DEVICE_CALLABLE(T) true
#endif

// Handle of a vertex, edge or face (VertexHandle / EdgeHandle / FaceHandle,
// handle.h:19-144).  RXMesh's handle packs (owner patch, local index); here
// it holds the element's linear id, which is unique over the mesh (owned
// elements of patch 0 first, then patch 1, ...) and indexes every
// per-element array directly.  Default-constructed handles are invalid.
template <int ELEM>
struct ElementHandle
{
    static constexpr int kElem = ELEM;  // RXG_ELEM_VERTEX, _EDGE or _FACE
    RXG_HD ElementHandle() {}
    RXG_HD explicit ElementHandle(int32_t linear_id) : m_id(linear_id) {}
    RXG_HD bool     is_valid() const { return m_id >= 0; }
    RXG_HD int32_t  linear_id() const { return m_id; }
    RXG_HD uint64_t unique_id() const { return (uint64_t)(uint32_t)m_id; }
    RXG_HD bool     operator==(const ElementHandle& o) const { return m_id == o.m_id; }
    RXG_HD bool     operator!=(const ElementHandle& o) const { return m_id != o.m_id; }
    int32_t         m_id = -1;
};
using VertexHandle = ElementHandle<RXG_ELEM_VERTEX>;
using EdgeHandle   = ElementHandle<RXG_ELEM_EDGE>;
using FaceHandle   = ElementHandle<RXG_ELEM_FACE>;

// Per-element attribute (Attribute<T, HandleT>, attribute.h): num_attributes
// values per element, row-major in linear order, with a device and/or a host
// copy.  A shallow view, copied by value into kernels and device lambdas as
// RXMesh's attributes are; the RXMeshStatic that created it owns the buffers
// (remove_attribute or the mesh's destruction frees them).
template <typename T, typename HandleT>
class Attribute
{
   public:
    Attribute() = default;
    // attr(handle, i): value i of the element; device copy in device code,
    // host copy in host code
    RXG_HD T& operator()(const HandleT& h, uint32_t attr = 0) const
    {
#if defined(__CUDA_ARCH__)
        return m_d[(int64_t)h.linear_id() * m_num_attr + attr];
#else
        return m_h[(int64_t)h.linear_id() * m_num_attr + attr];
#endif
    }
    RXG_HD uint32_t get_num_attributes() const { return m_num_attr; }
    RXG_HD int64_t  size() const { return m_n; }
    T*              data(locationT where = DEVICE) const { return where == HOST ? m_h : m_d; }
    locationT       get_allocated() const { return (locationT)m_alloc; }
    // copy the values from one location to the other (Attribute::move)
    void move(locationT source, locationT target, cudaStream_t s = nullptr) const
    {
        if (source == target) return;
        if (!m_d || !m_h) throw Error(RXG_ERR_INVALID, "attribute is not allocated on both sides");
        const size_t bytes = sizeof(T) * (size_t)m_n * m_num_attr;
        if (source == HOST && target == DEVICE)
            check_cuda(cudaMemcpyAsync(m_d, m_h, bytes, cudaMemcpyHostToDevice, s), "cudaMemcpyAsync");
        else if (source == DEVICE && target == HOST)
            check_cuda(cudaMemcpyAsync(m_h, m_d, bytes, cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
        check_cuda(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    }
    // every value to `value` where allocated among `location`
    void reset(T value, locationT location, cudaStream_t s = nullptr) const
    {
        const size_t       n = (size_t)m_n * m_num_attr;
        std::vector<T>     tmp;
        const std::vector<T>* src = nullptr;
        if ((location & HOST) && m_h) std::fill(m_h, m_h + n, value);
        if ((location & DEVICE) && m_d) {
            if (m_h && (location & HOST)) {
                check_cuda(cudaMemcpyAsync(m_d, m_h, sizeof(T) * n, cudaMemcpyHostToDevice, s),
                           "cudaMemcpyAsync");
            } else {
                tmp.assign(n, value);
                src = &tmp;
                check_cuda(cudaMemcpyAsync(m_d, src->data(), sizeof(T) * n, cudaMemcpyHostToDevice, s),
                           "cudaMemcpyAsync");
            }
            check_cuda(cudaStreamSynchronize(s), "cudaStreamSynchronize");
        }
    }

   private:
    friend class RXMeshStatic;
    T*       m_d        = nullptr;
    T*       m_h        = nullptr;
    int64_t  m_n        = 0;
    uint32_t m_num_attr = 1;
    uint32_t m_alloc    = LOCATION_NONE;
};
template <typename T>
using VertexAttribute = Attribute<T, VertexHandle>;
template <typename T>
using EdgeAttribute = Attribute<T, EdgeHandle>;
template <typename T>
using FaceAttribute = Attribute<T, FaceHandle>;

// The mesh as kernels see it (Context, context.h:15-120): patch records and
// the arena on the device, sizes, and per-patch maxima; passed by value.
struct Context
{
    rxg_device_context c{};
    RXG_HD int64_t get_num_vertices() const { return c.num_vertices; }
    RXG_HD int64_t get_num_edges() const { return c.num_edges; }
    RXG_HD int64_t get_num_faces() const { return c.num_faces; }
    RXG_HD int32_t get_num_patches() const { return c.num_patches; }
};

// Grid and dynamic shared memory of a query kernel (LaunchBox, launch_box.h)
template <uint32_t blockThreads>
struct LaunchBox
{
    uint32_t blocks         = 0;
    uint32_t num_threads    = blockThreads;
    uint32_t smem_bytes_dyn = 0;
};

#if defined(__CUDACC__)
namespace detail {
template <Op op, uint32_t blockThreads, typename LambdaT>
void for_each_impl(const RXMeshStatic& rx, const LaunchBox<blockThreads>* lb, const LambdaT& f,
                   bool oriented, cudaStream_t stream);
template <uint32_t blockThreads>
void prepare_launch_box_impl(const RXMeshStatic& rx, const std::vector<Op>& ops,
                             LaunchBox<blockThreads>& lb, const void* kernel, bool oriented,
                             bool with_vertex_valence, bool is_concurrent,
                             const std::function<size_t(uint32_t, uint32_t, uint32_t)>& user_shmem);
template <typename HandleT, typename LambdaT>
void for_each_element_device(const RXMeshStatic& rx, const LambdaT& f, cudaStream_t stream);
}  // namespace detail
#endif

// rows x cols dense matrix in device memory, row-major (one row per mesh
// element, as every rxg call expects).
template <typename T>
class DenseMatrix
{
   public:
    DenseMatrix() = default;
    DenseMatrix(int64_t rows, int64_t cols, locationT where = DEVICE)
        : m_rows(rows), m_cols(cols), m_d((size_t)(rows * cols))
    {
        (void)where;
        m_d.fill_zero();
        check_cuda(cudaStreamSynchronize(nullptr), "cudaStreamSynchronize");
    }
    // the reference's DenseMatrix(rx, rows, cols, location)
    // (matrix/dense_matrix.h); the mesh is not needed here
    DenseMatrix(const RXMeshStatic&, int64_t rows, int64_t cols, locationT where = DEVICE)
        : DenseMatrix(rows, cols, where)
    {
    }
    int64_t  rows() const { return m_rows; }
    int64_t  cols() const { return m_cols; }
    T*       data(locationT = DEVICE) { return m_d.data(); }
    const T* data(locationT = DEVICE) const { return m_d.data(); }
    void     reset(T v, locationT = DEVICE, cudaStream_t s = nullptr)
    {
        if (v == T(0)) {
            m_d.fill_zero(s);
            return;
        }
        std::vector<T> h(m_d.size(), v);
        m_d.upload(h.data(), h.size(), s);
    }
    void from_host(const std::vector<T>& h, cudaStream_t s = nullptr)
    {
        if ((int64_t)h.size() != m_rows * m_cols) throw Error(RXG_ERR_INVALID, "size mismatch");
        m_d.upload(h.data(), h.size(), s);
    }
    std::vector<T> to_host(cudaStream_t s = nullptr) const { return m_d.to_host(s); }

    // the vector operations of dense_matrix.h (axpy 442, dot 518, norm2 604,
    // multiply 717, copy_from 1031) over all rows x cols values
    void axpy(const DenseMatrix<T>& X, T alpha, cudaStream_t s = nullptr)  // this = alpha X + this
    {
        check(rxg_dense_axpby(size(), dtype_of<T>::value, (double)alpha, X.data(), 1.0, data(), s));
    }
    T dot(const DenseMatrix<T>& x, bool = false, cudaStream_t s = nullptr) const
    {
        double r = 0.0;
        check(rxg_dense_dot(size(), dtype_of<T>::value, data(), x.data(), &r, s));
        return (T)r;
    }
    T    norm2(cudaStream_t s = nullptr) const { return (T)std::sqrt((double)dot(*this, false, s)); }
    void multiply(T scalar, cudaStream_t s = nullptr)
    {
        check(rxg_dense_axpby(size(), dtype_of<T>::value, 0.0, nullptr, (double)scalar, data(), s));
    }
    void copy_from(const DenseMatrix<T>& source, locationT = DEVICE, locationT = DEVICE,
                   cudaStream_t s = nullptr)
    {
        check(rxg_dense_axpby(size(), dtype_of<T>::value, 1.0, source.data(), 0.0, data(), s));
    }

   private:
    int64_t        size() const { return m_rows * m_cols; }
    int64_t        m_rows = 0, m_cols = 0;
    DeviceArray<T> m_d;
};

// CSR adjacency of a query: offsets (rows+1, absent for FV/EV) and values,
// both in device memory, in linear ids.
struct QueryResult
{
    int64_t              rows = 0;
    DeviceArray<int32_t> offsets;
    DeviceArray<int32_t> values;
};

// Static triangle mesh split into patches of at most patch_size faces.
class RXMeshStatic
{
   public:
    // fv: one {v0, v1, v2} per face, input vertex ids (rxmesh_static.h:87-92).
    // patcher_file: a partition saved by RXMesh (or save()) for this mesh;
    // empty: the library's own partition into patches of patch_size faces,
    // by the host BFS partitioner or, with gpu_patcher, by Lloyd region
    // growing on the GPU (RXMesh's patcher).
    explicit RXMeshStatic(std::vector<std::vector<uint32_t>>& fv,
                          const std::string                   patcher_file = "",
                          const uint32_t                      patch_size   = 512,
                          bool                                host_only    = false,
                          bool                                gpu_patcher  = false)
    {
        std::vector<int32_t> flat;
        flat.reserve(3 * fv.size());
        int64_t nv = 0;
        for (const auto& f : fv) {
            if (f.size() != 3) throw Error(RXG_ERR_INVALID, "only triangle faces are supported");
            for (uint32_t v : f) {
                flat.push_back((int32_t)v);
                nv = std::max<int64_t>(nv, (int64_t)v + 1);
            }
        }
        create(flat, nv, patcher_file, patch_size, host_only, gpu_patcher);
    }
    // An OBJ file (RXMeshStatic(file_path, patcher_file, patch_size),
    // rxmesh_static.h:61-66, which reads it with import_obj): "v x y z" and
    // "f a b c ..." lines (a, a/t, a//n, a/t/n; negative = relative to the
    // vertices read so far), polygons fanned into triangles; the positions
    // become the input vertex coordinates (not on a host_only mesh).
    explicit RXMeshStatic(const std::string& file_path, const std::string patcher_file = "",
                          const uint32_t patch_size = 512, bool host_only = false,
                          bool gpu_patcher = false)
    {
        std::vector<std::vector<double>> xyz;
        std::vector<int32_t>             flat;
        read_obj(file_path, xyz, flat);
        create(flat, (int64_t)xyz.size(), patcher_file, patch_size, host_only, gpu_patcher);
        if (!host_only) add_vertex_coordinates(xyz);
    }
    // Several OBJ files as one mesh of disjoint regions (RXMeshStatic(
    // files_path, patch_size), rxmesh_static.cu:66-160): faces and vertices
    // follow file after file, and every face, vertex and edge carries the
    // index of its file as its region label.
    explicit RXMeshStatic(const std::vector<std::string>& files_path,
                          const uint32_t patch_size = 512, bool host_only = false)
    {
        std::vector<std::vector<double>> xyz;
        std::vector<int32_t>             flat;
        for (const auto& path : files_path) {
            std::vector<std::vector<double>> x;
            std::vector<int32_t>             f;
            read_obj(path, x, f);
            const int32_t base = (int32_t)xyz.size();
            for (int32_t v : f) flat.push_back(v + base);
            xyz.insert(xyz.end(), x.begin(), x.end());
            m_region_faces.push_back((int64_t)flat.size() / 3);
            m_region_vertices.push_back((int64_t)xyz.size());
        }
        if (files_path.empty()) throw Error(RXG_ERR_INVALID, "no files");
        create(flat, (int64_t)xyz.size(), "", patch_size, host_only, false);
        if (!host_only) add_vertex_coordinates(xyz);
    }
    // number of regions (files; 1 for the other constructors) and the region
    // label of every face / vertex / edge in input ids (get_face_region_label
    // and the like, rxmesh_static.h:826-849)
    int get_num_regions() const { return m_region_faces.empty() ? 1 : (int)m_region_faces.size(); }
    std::vector<int32_t> get_region_label(int32_t elem) const
    {
        const auto label_of = [](const std::vector<int64_t>& ends, int64_t id) {
            return (int32_t)(std::upper_bound(ends.begin(), ends.end(), id) - ends.begin());
        };
        std::vector<int32_t> out;
        if (elem == RXG_ELEM_FACE || elem == RXG_ELEM_VERTEX) {
            const int64_t n = elem == RXG_ELEM_FACE ? m_info.num_faces : m_info.num_vertices;
            out.resize((size_t)n, 0);
            if (!m_region_faces.empty())
                for (int64_t i = 0; i < n; ++i)
                    out[(size_t)i] = label_of(elem == RXG_ELEM_FACE ? m_region_faces : m_region_vertices, i);
        } else {
            std::vector<int32_t> ev(2 * (size_t)m_info.num_edges);
            check(rxg_mesh_input_edges(m_mesh.get(), ev.data()));
            out.resize((size_t)m_info.num_edges, 0);
            if (!m_region_faces.empty())
                for (size_t e = 0; e < out.size(); ++e) out[e] = label_of(m_region_vertices, ev[2 * e]);
        }
        return out;
    }
    // a given partition (rxg_mesh_create_partitioned): face_patch, one patch
    // id per face; vertex and edge owners by RXMesh's lowest-patch rule
    RXMeshStatic(std::vector<std::vector<uint32_t>>& fv, const std::vector<int32_t>& face_patch,
                 bool host_only = false)
    {
        std::vector<int32_t> flat;
        int64_t              nv = 0;
        for (const auto& f : fv) {
            if (f.size() != 3) throw Error(RXG_ERR_INVALID, "only triangle faces are supported");
            for (uint32_t v : f) {
                flat.push_back((int32_t)v);
                nv = std::max<int64_t>(nv, (int64_t)v + 1);
            }
        }
        if (face_patch.size() != fv.size()) throw Error(RXG_ERR_INVALID, "one patch id per face");
        rxg_mesh* m = nullptr;
        check(rxg_mesh_create_partitioned(flat.data(), (int64_t)fv.size(), nv, face_patch.data(),
                                          nullptr, nullptr, -1, host_only ? RXG_MESH_HOST_ONLY : 0,
                                          &m));
        m_mesh.reset(m);
        m_fv = flat;
        check(rxg_mesh_get_info(m, &m_info));
    }
    // per-element DenseMatrix between input and linear order on the device
    // (rxg_permute; Attribute::from_matrix / to_matrix)
    template <typename T>
    void to_linear(int32_t elem, const DenseMatrix<T>& input_order, DenseMatrix<T>& linear,
                   cudaStream_t s = nullptr) const
    {
        check(rxg_permute(handle(), elem, 1, dtype_of<T>::value, (int32_t)input_order.cols(),
                          input_order.data(), linear.data(), s));
    }
    template <typename T>
    void to_input(int32_t elem, const DenseMatrix<T>& linear, DenseMatrix<T>& input_order,
                  cudaStream_t s = nullptr) const
    {
        check(rxg_permute(handle(), elem, 0, dtype_of<T>::value, (int32_t)linear.cols(),
                          linear.data(), input_order.data(), s));
    }
    // RXMesh::save (rxmesh.h:326-329): the partition as a patcher file
    void save(const std::string& filename) const
    {
        check(rxg_mesh_save_patch_file(m_mesh.get(), filename.c_str()));
    }
    // export_obj (rxmesh_static.inl:366-397): vertices in linear order from
    // coords (linear order), faces in linear order over linear vertex ids
    void export_obj(const std::string& filename, const DenseMatrix<double>& coords) const
    {
        const std::vector<double>  x   = coords.to_host();
        const std::vector<int32_t> fl  = linear_to_input(RXG_ELEM_FACE);
        const std::vector<int32_t> vl  = linear_to_input(RXG_ELEM_VERTEX);
        if ((int64_t)x.size() != 3 * m_info.num_vertices)
            throw Error(RXG_ERR_INVALID, "one position per vertex expected");
        std::vector<int32_t> vi2l(vl.size());
        for (size_t l = 0; l < vl.size(); ++l) vi2l[(size_t)vl[l]] = (int32_t)l;
        std::FILE* fp = std::fopen(filename.c_str(), "w");
        if (!fp) throw Error(RXG_ERR_INVALID, "cannot create " + filename);
        for (size_t v = 0; v < vl.size(); ++v)
            std::fprintf(fp, "v %.17g %.17g %.17g\n", x[3 * v], x[3 * v + 1], x[3 * v + 2]);
        for (int32_t f : fl)
            std::fprintf(fp, "f %d %d %d\n", vi2l[(size_t)m_fv[3 * (size_t)f]] + 1,
                         vi2l[(size_t)m_fv[3 * (size_t)f + 1]] + 1, vi2l[(size_t)m_fv[3 * (size_t)f + 2]] + 1);
        if (std::fclose(fp) != 0) throw Error(RXG_ERR_INVALID, "write to " + filename + " failed");
    }
    // get_boundary_vertices (rxmesh_static.inl:281-323): 1 for the ends of
    // edges with fewer than two faces, linear order
    std::vector<int8_t> get_boundary_vertices() const
    {
        std::vector<int8_t> out((size_t)m_info.num_vertices);
        check(rxg_mesh_boundary_vertices(m_mesh.get(), out.data(), nullptr));
        return out;
    }
    // owner patch of every face, vertex and edge, in input ids
    void partition(std::vector<int32_t>& face_patch, std::vector<int32_t>& vertex_patch,
                   std::vector<int32_t>& edge_patch) const
    {
        face_patch.resize((size_t)m_info.num_faces);
        vertex_patch.resize((size_t)m_info.num_vertices);
        edge_patch.resize((size_t)m_info.num_edges);
        check(rxg_mesh_partition(m_mesh.get(), face_patch.data(), vertex_patch.data(),
                                 edge_patch.data()));
    }
    RXMeshStatic(const RXMeshStatic&)            = delete;
    RXMeshStatic& operator=(const RXMeshStatic&) = delete;

    uint32_t get_num_vertices() const { return (uint32_t)m_info.num_vertices; }
    uint32_t get_num_edges() const { return (uint32_t)m_info.num_edges; }
    uint32_t get_num_faces() const { return (uint32_t)m_info.num_faces; }
    uint32_t get_num_patches() const { return (uint32_t)m_info.num_patches; }
    uint32_t get_patch_size() const { return (uint32_t)m_info.patch_faces; }
    uint32_t get_input_max_valence() const { return (uint32_t)m_info.max_valence; }
    bool     is_closed() const { return m_info.is_closed != 0; }
    bool     is_edge_manifold() const { return m_info.is_edge_manifold != 0; }
    bool     is_oriented() const { return m_info.is_oriented != 0; }
    uint32_t get_num_components() const { return (uint32_t)m_info.num_components; }
    uint32_t get_input_max_edge_incident_faces() const { return (uint32_t)m_info.max_edge_incident_faces; }
    uint32_t get_input_max_face_adjacent_faces() const { return (uint32_t)m_info.max_face_adjacent_faces; }
    const rxg_mesh_info& info() const { return m_info; }
    const rxg_mesh*      handle() const { return m_mesh.get(); }

    // input id of every linear id (map_to_global, rxmesh_static.h:874-905)
    std::vector<int32_t> linear_to_input(int32_t elem = RXG_ELEM_VERTEX) const
    {
        const int64_t n = elem == RXG_ELEM_VERTEX ? m_info.num_vertices
                          : elem == RXG_ELEM_EDGE ? m_info.num_edges
                                                  : m_info.num_faces;
        std::vector<int32_t> out((size_t)n);
        check(rxg_mesh_linear_to_input(handle(), elem, out.data()));
        return out;
    }

    // Vertex coordinates in input order (add_vertex_coordinates,
    // rxmesh_static.h:110-112); kept on the device in linear order, FP64.
    void add_vertex_coordinates(const std::vector<std::vector<double>>& vertices,
                                cudaStream_t                            s = nullptr)
    {
        if ((int64_t)vertices.size() != m_info.num_vertices)
            throw Error(RXG_ERR_INVALID, "one coordinate triple per vertex expected");
        const std::vector<int32_t> l2i = linear_to_input(RXG_ELEM_VERTEX);
        std::vector<double>        h(3 * vertices.size());
        for (size_t l = 0; l < l2i.size(); ++l)
            for (int c = 0; c < 3; ++c) h[3 * l + c] = vertices[(size_t)l2i[l]].at(c);
        m_xyz = DenseMatrix<double>(m_info.num_vertices, 3);
        m_xyz.from_host(h, s);
    }
    DenseMatrix<double>&       get_input_vertex_coordinates() { return m_xyz; }
    const DenseMatrix<double>& get_input_vertex_coordinates() const { return m_xyz; }

    // for_each<op> materialising every owned element's adjacency
    // (Query::dispatch, query.h:21-75), CSR in linear ids.
    QueryResult query(Op op, cudaStream_t s = nullptr) const
    {
        QueryResult r;
        int64_t     nval = 0;
        check(rxg_query_size(handle(), (int32_t)op, &r.rows, &nval));
        const bool csr = op == Op::VV || op == Op::VE || op == Op::VF || op == Op::EF || op == Op::FF;
        if (csr) r.offsets.resize((size_t)r.rows + 1);
        r.values.resize((size_t)nval);
        check(rxg_query(handle(), (int32_t)op, csr ? r.offsets.data() : nullptr, r.values.data(), s));
        return r;
    }

    // oriented one-ring (rxmesh_queries.cuh:376-499): offsets, values, boundary flag
    void query_oriented_vv(DeviceArray<int32_t>& off, DeviceArray<int32_t>& val,
                           DeviceArray<int8_t>& bnd, cudaStream_t s = nullptr) const
    {
        off.resize((size_t)m_info.num_vertices + 1);
        val.resize((size_t)(2 * m_info.num_edges));
        bnd.resize((size_t)m_info.num_vertices);
        check(rxg_query_oriented_vv(handle(), off.data(), val.data(), bnd.data(), s));
    }

    // vertex normals of linear-order FP32 positions (compute_vertex_normal,
    // apps/VertexNormal/vertex_normal_kernel.cuh)
    void compute_vertex_normal(const DenseMatrix<float>& xyz, DenseMatrix<float>& out,
                               int32_t weighting = RXG_NORMAL_MAX, cudaStream_t s = nullptr) const
    {
        check(rxg_vertex_normals(handle(), weighting, xyz.data(), out.data(), s));
    }

    // ---- device-side queries (Query<bt>::dispatch, for_each, run_kernel) ----

    // the mesh as kernels see it (RXMeshStatic::get_context)
    Context get_context() const
    {
        Context c;
        check(rxg_mesh_device_context(handle(), &c.c));
        return c;
    }

    // ---- attributes (add_vertex_attribute ..., rxmesh_static.h:608-793) ----

    template <typename T>
    std::shared_ptr<VertexAttribute<T>> add_vertex_attribute(const std::string& name,
                                                             uint32_t num_attributes,
                                                             locationT location = LOCATION_ALL)
    {
        return add_attribute<T, VertexHandle>(name, num_attributes, location, m_info.num_vertices);
    }
    template <typename T>
    std::shared_ptr<EdgeAttribute<T>> add_edge_attribute(const std::string& name,
                                                         uint32_t num_attributes,
                                                         locationT location = LOCATION_ALL)
    {
        return add_attribute<T, EdgeHandle>(name, num_attributes, location, m_info.num_edges);
    }
    template <typename T>
    std::shared_ptr<FaceAttribute<T>> add_face_attribute(const std::string& name,
                                                         uint32_t num_attributes,
                                                         locationT location = LOCATION_ALL)
    {
        return add_attribute<T, FaceHandle>(name, num_attributes, location, m_info.num_faces);
    }
    // from per-vertex values in input order (add_vertex_attribute(value,
    // name), rxmesh_static.h:700-740): host and device, linear order
    template <typename T>
    std::shared_ptr<VertexAttribute<T>> add_vertex_attribute(const std::vector<std::vector<T>>& value,
                                                             const std::string& name)
    {
        if ((int64_t)value.size() != m_info.num_vertices || value.empty())
            throw Error(RXG_ERR_INVALID, "add_vertex_attribute: one row per vertex expected");
        const uint32_t na = (uint32_t)value[0].size();
        auto           a  = add_vertex_attribute<T>(name, na, LOCATION_ALL);
        const std::vector<int32_t> l2i = linear_to_input(RXG_ELEM_VERTEX);
        for (size_t l = 0; l < l2i.size(); ++l) {
            const std::vector<T>& row = value[(size_t)l2i[l]];
            if (row.size() != na) throw Error(RXG_ERR_INVALID, "add_vertex_attribute: ragged rows");
            for (uint32_t k = 0; k < na; ++k) a->data(HOST)[l * na + k] = row[k];
        }
        a->move(HOST, DEVICE);
        return a;
    }
    template <typename T>
    std::shared_ptr<VertexAttribute<T>> get_vertex_attribute(const std::string& name) const
    {
        return get_attribute<T, VertexHandle>(name);
    }
    template <typename T>
    std::shared_ptr<EdgeAttribute<T>> get_edge_attribute(const std::string& name) const
    {
        return get_attribute<T, EdgeHandle>(name);
    }
    template <typename T>
    std::shared_ptr<FaceAttribute<T>> get_face_attribute(const std::string& name) const
    {
        return get_attribute<T, FaceHandle>(name);
    }
    bool does_attribute_exist(const std::string& name) const
    {
        for (const auto& a : m_attrs)
            if (a->name == name) return true;
        return false;
    }
    // frees the attribute's buffers; views of it must not be used afterwards
    void remove_attribute(const std::string& name)
    {
        for (size_t i = 0; i < m_attrs.size(); ++i)
            if (m_attrs[i]->name == name) {
                m_attrs.erase(m_attrs.begin() + (long)i);
                return;
            }
    }

    // ---- per-element loops (for_each_vertex / edge / face, rxmesh_static.h:205-379) ----
    // apply(handle) for every vertex (edge, face).  HOST: a loop on this
    // thread (apply must be callable on the host); DEVICE: one kernel, one
    // thread per element (apply a __device__ or __host__ __device__ lambda;
    // the caller is compiled by nvcc); LOCATION_ALL: both.
    template <typename LambdaT>
    void for_each_vertex(locationT location, LambdaT apply, cudaStream_t stream = nullptr) const
    {
        for_each_element<VertexHandle>(location, apply, stream, m_info.num_vertices);
    }
    template <typename LambdaT>
    void for_each_edge(locationT location, LambdaT apply, cudaStream_t stream = nullptr) const
    {
        for_each_element<EdgeHandle>(location, apply, stream, m_info.num_edges);
    }
    template <typename LambdaT>
    void for_each_face(locationT location, LambdaT apply, cudaStream_t stream = nullptr) const
    {
        for_each_element<FaceHandle>(location, apply, stream, m_info.num_faces);
    }

#if defined(__CUDACC__)
    // for_each<op, blockThreads>(lambda, oriented, stream) (rxmesh_static.h:
    // 524-566): one CTA per patch runs Query<blockThreads>::dispatch<op> and
    // calls lambda(source handle, output iterator) for every owned source
    // element of its patch.  The iterator's handles carry linear ids.
    template <Op op, uint32_t blockThreads, typename LambdaT>
    void for_each(const LambdaT user_lambda, const bool oriented = false,
                  cudaStream_t stream = nullptr) const
    {
        detail::for_each_impl<op, blockThreads>(*this, nullptr, user_lambda, oriented, stream);
    }
    template <Op op, uint32_t blockThreads, typename LambdaT>
    void for_each(LaunchBox<blockThreads> lb, const LambdaT user_lambda, const bool oriented = false,
                  cudaStream_t stream = nullptr) const
    {
        detail::for_each_impl<op, blockThreads>(*this, &lb, user_lambda, oriented, stream);
    }
    // grid (one CTA per patch) and dynamic shared memory for a kernel that
    // runs the queries `op` (prepare_launch_box, rxmesh_static.h:585-594;
    // shared memory as calc_shared_memory, rxmesh_static.inl:548-741): the
    // largest op's need (their sum when is_concurrent), plus the valence
    // array, plus user_shmem(max local vertices, edges, faces).
    template <uint32_t blockThreads>
    void prepare_launch_box(const std::vector<Op> op, LaunchBox<blockThreads>& launch_box,
                            const void* kernel, const bool oriented = false,
                            const bool with_vertex_valence = false, const bool is_concurrent = false,
                            std::function<size_t(uint32_t, uint32_t, uint32_t)> user_shmem =
                                [](uint32_t, uint32_t, uint32_t) { return (size_t)0; }) const
    {
        detail::prepare_launch_box_impl<blockThreads>(*this, op, launch_box, kernel, oriented,
                                                      with_vertex_valence, is_concurrent, user_shmem);
    }
    // run_kernel (rxmesh_static.h:450-505): prepare the launch box for `op`
    // and launch kernel<<<patches, blockThreads, smem>>>(args...)
    template <uint32_t blockThreads, typename KernelT, typename... ArgsT>
    void run_kernel(const std::vector<Op> op, KernelT kernel, ArgsT... args) const
    {
        LaunchBox<blockThreads> lb;
        prepare_launch_box(op, lb, (const void*)kernel);
        run_kernel(lb, kernel, args...);
    }
    template <uint32_t blockThreads, typename KernelT, typename... ArgsT>
    void run_kernel(const LaunchBox<blockThreads>& lb, KernelT kernel, ArgsT... args) const
    {
        kernel<<<lb.blocks, lb.num_threads, lb.smem_bytes_dyn>>>(args...);
        check_cuda(cudaGetLastError(), "run_kernel launch");
    }
#endif

   private:
    struct Del
    {
        void operator()(rxg_mesh* m) const { rxg_mesh_destroy(m); }
    };
    // buffers of one attribute (freed with it)
    struct AttrStore
    {
        std::string           name;
        const std::type_info* type = nullptr;
        void*                 d    = nullptr;
        void*                 h    = nullptr;
        std::shared_ptr<void> view;
        AttrStore() = default;
        AttrStore(const AttrStore&) = delete;
        AttrStore& operator=(const AttrStore&) = delete;
        ~AttrStore()
        {
            if (d) cudaFree(d);
            std::free(h);
        }
    };
    std::vector<std::unique_ptr<AttrStore>> m_attrs;

    template <typename T, typename HandleT>
    std::shared_ptr<Attribute<T, HandleT>> add_attribute(const std::string& name, uint32_t na,
                                                         locationT location, int64_t n)
    {
        if (does_attribute_exist(name)) throw Error(RXG_ERR_INVALID, "attribute " + name + " exists");
        if (na == 0) throw Error(RXG_ERR_INVALID, "attribute needs at least one value per element");
        std::unique_ptr<AttrStore> st(new AttrStore);
        st->name           = name;
        st->type           = &typeid(Attribute<T, HandleT>);
        const size_t bytes = sizeof(T) * (size_t)n * na;
        auto         a     = std::make_shared<Attribute<T, HandleT>>();
        a->m_n             = n;
        a->m_num_attr      = na;
        a->m_alloc         = location;
        if (location & DEVICE) {
            check_cuda(cudaMalloc(&st->d, bytes ? bytes : 1), "cudaMalloc");
            check_cuda(cudaMemset(st->d, 0, bytes), "cudaMemset");
            a->m_d = static_cast<T*>(st->d);
        }
        if (location & HOST) {
            st->h = std::calloc(bytes ? bytes : 1, 1);
            if (!st->h) throw Error(RXG_ERR_NOMEM, "attribute host allocation");
            a->m_h = static_cast<T*>(st->h);
        }
        st->view = a;
        m_attrs.push_back(std::move(st));
        return a;
    }
    template <typename T, typename HandleT>
    std::shared_ptr<Attribute<T, HandleT>> get_attribute(const std::string& name) const
    {
        for (const auto& a : m_attrs)
            if (a->name == name) {
                if (*a->type != typeid(Attribute<T, HandleT>))
                    throw Error(RXG_ERR_INVALID, "attribute " + name + " has another type");
                return std::static_pointer_cast<Attribute<T, HandleT>>(a->view);
            }
        throw Error(RXG_ERR_INVALID, "no attribute " + name);
    }
    template <typename HandleT, typename LambdaT>
    void for_each_element(locationT location, LambdaT& apply, cudaStream_t stream, int64_t n) const
    {
        if (location & HOST) {
            if constexpr (!RXG_IS_D_LAMBDA(LambdaT)) {
                for (int64_t i = 0; i < n; ++i) apply(HandleT((int32_t)i));
            } else {
                throw Error(RXG_ERR_INVALID,
                            "for_each on HOST needs a host-callable lambda (this one is __device__)");
            }
        }
        if (location & DEVICE) {
#if defined(__CUDACC__)
            if constexpr (RXG_DEVICE_CALLABLE(LambdaT))
                detail::for_each_element_device<HandleT>(*this, apply, stream);
            else
                throw Error(RXG_ERR_INVALID,
                            "for_each on DEVICE needs a __device__ or __host__ __device__ lambda");
#else
            (void)stream;
            throw Error(RXG_ERR_UNSUPPORTED, "for_each on DEVICE needs the caller compiled by nvcc");
#endif
        }
    }
    std::unique_ptr<rxg_mesh, Del> m_mesh;

    std::vector<int64_t>           m_region_faces, m_region_vertices;  // cumulative, per file
    std::vector<int32_t>           m_fv;  // the input faces (export_obj)

    void create(const std::vector<int32_t>& flat, int64_t nv, const std::string& patcher_file,
                uint32_t patch_size, bool host_only, bool gpu_patcher)
    {
        rxg_mesh*     m     = nullptr;
        const int32_t flags =
            (host_only ? RXG_MESH_HOST_ONLY : 0) | (gpu_patcher ? RXG_MESH_GPU_PATCHER : 0);
        const int64_t nf = (int64_t)flat.size() / 3;
        m_fv             = flat;
        if (patcher_file.empty())
            check(rxg_mesh_create_ex(flat.data(), nf, nv, (int32_t)patch_size, flags, &m));
        else
            check(rxg_mesh_create_from_patch_file(flat.data(), nf, nv, patcher_file.c_str(), flags,
                                                  &m));
        m_mesh.reset(m);
        check(rxg_mesh_get_info(m, &m_info));
    }
    static void read_obj(const std::string& path, std::vector<std::vector<double>>& xyz,
                         std::vector<int32_t>& flat)
    {
        std::FILE* fp = std::fopen(path.c_str(), "r");
        if (!fp) throw Error(RXG_ERR_INVALID, "cannot open " + path);
        std::string line;
        char        buf[4096];
        auto        fail = [&](const std::string& why) {
            std::fclose(fp);
            throw Error(RXG_ERR_INVALID, path + ": " + why);
        };
        while (std::fgets(buf, sizeof(buf), fp)) {
            line.assign(buf);
            while (!line.empty() && line.back() != '\n' && std::fgets(buf, sizeof(buf), fp))
                line.append(buf);
            const char* c = line.c_str();
            if (c[0] == 'v' && (c[1] == ' ' || c[1] == '\t')) {
                double p[3];
                char*  e = const_cast<char*>(c + 1);
                for (double& q : p) {
                    char* start = e;
                    q           = std::strtod(start, &e);
                    if (e == start) fail("malformed vertex line");
                }
                xyz.push_back({p[0], p[1], p[2]});
            } else if (c[0] == 'f' && (c[1] == ' ' || c[1] == '\t')) {
                std::vector<int32_t> ids;
                const char*          q = c + 1;
                while (true) {
                    while (*q == ' ' || *q == '\t') ++q;
                    if (*q == '\0' || *q == '\n' || *q == '\r' || *q == '#') break;
                    char*      e = nullptr;
                    const long i = std::strtol(q, &e, 10);
                    if (e == q || i == 0) fail("malformed face line");
                    const long n = (long)xyz.size();
                    const long v = i > 0 ? i - 1 : n + i;  // 1-based, or relative
                    if (v < 0 || v >= n) fail("face references a vertex not yet defined");
                    ids.push_back((int32_t)v);
                    q = e;
                    while (*q && *q != ' ' && *q != '\t' && *q != '\n' && *q != '\r') ++q;
                }
                if (ids.size() < 3) fail("face with fewer than three vertices");
                for (size_t k = 1; k + 1 < ids.size(); ++k) {
                    flat.push_back(ids[0]);
                    flat.push_back(ids[k]);
                    flat.push_back(ids[k + 1]);
                }
            }
        }
        std::fclose(fp);
        if (flat.empty()) throw Error(RXG_ERR_INVALID, path + ": no faces");
    }
    rxg_mesh_info                  m_info{};
    DenseMatrix<double>            m_xyz;
};

// CSR over linear vertex ids with the [diagonal, one-ring] pattern of the
// mesh (SparseMatrix<T>(rx), sparse_matrix.h:77).
template <typename T>
class SparseMatrix
{
   public:
    explicit SparseMatrix(const RXMeshStatic& rx)
    {
        int64_t n = 0, nnz = 0;
        check(rxg_mcf_pattern_size(rx.handle(), &n, &nnz));
        m_n = n;
        m_row_ptr.resize((size_t)n + 1);
        m_col.resize((size_t)nnz);
        m_val.resize((size_t)nnz);
        m_row_ptr.fill_zero();
        m_col.fill_zero();
        m_val.fill_zero();
        check_cuda(cudaStreamSynchronize(nullptr), "cudaStreamSynchronize");
    }
    // an n x n CSR with room for nnz entries (filled by the caller, e.g.
    // BlockSparseMatrix::to_csr)
    SparseMatrix(int64_t n, int64_t nnz) : m_n(n), m_row_ptr((size_t)n + 1), m_col((size_t)nnz), m_val((size_t)nnz)
    {
    }
    int64_t rows() const { return m_n; }
    int64_t cols() const { return m_n; }
    int64_t non_zeros() const { return (int64_t)m_col.size(); }
    rxg_csr csr()
    {
        rxg_csr c;
        c.n       = m_n;
        c.nnz     = (int64_t)m_col.size();
        c.row_ptr = m_row_ptr.data();
        c.col     = m_col.data();
        c.val     = m_val.data();
        c.dtype   = dtype_of<T>::value;
        return c;
    }
    // Y = A X (sparse_matrix.h:1173-1263)
    void multiply(const DenseMatrix<T>& X, DenseMatrix<T>& Y, cudaStream_t s = nullptr)
    {
        rxg_csr c = csr();
        check(rxg_spmm(&c, (int32_t)X.cols(), X.data(), Y.data(), s));
    }
    DeviceArray<int32_t>& row_ptr() { return m_row_ptr; }
    DeviceArray<int32_t>& col_idx() { return m_col; }
    DeviceArray<T>&       values() { return m_val; }
    // A(row, col), 0 where the pattern has no entry (operator(),
    // sparse_matrix.h:412-471); a host lookup that reads the row back
    T operator()(int64_t row, int64_t col) const
    {
        if (row < 0 || row >= m_n) throw Error(RXG_ERR_INVALID, "row out of range");
        int32_t be[2];
        check_cuda(cudaMemcpy(be, m_row_ptr.data() + row, sizeof(be), cudaMemcpyDeviceToHost),
                   "cudaMemcpy");
        const size_t         len = (size_t)(be[1] - be[0]);
        std::vector<int32_t> c(len);
        std::vector<T>       v(len);
        if (len) {
            check_cuda(cudaMemcpy(c.data(), m_col.data() + be[0], len * 4, cudaMemcpyDeviceToHost),
                       "cudaMemcpy");
            check_cuda(cudaMemcpy(v.data(), m_val.data() + be[0], len * sizeof(T),
                                  cudaMemcpyDeviceToHost),
                       "cudaMemcpy");
        }
        for (size_t k = 0; k < len; ++k)
            if (c[k] == col) return v[k];
        return T(0);
    }

   private:
    int64_t              m_n = 0;
    DeviceArray<int32_t> m_row_ptr, m_col;
    DeviceArray<T>       m_val;
};

// (A, B) of the implicit MCF system at linear-order positions xyz
// (mcf_A_setup / mcf_B_setup, apps/MCF/mcf_kernels.cuh:302-426)
template <typename T>
inline void mcf_assemble(const RXMeshStatic& rx, double dt, const DenseMatrix<double>& xyz,
                         SparseMatrix<T>& A, DenseMatrix<T>& B, cudaStream_t s = nullptr)
{
    rxg_csr c = A.csr();
    check(rxg_mcf_assemble(rx.handle(), dt, xyz.data(), &c, B.data(), s));
}

// CG (cg_solver.h:17-130); PCG adds the Jacobi preconditioner
// (pcg_solver.h:14-213).  pre_solve is folded into solve, which runs the whole
// solve in one device launch.
template <typename T>
struct CGSolver
{
    CGSolver(SparseMatrix<T>& sys, int unknown_dim, int max_iter, T abs_tol = 1e-6, T rel_tol = 0.0)
        : A(&sys), m_nc(unknown_dim), m_max_iter(max_iter), m_abs_tol(abs_tol), m_rel_tol(rel_tol)
    {
    }
    virtual ~CGSolver() = default;
    virtual void pre_solve(const DenseMatrix<T>&, DenseMatrix<T>&, cudaStream_t = nullptr) {}
    virtual void solve(const DenseMatrix<T>& B, DenseMatrix<T>& X, cudaStream_t s = nullptr)
    {
        run(B, X, s, false);
    }
    // the same solve with no device allocation (rxg_cg_solve_noalloc: a
    // static scratch array, at most 131,072 rows; calls must not overlap)
    void solve_noalloc(const DenseMatrix<T>& B, DenseMatrix<T>& X, cudaStream_t s = nullptr)
    {
        run(B, X, s, true);
    }
    virtual std::string name() { return "CG"; }
    int                 iter_taken() const { return m_stats.iters; }
    T                   start_residual() const { return (T)m_stats.start_res; }
    T                   final_residual() const { return (T)m_stats.final_res; }
    bool                converged() const { return m_stats.converged != 0; }

   protected:
    void run(const DenseMatrix<T>& B, DenseMatrix<T>& X, cudaStream_t s, bool noalloc)
    {
        rxg_solver_opts o;
        o.max_iter    = m_max_iter;
        o.abs_tol     = (double)m_abs_tol;
        o.rel_tol     = (double)m_rel_tol;
        o.precond     = precond();
        rxg_csr    c  = A->csr();
        rxg_status st = noalloc
                            ? rxg_cg_solve_noalloc(&c, m_nc, B.data(), X.data(), &o, &m_stats, s)
                            : rxg_cg_solve(&c, m_nc, B.data(), X.data(), &o, &m_stats, s);
        if (st != RXG_ERR_NOT_CONVERGED) check(st);
    }
    virtual int32_t  precond() const { return 0; }
    SparseMatrix<T>* A;
    int              m_nc, m_max_iter;
    T                m_abs_tol, m_rel_tol;
    rxg_solver_stats m_stats{};
};

template <typename T>
struct PCGSolver : public CGSolver<T>
{
    using CGSolver<T>::CGSolver;
    std::string name() override { return "PCG"; }

   protected:
    int32_t precond() const override { return 1; }
};

// nsteps implicit MCF steps in place on linear-order FP64 positions
// (run_cg of apps/MCF/mcf_cg.h:12-129); precision RXG_F64 (plain) or
// RXG_F32 (FP32 inner solves with FP64 refinement).
inline rxg_solver_stats mcf_step(const RXMeshStatic& rx, DenseMatrix<double>& xyz, double dt,
                                 int32_t nsteps = 1, int32_t precision = RXG_F64,
                                 double tol = 1e-6, int32_t max_iter = 5000,
                                 cudaStream_t s = nullptr)
{
    rxg_solver_stats st{};
    rxg_status       r =
        rxg_mcf_step(rx.handle(), dt, nsteps, precision, tol, max_iter, xyz.data(), &st, s);
    if (r != RXG_ERR_NOT_CONVERGED) check(r);
    return st;
}

// dl/dx_in of one plain implicit MCF step given dl/dx_out (adjoint solve
// with the same matrix); FP64, linear order.
inline rxg_solver_stats mcf_step_backward(const RXMeshStatic& rx, double dt,
                                          const DenseMatrix<double>& x_in,
                                          const DenseMatrix<double>& x_out,
                                          const DenseMatrix<double>& g_out,
                                          DenseMatrix<double>& g_in, double tol = 1e-12,
                                          int32_t max_iter = 20000, cudaStream_t s = nullptr)
{
    rxg_solver_stats st{};
    rxg_status       r = rxg_mcf_step_backward(rx.handle(), dt, x_in.data(), x_out.data(),
                                               g_out.data(), g_in.data(), tol, max_iter, &st, s);
    if (r != RXG_ERR_NOT_CONVERGED) check(r);
    return st;
}

// 3x3-block CSR over the [diagonal, one-ring] pattern (HessianSparseMatrix,
// diff/hessian_sparse_matrix.h:16-137)
template <typename T>
class BlockSparseMatrix
{
   public:
    // n block rows, nnzb blocks of dim x dim (HessianSparseMatrix<T, dim>)
    BlockSparseMatrix(int64_t n, int64_t nnzb, int dim = 3)
        : m_n(n), m_dim(dim), m_row_ptr(n + 1), m_col(nnzb), m_val((size_t)(dim * dim * nnzb))
    {
    }
    rxg_bcsr bcsr()
    {
        rxg_bcsr b;
        b.n         = m_n;
        b.nnzb      = (int64_t)m_col.size();
        b.row_ptr   = m_row_ptr.data();
        b.col       = m_col.data();
        b.val       = m_val.data();
        b.dtype     = dtype_of<T>::value;
        b.block_dim = m_dim;
        return b;
    }
    int block_dim() const { return m_dim; }
    int64_t               rows() const { return m_n; }
    int64_t               non_zero_blocks() const { return (int64_t)m_col.size(); }
    // the scalar 3n x 3n form the CG/PCG solvers take (out: 3n rows, 9 nnzb)
    void to_csr(SparseMatrix<T>& out, cudaStream_t s = nullptr)
    {
        rxg_bcsr b = bcsr();
        rxg_csr  c = out.csr();
        check(rxg_bcsr_to_csr(&b, &c, s));
    }
    // NewtonSolver::apply_bc on this Hessian and the gradient (bc: n int8, device)
    void apply_bc(const int8_t* bc, DenseMatrix<T>* grad, cudaStream_t s = nullptr)
    {
        rxg_bcsr b = bcsr();
        check(rxg_bcsr_apply_bc(&b, bc, grad ? grad->data() : nullptr, s));
    }
    DeviceArray<int32_t>& row_ptr() { return m_row_ptr; }
    DeviceArray<int32_t>& col_idx() { return m_col; }
    DeviceArray<T>&       values() { return m_val; }

   private:
    int64_t              m_n;
    int                  m_dim;
    DeviceArray<int32_t> m_row_ptr, m_col;
    DeviceArray<T>       m_val;
};

// Energy / gradient / Hessian driver for the per-face ARAP term
// (DiffScalarProblem<T, 3, VertexHandle, true>, diff_scalar_problem.h:27-401;
// the reference takes a user lambda per face, which a C ABI cannot carry, so
// the term is fixed: add_arap_term(rest positions)).
template <typename T, int VariableDim = 3>
class DiffScalarProblem
{
   public:
    static_assert(VariableDim >= 1 && VariableDim <= 3, "1, 2 or 3 components per vertex");
    explicit DiffScalarProblem(const RXMeshStatic& rx, bool assemble_hessian = true) : m_rx(&rx)
    {
        int64_t n = 0, nnz = 0;
        check(rxg_mcf_pattern_size(rx.handle(), &n, &nnz));
        grad = DenseMatrix<T>(n, VariableDim);
        face_energy.resize(rx.get_num_faces());
        if (assemble_hessian) hess.reset(new BlockSparseMatrix<T>(n, nnz, VariableDim));
    }
    // rest: linear-order FP64 positions of the flat rest shape
    // project_hessian: the reference's add_term<Op::FV, ProjectHess = true>
    void add_arap_term(const DenseMatrix<double>& rest, cudaStream_t s = nullptr,
                       bool project_hessian = false)
    {
        static_assert(VariableDim == 3, "the ARAP term is on 3-D positions");
        m_project = project_hessian;
        m_rest.resize(4 * (size_t)m_rx->get_num_faces());
        check(rxg_arap_rest(m_rx->handle(), rest.data(), dtype_of<T>::value, m_rest.data(), s));
    }
#if defined(__CUDACC__)
    // add_term<op, ProjectHess>(energy) (diff_scalar_problem.h:127-194), a
    // __device__ lambda or functor over the optimisation variable (linear
    // order) of one element's vertices, as Scalar<T, K, true> values, v[k *
    // VariableDim + d] = component d of the element's vertex k:
    //   Op::FV  energy(face id, v), K = 3 VariableDim, the face's vertices in
    //           input order;
    //   Op::EV  energy(edge id, v), K = 2 VariableDim, the edge's two
    //           vertices in EV order;
    //   Op::V   energy(vertex id, v), K = VariableDim.
    // Terms add up.
    template <Op op, bool ProjectHess = false, typename LambdaT>
    void add_term(LambdaT energy)
    {
        static_assert(op == Op::FV || op == Op::EV || op == Op::V, "terms are per face, edge or vertex");
        if constexpr (op == Op::FV) {
            if (m_fv.size() == 0) m_fv = std::move(m_rx->query(Op::FV).values);
            const int64_t  nf = m_rx->get_num_faces();
            const int32_t* fv = m_fv.data();
            m_terms.push_back({0, [=](const T* x, T* rec, cudaStream_t s) {
                                   check_cuda(launch_face_term<T, VariableDim, ProjectHess>(nf, fv, x, energy, rec, s),
                                              "face term launch");
                               }});
        } else if constexpr (op == Op::EV) {
            if (m_ev.size() == 0) m_ev = std::move(m_rx->query(Op::EV).values);
            const int64_t  ne = m_rx->get_num_edges();
            const int32_t* ev = m_ev.data();
            m_terms.push_back({1, [=](const T* x, T* rec, cudaStream_t s) {
                                   check_cuda(launch_edge_term<T, VariableDim, ProjectHess>(ne, ev, x, energy, rec, s),
                                              "edge term launch");
                               }});
        } else {
            const int64_t nv = m_rx->get_num_vertices();
            m_terms.push_back({2, [=](const T* x, T* rec, cudaStream_t s) {
                                   check_cuda(launch_vertex_term<T, VariableDim, ProjectHess>(nv, x, energy, rec, s),
                                              "vertex term launch");
                               }});
        }
    }
#endif
    // inertia of a mass-spring system, mass/2 |x - x_target|^2 per vertex
    // (add_inertia_term, tests/RXMesh_test/test_hess.cu:13-29); x_target in
    // linear order, copied
    void add_inertia_term(const DenseMatrix<T>& x_target, T mass, cudaStream_t s = nullptr)
    {
        m_xt.resize((size_t)x_target.size());
        check_cuda(cudaMemcpyAsync(m_xt.data(), x_target.data(), sizeof(T) * (size_t)x_target.size(),
                                   cudaMemcpyDeviceToDevice, s),
                   "cudaMemcpyAsync");
        m_mass = mass;
    }
    // evaluate at linear-order positions x (eval_terms, diff_scalar_problem.h:310-321)
    void eval_terms(const DenseMatrix<T>& x, cudaStream_t s = nullptr)
    {
        run(x, true, s);
    }
    // energy alone (eval_terms_passive): gradient and Hessian untouched
    T eval_terms_passive(const DenseMatrix<T>& x, cudaStream_t s = nullptr)
    {
        run(x, false, s);
        return (T)m_loss;
    }
    // y = H(x) v without an assembled Hessian (eval_matvec); bc may be null
    void eval_matvec(const DenseMatrix<T>& x, const DenseMatrix<T>& v, DenseMatrix<T>& y,
                     const int8_t* bc = nullptr, cudaStream_t s = nullptr)
    {
        check(rxg_arap_hvp(m_rx->handle(), dtype_of<T>::value, x.data(), m_rest.data(),
                           m_project ? RXG_ARAP_PROJECT_HESSIAN : 0, bc, v.data(), y.data(), s));
    }
    // matrix-free CG on H(x) X = B (CGMatFreeSolver); returns the statistics
    rxg_solver_stats solve_matfree(const DenseMatrix<T>& x, const int8_t* bc,
                                   const DenseMatrix<T>& B, DenseMatrix<T>& X, int max_iter,
                                   double abs_tol, double rel_tol, cudaStream_t s = nullptr)
    {
        rxg_solver_opts  o{max_iter, abs_tol, rel_tol, 0};
        rxg_solver_stats st{};
        rxg_status r = rxg_arap_cg_matfree(m_rx->handle(), dtype_of<T>::value, x.data(),
                                           m_rest.data(), m_project ? RXG_ARAP_PROJECT_HESSIAN : 0,
                                           bc, B.data(), X.data(), &o, &st, s);
        if (r != RXG_ERR_NOT_CONVERGED) check(r);
        return st;
    }
    T get_current_loss() const { return (T)m_loss; }

    DenseMatrix<T>                        grad;
    DeviceArray<T>                        face_energy;
    std::unique_ptr<BlockSparseMatrix<T>> hess;

   private:
    // the ARAP term (if added) first, then the added terms, accumulated
    void run(const DenseMatrix<T>& x, bool derivatives, cudaStream_t s)
    {
        if (!m_rest.size() && m_terms.empty() && !m_xt.size())
            throw Error(RXG_ERR_INVALID, "add a term first");
        rxg_bcsr b    = hess ? hess->bcsr() : rxg_bcsr{};
        rxg_bcsr* hb  = (derivatives && hess) ? &b : nullptr;
        T*        g   = derivatives ? grad.data() : nullptr;
        T*        fe  = derivatives ? face_energy.data() : nullptr;
        double    sum = 0.0;
        bool      first = true;
        if (m_rest.size()) {
            check(rxg_arap_eval_ex(m_rx->handle(), dtype_of<T>::value, x.data(), m_rest.data(),
                                   (m_project && derivatives) ? RXG_ARAP_PROJECT_HESSIAN : 0, &m_loss,
                                   fe, g, hb, s));
            sum   = m_loss;
            first = false;
        }
        if (!m_terms.empty()) {
            // records [E, gradient, packed Hessian] of the largest term kind
            size_t words = 0;
            for (auto& t : m_terms) {
                const int     c = 3 - t.kind;  // vertices per element
                const int64_t n = t.kind == 0 ? m_rx->get_num_faces()
                                  : t.kind == 1 ? m_rx->get_num_edges() : m_rx->get_num_vertices();
                const int     K = c * VariableDim;
                words = std::max(words, (size_t)(1 + K + K * (K + 1) / 2) * (size_t)n);
            }
            if (m_rec.size() < words) m_rec.resize(words);
            for (auto& t : m_terms) {
                t.launch(x.data(), m_rec.data(), s);
                double        e  = 0.0;
                const int32_t fl = first ? 0 : RXG_TERM_ACCUMULATE;
                if (t.kind == 0)
                    check(rxg_face_term_gather(m_rx->handle(), dtype_of<T>::value, VariableDim, m_rec.data(), fl,
                                               &e, first ? fe : nullptr, g, hb, s));
                else if (t.kind == 1)
                    check(rxg_edge_term_gather(m_rx->handle(), dtype_of<T>::value, VariableDim, m_rec.data(), fl,
                                               &e, nullptr, g, hb, s));
                else
                    check(rxg_vertex_term_gather(m_rx->handle(), dtype_of<T>::value, VariableDim, m_rec.data(),
                                                 fl, &e, nullptr, g, hb, s));
                sum += e;
                first = false;
            }
        }
        if (m_xt.size()) {
            double e = 0.0;
            check(rxg_inertia_eval(m_rx->handle(), dtype_of<T>::value, VariableDim, x.data(), m_xt.data(),
                                   (double)m_mass, first ? 0 : RXG_TERM_ACCUMULATE, &e, g, hb, s));
            sum += e;
        }
        m_loss = sum;
    }
    DeviceArray<T>                                               m_xt;
    T                                                            m_mass = T(0);
    struct Term
    {
        int                                            kind;  // 0 per face, 1 per edge, 2 per vertex
        std::function<void(const T*, T*, cudaStream_t)> launch;
    };
    std::vector<Term>                                            m_terms;
    DeviceArray<int32_t>                                         m_fv, m_ev;
    DeviceArray<T>                                               m_rec;
   private:
    const RXMeshStatic* m_rx;
    DeviceArray<T>      m_rest;
    double              m_loss    = 0.0;
    bool                m_project = false;
};

// NewtonSolver (diff/newton_solver.h:17-330) on a DiffScalarProblem and its
// optimisation variable x (linear-order positions, updated in place by
// line_search): compute_direction() solves H dir = -grad with PCG (or CG) on
// the scalar Hessian, or with the matrix-free CG; line_search() backtracks
// with the Armijo test of diff/armijo_condition.h.  As in the reference,
// compute_direction leaves grad negated and the Armijo test uses dir . grad.
// VariableDim: the problem's components per vertex (1, 2 or 3); the
// matrix-free CG (CG_MATFREE) is the ARAP term's, on 3 components.
template <typename T, int VariableDim = 3>
class NewtonSolver
{
   public:
    enum Kind { PCG, CG, CG_MATFREE };
    NewtonSolver(DiffScalarProblem<T, VariableDim>& p, DenseMatrix<T>& x, Kind kind = PCG, int max_iter = 1000,
                 T abs_tol = T(0), T rel_tol = T(1e-6))
        : problem(p), opt_var(x), dir(x.rows(), VariableDim), m_tmp(x.rows(), VariableDim), m_kind(kind),
          m_max_iter(max_iter), m_abs_tol(abs_tol), m_rel_tol(rel_tol)
    {
        if (kind != CG_MATFREE && !p.hess) throw Error(RXG_ERR_INVALID, "the problem has no Hessian");
        if (kind == CG_MATFREE && VariableDim != 3)
            throw Error(RXG_ERR_INVALID, "the matrix-free CG is the ARAP term's (3 components per vertex)");
    }
    void apply_bc(const DeviceArray<int8_t>& bc, cudaStream_t s = nullptr)
    {
        m_bc = bc.data();
        if (m_kind == CG_MATFREE) {
            // no assembled Hessian: the constrained gradient rows only
            check(rxg_dense_zero_rows((int64_t)bc.size(), VariableDim, dtype_of<T>::value, bc.data(),
                                      problem.grad.data(), s));
        } else {
            problem.hess->apply_bc(bc.data(), &problem.grad, s);
        }
    }
    void compute_direction(cudaStream_t s = nullptr)
    {
        problem.grad.multiply(T(-1), s);
        dir.reset(T(0), DEVICE, s);
        if (m_kind == CG_MATFREE) {
            m_stats = problem.solve_matfree(opt_var, m_bc, problem.grad, dir, m_max_iter,
                                            (double)m_abs_tol, (double)m_rel_tol, s);
            return;
        }
        if (!m_A)
            m_A.reset(new SparseMatrix<T>(VariableDim * problem.hess->rows(),
                                          VariableDim * VariableDim * problem.hess->non_zero_blocks()));
        problem.hess->to_csr(*m_A, s);
        rxg_solver_opts o{m_max_iter, (double)m_abs_tol, (double)m_rel_tol, m_kind == PCG ? 1 : 0};
        rxg_csr         c = m_A->csr();
        rxg_status      r = rxg_cg_solve(&c, 1, problem.grad.data(), dir.data(), &o, &m_stats, s);
        if (r != RXG_ERR_NOT_CONVERGED) check(r);
    }
    bool line_search(T s_max = T(1), T shrink = T(0.8), int max_iters = 64, T armijo_const = T(1e-4),
                     cudaStream_t s = nullptr)
    {
        const bool try_one = s_max > T(1);
        T          step    = s_max;
        const T    f       = problem.get_current_loss();
        const T    slope   = dir.dot(problem.grad, false, s);
        for (int i = 0; i < max_iters; ++i) {
            m_tmp.copy_from(opt_var, DEVICE, DEVICE, s);
            m_tmp.axpy(dir, step, s);
            const T f_new = problem.eval_terms_passive(m_tmp, s);
            if (f_new <= f + armijo_const * step * slope) {
                opt_var.copy_from(m_tmp, DEVICE, DEVICE, s);
                return true;
            }
            if (try_one && step > T(1) && step * shrink < T(1)) step = T(1);
            else step *= shrink;
        }
        return false;
    }
    int iter_taken() const { return m_stats.iters; }

    DiffScalarProblem<T, VariableDim>& problem;
    DenseMatrix<T>&                    opt_var;
    DenseMatrix<T>                     dir;

   private:
    DenseMatrix<T>                   m_tmp;
    Kind                             m_kind;
    int                              m_max_iter;
    T                                m_abs_tol, m_rel_tol;
    const int8_t*                    m_bc = nullptr;
    std::unique_ptr<SparseMatrix<T>> m_A;
    rxg_solver_stats                 m_stats{};
};

// Many meshes of uneven size, mixed-precision implicit MCF in one persistent
// launch (graph-captured after the first call).
class MeshBatch
{
   public:
    // meshes: (fv, nv) per mesh, vertex ids local to the mesh
    MeshBatch(const std::vector<std::pair<std::vector<int32_t>, int64_t>>& meshes,
              int32_t                                                     patch_faces = 256)
    {
        std::vector<int32_t> fv;
        std::vector<int64_t> nf, nv;
        for (const auto& m : meshes) {
            fv.insert(fv.end(), m.first.begin(), m.first.end());
            nf.push_back((int64_t)m.first.size() / 3);
            nv.push_back(m.second);
            m_total_vertices += m.second;
        }
        rxg_batch* b = nullptr;
        check(rxg_batch_create((int32_t)meshes.size(), fv.data(), nf.data(), nv.data(), patch_faces,
                               &b));
        m_b.reset(b);
        m_n = (int32_t)meshes.size();
    }
    // xyz: all meshes' FP64 positions one after another, in input order
    void mcf(DenseMatrix<double>& xyz, double dt, int32_t nsteps = 1, double tol = 1e-6,
             int32_t max_iter = 5000, cudaStream_t s = nullptr)
    {
        check(rxg_batch_mcf(m_b.get(), dt, nsteps, tol, max_iter, xyz.data(), s));
    }
    void stats(std::vector<int32_t>& iters, std::vector<int32_t>& converged) const
    {
        iters.resize((size_t)m_n);
        converged.resize((size_t)m_n);
        check(rxg_batch_stats(m_b.get(), iters.data(), converged.data()));
    }
    int32_t num_meshes() const { return m_n; }
    int64_t num_vertices() const { return m_total_vertices; }
    // time the launch shapes on a copy of xyz and keep the fastest
    // (rxg_batch_autotune); returns the chosen threads per CTA
    int32_t autotune(const DenseMatrix<double>& xyz, double dt, int32_t nsteps = 1,
                     double tol = 1e-6, int32_t max_iter = 5000, cudaStream_t s = nullptr)
    {
        int32_t threads = 0, per_sm = 0;
        float   ms      = 0.f;
        check(rxg_batch_autotune(m_b.get(), dt, nsteps, tol, max_iter, xyz.data(), &threads,
                                 &per_sm, &ms, s));
        return threads;
    }
    // the union mesh of all meshes (queries and numbering); owned by the batch
    const rxg_mesh* mesh() const
    {
        const rxg_mesh* m = nullptr;
        check(rxg_batch_mesh(m_b.get(), &m));
        return m;
    }

   private:
    struct Del
    {
        void operator()(rxg_batch* b) const { rxg_batch_destroy(b); }
    };
    std::unique_ptr<rxg_batch, Del> m_b;
    int32_t                         m_n              = 0;
    int64_t                         m_total_vertices = 0;
};

}  // namespace rxg

#if defined(__CUDACC__)
#include "query.cuh"
#endif

#endif  // RXG_RXMESH_HPP
