/*
 * rxg.h -- C ABI of the GB300-native RXMesh hot path (librxg.so).
 *
 * Plain pointers and sizes only.  Every call returns an rxg_status; nothing
 * exits or aborts.  `stream` is a cudaStream_t passed as void* (NULL = the
 * legacy default stream).  Unless a function says otherwise, array arguments
 * may live in device memory or in host memory (pageable or pinned); host
 * arrays are staged through library-owned device buffers inside the call and
 * the call returns after the result has landed in the host array.
 *
 * Element numbering.  A mesh keeps two numberings for vertices, edges and
 * faces:
 *   - input ids: the caller's vertex ids, face ids in input order, and edge
 *     ids in first-appearance order over faces, (v0,v1),(v1,v2),(v2,v0) per
 *     face, exactly as RXMesh numbers its global edges
 *     (include/rxmesh/rxmesh.cpp:518-620);
 *   - linear ids: patch-ordered ids, owned elements of patch 0 first, then
 *     patch 1, ... (RXMesh's linear_id, include/rxmesh/context.h:299-331).
 * Queries and per-element arrays passed to kernels use linear ids; the
 * rxg_mesh_linear_to_input gives the permutation and rxg_permute applies it.
 */
#ifndef RXG_H
#define RXG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int rxg_status;
enum {
    RXG_OK                 = 0,
    RXG_ERR_INVALID        = 1, /* bad argument, out-of-range index, size mismatch */
    RXG_ERR_NOMEM          = 2, /* host or device allocation failed */
    RXG_ERR_CUDA           = 3, /* a CUDA runtime call failed (message: rxg_last_error) */
    RXG_ERR_NONMANIFOLD    = 4, /* operation needs an edge- and vertex-manifold mesh */
    RXG_ERR_PATCH_LIMIT    = 5, /* a patch exceeds the 16-bit local-index limits */
    RXG_ERR_NOT_CONVERGED  = 6, /* iterative solver hit max_iter (outputs still valid) */
    RXG_ERR_DEVICE_TIMEOUT = 7, /* a bounded device-side wait gave up */
    RXG_ERR_UNSUPPORTED    = 8,
    RXG_ERR_NO_DEVICE      = 9
};

/* Query operations (RXMesh Op, include/rxmesh/types.h) */
enum {
    RXG_OP_VV = 0, /* vertex -> adjacent vertices   (CSR over vertices) */
    RXG_OP_VE = 1, /* vertex -> incident edges      (CSR over vertices) */
    RXG_OP_VF = 2, /* vertex -> incident faces      (CSR over vertices) */
    RXG_OP_FV = 3, /* face   -> 3 vertices          (dense nf x 3)      */
    RXG_OP_EV = 4, /* edge   -> 2 vertices          (dense ne x 2)      */
    RXG_OP_EF = 5, /* edge   -> incident faces      (CSR over edges)    */
    RXG_OP_FE = 6, /* face   -> 3 edges, edge k from corner k to k+1 (dense nf x 3) */
    RXG_OP_FF = 7, /* face   -> faces sharing an edge (CSR over faces)  */
    RXG_OP_EVD = 8 /* edge   -> diamond: v0, vertex opposite in the face traversing
                      v0->v1, v1, vertex opposite in the face traversing v1->v0;
                      -1 where there is no such face (dense ne x 4; Op::EVDiamond,
                      kernels/rxmesh_queries.cuh:197-262; edge-manifold, consistently
                      oriented meshes, else RXG_ERR_NONMANIFOLD) */,
    RXG_OP_EE = 9  /* edge   -> edges of its faces: for the face traversing the edge
                      from its first vertex (as EV lists it), that face's next and
                      previous edge, then the same for the face traversing it from
                      its second vertex; -1 where there is no such face (dense ne x 4;
                      Op::EE, kernels/rxmesh_queries.cuh:269-340; edge-manifold,
                      consistently oriented meshes, else RXG_ERR_NONMANIFOLD) */
};

enum { RXG_ELEM_VERTEX = 0, RXG_ELEM_EDGE = 1, RXG_ELEM_FACE = 2 };
enum { RXG_F32 = 0, RXG_F64 = 1 };
enum { RXG_NORMAL_MAX = 0, RXG_NORMAL_AREA = 1 };

typedef struct rxg_mesh rxg_mesh;

typedef struct rxg_mesh_info {
    int64_t num_vertices, num_edges, num_faces;
    int64_t num_patches;
    int64_t max_valence;
    int32_t is_closed;          /* every edge has two faces */
    int32_t is_edge_manifold;   /* no edge has more than two faces */
    int32_t patch_faces;        /* requested faces per patch */
    int32_t max_local_vertices; /* largest patch, owned + ribbon */
    int32_t max_local_edges;
    int32_t max_local_faces;
    int64_t ribbon_vertices;    /* sum over patches of not-owned local vertices */
    int64_t ribbon_faces;
    int64_t device_bytes;       /* device memory held by the mesh topology */
    int32_t num_components;     /* face-connected components (get_num_components) */
    int32_t is_oriented;        /* no edge traversed in one direction by two faces */
    int32_t max_edge_incident_faces;  /* get_input_max_edge_incident_faces */
    int32_t max_face_adjacent_faces;  /* get_input_max_face_adjacent_faces */
    int32_t num_face_patches;   /* patches that own faces (the rest hold vertices in no face) */
    int32_t lloyd_runs;         /* GPU patcher iterations (0: not used) */
} rxg_mesh_info;

/* Status name and the last error message of the calling thread. */
const char* rxg_status_string(rxg_status s);
const char* rxg_last_error(void);

/*
 * Build a static mesh from a triangle list (host arrays).  fv: nf*3 vertex
 * ids in [0, nv).  Faces are partitioned into patches of at most patch_faces
 * faces (RXMeshStatic(fv, patcher_file, patch_size), rxmesh_static.h:61-100;
 * build pipeline rxmesh.cpp:86-225).  Topology is uploaded to the current
 * CUDA device.
 */
rxg_status rxg_mesh_create(const int32_t* fv, int64_t nf, int64_t nv,
                           int32_t patch_faces, rxg_mesh** out);
void       rxg_mesh_destroy(rxg_mesh* m);

/* rxg_mesh_create with flags.  RXG_MESH_HOST_ONLY builds the patches on the
 * host and uploads nothing (for inspecting a partition without a GPU; such a
 * mesh can only be passed to the rxg_mesh_* introspection calls).
 * RXG_MESH_SPLIT_COMPONENTS never lets a patch span two connected
 * components, so each component's elements get contiguous linear ids in
 * input order of components (used to pack many meshes into one).
 * RXG_MESH_GPU_PATCHER partitions on the current CUDA device with Lloyd
 * region growing (RXMesh's patcher, patcher/patcher.cu:828-960; needs a GPU,
 * deterministic, patches of at most patch_faces faces, vertex and edge
 * owners as rxg_mesh_create_partitioned gives them); RXG_ERR_NOT_CONVERGED
 * if it has not met the bound after 200 iterations. */
enum { RXG_MESH_HOST_ONLY = 1, RXG_MESH_SPLIT_COMPONENTS = 2, RXG_MESH_GPU_PATCHER = 4 };
rxg_status rxg_mesh_create_ex(const int32_t* fv, int64_t nf, int64_t nv,
                              int32_t patch_faces, int32_t flags, rxg_mesh** out);

/*
 * Build a mesh on a given partition (host arrays, input ids), for
 * reproducible patches.  face_patch: nf patch ids; every id in [0, np) must
 * own 1 to 4096 faces.  vertex_patch (nv) and edge_patch (ne, in
 * rxg_mesh_input_edges order, which is RXMesh's edge numbering) give owners;
 * each must be the patch of one of the element's faces (entries of vertices
 * in no face are ignored).  Either may be NULL: the owner is then the lowest
 * patch among the element's faces (Patcher::assign_patch,
 * patcher/patcher.cu:719-757).  ne: entries of edge_patch, checked against
 * the mesh.  flags: RXG_MESH_HOST_ONLY.
 */
rxg_status rxg_mesh_create_partitioned(const int32_t* fv, int64_t nf, int64_t nv,
                                       const int32_t* face_patch, const int32_t* vertex_patch,
                                       const int32_t* edge_patch, int64_t ne, int32_t flags,
                                       rxg_mesh** out);
/* The partition of a mesh in input ids (host arrays; any may be NULL):
 * nf face, nv vertex and ne edge owner patches.  Vertices in no face are in
 * patches numbered after the face-owning ones. */
rxg_status rxg_mesh_partition(const rxg_mesh* m, int32_t* face_patch, int32_t* vertex_patch,
                              int32_t* edge_patch);
/*
 * RXMeshStatic(fv, patcher_file) (rxmesh_static.h:61-100; Patcher(filename),
 * patcher/patcher.cu:25-32): build on the partition in a patcher file that
 * RXMesh saved (a cereal portable binary archive of Patcher::serialize,
 * patcher/patcher.h:162-181).  The file must be written for this mesh (its
 * vertex, face and edge counts are checked).  RXG_ERR_INVALID with a message
 * for an unreadable, truncated or mismatched file.
 */
rxg_status rxg_mesh_create_from_patch_file(const int32_t* fv, int64_t nf, int64_t nv,
                                           const char* patcher_file, int32_t flags,
                                           rxg_mesh** out);
/* RXMesh::save(filename) (rxmesh.h:326-329): write the mesh's partition as a
 * patcher file that RXMesh and rxg_mesh_create_from_patch_file load. */
rxg_status rxg_mesh_save_patch_file(const rxg_mesh* m, const char* patcher_file);

/*
 * Patch layout for inspection: hdr receives num_patches records of 16 int32
 * {nVo,nVl,nEo,nEl,nFo,nFl, v_base,e_base,f_base, vv_base,vf_base,
 *  ev_off,fe_off,rv_off,re_off,rf_off}; arena receives *words uint32 words
 * (EV as u16 pairs, FE as u16 (edge<<1|dir) triples, ribbon -> linear id
 * tables).  Either may be NULL; *words is always set.  Counterpart of
 * RXMesh's PatchInfo (include/rxmesh/patch_info.h:24-92).
 */
rxg_status rxg_mesh_patches(const rxg_mesh* m, int32_t* hdr, uint32_t* arena,
                            int64_t* words);
rxg_status rxg_mesh_get_info(const rxg_mesh* m, rxg_mesh_info* info);

/*
 * Device view of a mesh's patches, for kernels that run queries themselves
 * (include/rxg/query.cuh: Query<blockThreads>::dispatch, the facade's
 * for_each / run_kernel).  Counterpart of RXMesh's Context
 * (include/rxmesh/context.h:15-120), which kernels receive by value.
 * patch_hdr: num_patches records of 16 int32 in rxg_mesh_patches' layout
 * {nVo,nVl,nEo,nEl,nFo,nFl, v_base,e_base,f_base, vv_base,vf_base,
 *  ev_off,fe_off,rv_off,re_off,rf_off}; arena: the patches' EV (u16 pairs),
 * FE (u16 edge<<1|dir triples) and ribbon -> linear id tables, at those word
 * offsets, every slice 16-byte aligned.  Both are device pointers owned by
 * the mesh (valid until rxg_mesh_destroy).  The max_* fields bound every
 * patch (shared-memory sizing).  RXG_ERR_INVALID for a host-only mesh.
 */
typedef struct rxg_device_context {
    int64_t         num_vertices, num_edges, num_faces;
    int32_t         num_patches;
    int32_t         max_local_vertices, max_local_edges, max_local_faces;
    int32_t         max_owned_vertices, max_owned_edges, max_owned_faces;
    int32_t         max_valence;
    int32_t         max_face_adjacent_faces;
    int32_t         device; /* CUDA ordinal holding the arrays */
    const int32_t*  patch_hdr;
    const uint32_t* arena;
} rxg_device_context;
rxg_status rxg_mesh_device_context(const rxg_mesh* m, rxg_device_context* ctx);

/* lin_to_input (host, n_elem ints): input id of each linear id
 * (RXMeshStatic::map_to_global, rxmesh_static.h:874-905). */
rxg_status rxg_mesh_linear_to_input(const rxg_mesh* m, int32_t elem,
                                    int32_t* lin_to_input);
/* RXMeshStatic::get_boundary_vertices (rxmesh_static.inl:281-323,
 * kernels/boundary.cuh): out[v] = 1 for the ends of every edge with fewer
 * than two faces, else 0; nv int8 in linear order, host or device (a device
 * copy is made on stream, which is synchronised). */
rxg_status rxg_mesh_boundary_vertices(const rxg_mesh* m, int8_t* out, void* stream);
/* Input-numbered edge list (host, ne*2), RXMesh's m_edges_map order. */
rxg_status rxg_mesh_input_edges(const rxg_mesh* m, int32_t* ev);

/*
 * Gather/scatter between input and linear order for per-element arrays of
 * `ncomp` components of `dtype` (RXG_F32/RXG_F64).  to_linear=1: dst[lin] =
 * src[input(lin)], else dst[input(lin)] = src[lin].  Device arrays only.
 * Replaces Attribute construction from / export to input order
 * (rxmesh_static.h:608-793, attribute.h:326-390).
 */
rxg_status rxg_permute(const rxg_mesh* m, int32_t elem, int32_t to_linear,
                       int32_t dtype, int32_t ncomp, const void* src, void* dst,
                       void* stream);

/* ------------------------------------------------------------------ */
/* Queries (Query<blockThreads>::dispatch, query.h:21-75;               */
/* RXMeshStatic::for_each<Op>, rxmesh_static.h:524-566)                 */
/* ------------------------------------------------------------------ */

/* Sizes of a query's output: rows (V, V, V, F, E) and values (2E, 2E, 3F, 3F, 2E). */
rxg_status rxg_query_size(const rxg_mesh* m, int32_t op, int64_t* n_rows,
                          int64_t* n_values);

/*
 * Materialise a query for every owned element, in linear ids.  For
 * VV/VE/VF/EF/FF, offsets has n_rows+1 entries (CSR, row = linear id of the
 * vertex, edge or face); for FV/EV/FE/EVD offsets may be NULL (fixed 3, 2, 3
 * or 4 entries per row).  Order inside a CSR row is unspecified (RXMesh
 * compares rows as sets, tests/RXMesh_test/rxmesh_test.h:347-440).  EF, FE
 * and FF are Op::EF/FE/FF of kernels/rxmesh_queries.cuh:733-858.
 */
rxg_status rxg_query(const rxg_mesh* m, int32_t op, int32_t* offsets,
                     int32_t* values, void* stream);

/*
 * rxg_query and rxg_vertex_normals with flags, for host arrays allocated
 * page-locked (cudaHostAlloc, or registered with cudaHostRegister); both
 * flags make the call stream-ordered: it enqueues its work on `stream` and
 * returns, and the results are in the host arrays once the work `stream`
 * held at return has completed (synchronise the stream or wait on an event
 * recorded on it).  Independent calls on different streams then overlap.
 *   RXG_HOST_ASYNC:  the kernel writes device scratch and a stream-ordered
 *                    copy takes it to the host array (positions come in the
 *                    same way).
 *   RXG_HOST_DIRECT: the kernel reads and writes the page-locked arrays in
 *                    place over the host link: no scratch, no copy.
 * flags = 0, a device or pageable output array, or an argument error: the
 * call is rxg_query / rxg_vertex_normals (synchronous for host arrays).
 * No reference counterpart (RXMesh's queries write device memory only).
 */
enum { RXG_HOST_ASYNC = 1, RXG_HOST_DIRECT = 2 };
rxg_status rxg_query_ex(const rxg_mesh* m, int32_t op, int32_t* offsets, int32_t* values,
                        int32_t flags, void* stream);
rxg_status rxg_vertex_normals_ex(const rxg_mesh* m, int32_t weighting, const float* xyz,
                                 float* out, int32_t flags, void* stream);

/*
 * Several of the vertex-centred queries and the vertex normals in one launch
 * (one CTA per patch): the patch's topology slices are staged once for all
 * of them, and VV and VE share one counting sort.  Any output left NULL is
 * not computed; CSR outputs (VV, VE, VF) come as offsets + values pairs.
 * Each output equals the one rxg_query / rxg_vertex_normals writes (rows of
 * VV, VE, VF as the same sets; FV, EV and normals bit for bit).  Device
 * arrays only; value arrays 16-byte aligned.  The reference runs each query
 * as its own for_each; RXMesh's run_kernel also takes several ops for one
 * kernel of the application's (rxmesh_static.h:450-505).
 */
typedef struct rxg_sweep_out {
    int32_t* vv_offsets; /* nv + 1 */
    int32_t* vv_values;  /* 2 ne */
    int32_t* ve_offsets; /* nv + 1 */
    int32_t* ve_values;  /* 2 ne */
    int32_t* vf_offsets; /* nv + 1 */
    int32_t* vf_values;  /* 3 nf */
    int32_t* fv_values;  /* 3 nf */
    int32_t* ev_values;  /* 2 ne */
    const float* xyz;    /* linear-order positions (nv x 3) for the normals */
    float*   normals;    /* nv x 3 */
    int32_t  weighting;  /* RXG_NORMAL_MAX or RXG_NORMAL_AREA */
} rxg_sweep_out;
rxg_status rxg_query_sweep(const rxg_mesh* m, const rxg_sweep_out* out, void* stream);
/*
 * The same outputs with flags = RXG_HOST_ASYNC: every array (and xyz) may
 * be device memory or page-locked host memory, and the call is stream
 * ordered (it returns at once; the host arrays hold the results when
 * `stream` reaches that point).  The queries then run as separate kernels
 * on the mesh's own streams, quickest first and at the highest priority,
 * and each host result is copied out as soon as its kernel ends, so the
 * host link starts early and stays busy.  flags = 0: rxg_query_sweep.
 */
rxg_status rxg_query_sweep_ex(const rxg_mesh* m, const rxg_sweep_out* out, int32_t flags, void* stream);

/*
 * Oriented VV (Query::dispatch<Op::VV>(..., oriented=true),
 * rxmesh_queries.cuh:376-499): each row lists the one-ring in the rotational
 * order of the incident faces.  A boundary vertex's row starts and ends at
 * its two boundary neighbours and gets boundary[v]=1 (boundary may be NULL).
 * Needs a manifold mesh.
 */
rxg_status rxg_query_oriented_vv(const rxg_mesh* m, int32_t* offsets,
                                 int32_t* values, int8_t* boundary,
                                 void* stream);

/*
 * Per-vertex normals in linear order, FP32.  weighting RXG_NORMAL_MAX:
 * sum over faces of n_f/(|e_a|^2+|e_b|^2) (compute_vertex_normal,
 * apps/VertexNormal/vertex_normal_kernel.cuh:10-43); RXG_NORMAL_AREA: sum of
 * the unnormalised face normals.  xyz, out: nv*3 floats, linear order.
 */
rxg_status rxg_vertex_normals(const rxg_mesh* m, int32_t weighting,
                              const float* xyz, float* out, void* stream);

/*
 * Synchronise `stream`, then read and clear the device error word that
 * bounded device-side waits set instead of hanging (RXG_ERR_DEVICE_TIMEOUT,
 * RXG_ERR_NONMANIFOLD).  No reference counterpart: RXMesh device code uses
 * assert (e.g. kernels/rxmesh_queries.cuh:60-95).
 */
rxg_status rxg_device_check(void* stream);

/*
 * Exercise the bounded-wait error path without faulting or hanging the GPU:
 * one CTA waits on an mbarrier that nothing arrives at, gives up after about
 * 0.1 ms, sets the device error word and returns.  A following
 * rxg_device_check(stream) returns RXG_ERR_DEVICE_TIMEOUT (and clears the
 * word); the context stays usable.  Enqueues only.
 */
rxg_status rxg_selftest_bounded_wait(void* stream);

/* ------------------------------------------------------------------ */
/* Cotangent Laplacian, SpMV, CG/PCG, implicit MCF                      */
/* ------------------------------------------------------------------ */

/* CSR matrix in linear vertex order, diagonal first in each row
 * (SparseMatrix<T>(rx, Op::VV), sparse_matrix.h:77-78,133-241). */
typedef struct rxg_csr {
    int64_t  n;       /* rows = cols */
    int64_t  nnz;
    int32_t* row_ptr; /* device, n+1 */
    int32_t* col;     /* device, nnz */
    void*    val;     /* device, nnz of dtype */
    int32_t  dtype;   /* RXG_F32 or RXG_F64 */
} rxg_csr;

/* Number of rows and non-zeros of the mesh's VV+diagonal pattern. */
rxg_status rxg_mcf_pattern_size(const rxg_mesh* m, int64_t* n, int64_t* nnz);

/*
 * Assemble the implicit-MCF system of mcf_A_setup / mcf_B_setup
 * (apps/MCF/mcf_kernels.cuh:302-426, cotangent weights of
 * geometry_util.cuh:107-206): A = 2M + dt*L, B = 2M x.  xyz: nv*3 FP64,
 * linear order, device.  A must have row_ptr/col/val of the pattern size
 * (they are filled); B: nv*3 of A.dtype (may be NULL).  dtype RXG_F32
 * computes weights in FP32, except for triangles with an angle below 1e-3
 * rad, which are computed in FP64.
 */
rxg_status rxg_mcf_assemble(const rxg_mesh* m, double dt, const double* xyz,
                            rxg_csr* A, void* B, void* stream);

/* Y = A X for nc right-hand sides (row-major n x nc, nc <= 4), dtype of A.
 * (SparseMatrix::multiply, sparse_matrix.h:1173-1263) */
rxg_status rxg_spmm(const rxg_csr* A, int32_t nc, const void* X, void* Y,
                    void* stream);

typedef struct rxg_solver_opts {
    int32_t max_iter;
    double  abs_tol;  /* on delta = |r|^2 (CG) or r.z (PCG) */
    double  rel_tol;  /* on delta / delta_0 */
    int32_t precond;  /* 0 = CG, 1 = Jacobi PCG */
} rxg_solver_opts;

typedef struct rxg_solver_stats {
    int32_t iters;      /* completed iterations (CGSolver::iter_taken) */
    int32_t converged;
    double  start_res;  /* delta_0 */
    double  final_res;  /* final delta */
} rxg_solver_stats;

/*
 * Solve A X = B (nc columns as one long vector), X in/out as the initial
 * guess.  CGSolver / PCGSolver::pre_solve+solve (cg_solver.h:37-125,
 * pcg_solver.h:34-144, iterative_solver.h:52-58).  All scalars stay on the
 * device; the host reads only the final statistics.  Device arrays only
 * (A's row_ptr, col and val, B and X; a host array returns RXG_ERR_INVALID).
 */
rxg_status rxg_cg_solve(const rxg_csr* A, int32_t nc, const void* B, void* X,
                        const rxg_solver_opts* opts, rxg_solver_stats* stats,
                        void* stream);

/*
 * rxg_cg_solve without any device allocation.  No counterpart in the
 * reference: it exists for callers that may not allocate device memory at
 * solve time (an application that owns all device memory through its own
 * pool and budget, a plugin that must not allocate behind its host, code
 * that allocates only at start-up).  Same solver, arguments and statistics
 * as rxg_cg_solve; the work vectors live in a fixed static device array of
 * just over 16 MiB inside the library, which every GPU that loads the
 * library holds until the process exits.
 * Limits: A->n <= 131072 rows and nc <= 3 columns; larger problems return
 * RXG_ERR_INVALID with a message (use rxg_cg_solve).
 * The first call on a device also looks up the array's device address (once
 * per device, with that device current).  Every call reads the solver
 * statistics back to the host, so it returns only after its work on `stream`
 * has finished.  All calls share the
 * one array: calls that overlap on the GPU (other streams, other host
 * threads) race and must be serialised by the caller.  Device arrays only
 * (A's row_ptr, col and val, B and X; a host array returns RXG_ERR_INVALID).
 */
rxg_status rxg_cg_solve_noalloc(const rxg_csr* A, int32_t nc, const void* B,
                                void* X, const rxg_solver_opts* opts,
                                rxg_solver_stats* stats, void* stream);

/*
 * Matrix-free implicit MCF operator: the weights of A = 2M + dt*L (as
 * rxg_mcf_assemble builds it) are recomputed from the positions xyz on every
 * call and nothing is assembled (matvec / precond_matvec / init_B,
 * apps/MCF/mcf_kernels.cuh:58-299).  flags: RXG_MCF_UNIFORM_LAPLACE (weight
 * 1 per neighbour, the valence as vertex weight: use_uniform_laplace),
 * RXG_MCF_JACOBI (rxg_mcf_matvec only: out = D^-1 in, D = diag(A), the
 * preconditioner's product).  xyz: nv*3 FP64; in, out, B: nv*3 of dtype; all
 * linear order, device arrays.  With flags 0, out equals rxg_spmm on the
 * assembled matrix up to rounding.
 */
enum { RXG_MCF_UNIFORM_LAPLACE = 1, RXG_MCF_JACOBI = 2 };
rxg_status rxg_mcf_matvec(const rxg_mesh* m, double dt, int32_t flags, int32_t dtype,
                          const double* xyz, const void* in, void* out, void* stream);
/* B = (1 / v_weight) * xyz: 2 * Voronoi area (cotangent mode) or the
 * valence (uniform mode) times the positions (init_B). */
rxg_status rxg_mcf_init_b(const rxg_mesh* m, int32_t flags, int32_t dtype, const double* xyz,
                          void* B, void* stream);
/*
 * Solve A(xyz) X = B with the matrix-free operator (CGMatFreeAttrSolver /
 * PCGMatFreeAttrSolver, matrix/cg_mat_free_attr_solver.h:45-115): one
 * cooperative launch, the operator's weights recomputed in every product;
 * opts as rxg_cg_solve (3 columns as one vector, X in/out as the initial
 * guess).  flags: RXG_MCF_UNIFORM_LAPLACE.
 */
rxg_status rxg_mcf_solve_matfree(const rxg_mesh* m, double dt, int32_t flags, int32_t dtype,
                                 const double* xyz, const void* B, void* X,
                                 const rxg_solver_opts* opts, rxg_solver_stats* stats,
                                 void* stream);
/*
 * nsteps implicit MCF steps in place on xyz (nv*3 FP64, linear order,
 * device) with the matrix-free operator in FP64 and Jacobi PCG, stopped by
 * the rule of rxg_mcf_step (run_cg_mat_free, apps/MCF/mcf_cg_mat_free.h).
 * flags: RXG_MCF_UNIFORM_LAPLACE.
 */
rxg_status rxg_mcf_step_matfree(const rxg_mesh* m, double dt, int32_t nsteps, int32_t flags,
                                double tol, int32_t max_iter, double* xyz,
                                rxg_solver_stats* stats, void* stream);

/*
 * One or more implicit MCF steps in place on xyz (nv*3 FP64, linear order,
 * device or host).  precision RXG_F64: the plain path (FP64 assembly and the
 * reference's Jacobi-PCG recurrence in FP64).  RXG_F32: FP32 assembly (FP64
 * for triangles with an angle below 1e-3 rad) and FP32 Jacobi-PCG inner
 * solves inside an iterative-refinement loop whose residual B - A x is
 * accumulated in FP64.  Both stop when the Jacobi-weighted residual
 * r.D^-1 r has fallen by tol^2 from its value at the step's start (the PCG
 * measure of pcg_solver.h:34-144), or after max_iter PCG iterations.
 * stats (may be NULL) receives the totals of the last step.
 * (mcf(), apps/MCF/mcf.cu:93-134, run_cg apps/MCF/mcf_cg.h:12-129)
 */
rxg_status rxg_mcf_step(const rxg_mesh* m, double dt, int32_t nsteps,
                        int32_t precision, double tol, int32_t max_iter,
                        double* xyz, rxg_solver_stats* stats, void* stream);

/*
 * Adjoint of one plain (FP64) implicit MCF step x_out = A(x_in)^{-1} B(x_in):
 * given g_out = dl/dx_out, writes g_in = dl/dx_in, including the dependence
 * of the cotangent weights and Voronoi areas on x_in.  One extra Jacobi-PCG
 * solve with the same matrix (A is symmetric) to relative residual tol.
 * All arrays nv*3 FP64, linear order, device.  No counterpart in the
 * reference (its MCF is not differentiable); the forward it inverts is
 * mcf_A_setup / mcf_B_setup (apps/MCF/mcf_kernels.cuh:302-426).
 */
rxg_status rxg_mcf_step_backward(const rxg_mesh* m, double dt,
                                 const double* x_in, const double* x_out,
                                 const double* g_out, double* g_in, double tol,
                                 int32_t max_iter, rxg_solver_stats* stats,
                                 void* stream);

/* ------------------------------------------------------------------ */
/* Batched MCF: many meshes in one persistent launch                    */
/* ------------------------------------------------------------------ */

typedef struct rxg_batch rxg_batch;

/*
 * Pack nmesh triangle meshes into one batch (host arrays).  fv holds the
 * meshes' faces one after another, each with vertex ids local to its mesh;
 * nf[m] / nv[m] are the face / vertex counts of mesh m.  Internally one mesh
 * whose patches never span two meshes (RXMeshStatic packing several meshes,
 * include/rxmesh/rxmesh_static.cu:66-160).  Every mesh must be manifold and
 * use all of its vertices.
 */
rxg_status rxg_batch_create(int32_t nmesh, const int32_t* fv, const int64_t* nf,
                            const int64_t* nv, int32_t patch_faces,
                            rxg_batch** out);
void       rxg_batch_destroy(rxg_batch* b);
/* The union mesh (for queries and numbering); owned by the batch. */
rxg_status rxg_batch_mesh(const rxg_batch* b, const rxg_mesh** mesh);

/*
 * nsteps mixed-precision implicit MCF steps (as rxg_mcf_step with
 * RXG_F32) on every mesh of the batch, in place on xyz (device, sum(nv)*3
 * FP64, meshes one after another in their input order).  One persistent
 * launch: each CTA takes a mesh (largest first) and runs its whole flow.
 * The first call on a batch allocates its work arrays; later calls
 * allocate nothing and do not synchronise, so they can be captured in a
 * CUDA graph.  No counterpart in the reference (one mesh per launch there).
 */
rxg_status rxg_batch_mcf(rxg_batch* b, double dt, int32_t nsteps, double tol,
                         int32_t max_iter, double* xyz, void* stream);

/* Per-mesh PCG iterations and convergence flags of the last rxg_batch_mcf
 * (host arrays of nmesh ints, either may be NULL; synchronises). */
rxg_status rxg_batch_stats(const rxg_batch* b, int32_t* iters, int32_t* converged);

/*
 * Autotuner: times rxg_batch_mcf on a copy of xyz for CTA sizes 256/512/1024
 * and 1-8 CTAs per SM (within occupancy) and keeps the fastest for later
 * calls.  xyz is not modified.
 */
rxg_status rxg_batch_autotune(rxg_batch* b, double dt, int32_t nsteps, double tol,
                              int32_t max_iter, const double* xyz, int32_t* threads,
                              int32_t* blocks_per_sm, float* best_ms, void* stream);

/* ------------------------------------------------------------------ */
/* Per-face ARAP energy, gradient, Hessian (DiffScalarProblem path)     */
/* ------------------------------------------------------------------ */

/* D x D-block CSR over the [diagonal, one-ring] pattern of
 * rxg_mcf_pattern_size (HessianSparseMatrix<T,K>,
 * diff/hessian_sparse_matrix.h:16-137); val holds nnzb row-major D x D
 * blocks.  block_dim: 1, 2 or 3 (0 means 3). */
typedef struct rxg_bcsr {
    int64_t  n;         /* block rows */
    int64_t  nnzb;      /* blocks */
    int32_t* row_ptr;   /* device, n+1 */
    int32_t* col;       /* device, nnzb */
    void*    val;       /* device, D*D*nnzb of dtype */
    int32_t  dtype;
    int32_t  block_dim; /* D: 1, 2 or 3; 0 = 3 */
} rxg_bcsr;

/*
 * Flat rest frame per face from rest positions (FP64, nv*3, linear order):
 * rest receives Mr^{-1} (row-major 2x2, nf*4 of dtype, face linear order),
 * Mr built as apps/Param/param.cu:113-141 does.  Device arrays.
 */
rxg_status rxg_arap_rest(const rxg_mesh* m, const double* xyz_rest,
                         int32_t dtype, void* rest, void* stream);

/*
 * Per-face ARAP energy E_f = A_f ||J_f - R(J_f)||_F^2, J_f = [b-a, c-a] Mr^{-1},
 * R the polar factor, A_f the rest area; its gradient and exact Hessian
 * (DiffScalarProblem::eval_terms / grad / hess / get_current_loss,
 * diff/diff_scalar_problem.h:310-363; per-element kernel
 * diff/diff_query_kernel.cuh:199-322).  x: nv*3 of dtype (linear order);
 * energy: total (device or host double, may be NULL); face_E (nf, may be
 * NULL); grad (nv*3, may be NULL, overwritten); hess (may be NULL; row_ptr,
 * col and val are overwritten).  Needs a manifold mesh.
 */
rxg_status rxg_arap_eval(const rxg_mesh* m, int32_t dtype, const void* x,
                         const void* rest, double* energy, void* face_E,
                         void* grad, rxg_bcsr* hess, void* stream);

/*
 * rxg_arap_eval with flags.  RXG_ARAP_PROJECT_HESSIAN: each face's 9x9
 * Hessian is made positive definite before assembly, as the reference's
 * add_term<Op::FV, ProjectHess = true> (diff/diff_query_kernel.cuh:244-251,
 * project_positive_definite of diff/hessian_projection.h:21-95: left alone
 * when positive diagonally dominant with margin eps, else eigenvalues below
 * eps raised to eps; eps 1e-9 FP64, 1e-6 FP32).  Energy and gradient are
 * unaffected; without a Hessian the flag has no effect.
 */
enum { RXG_ARAP_PROJECT_HESSIAN = 1 };
rxg_status rxg_arap_eval_ex(const rxg_mesh* m, int32_t dtype, const void* x,
                            const void* rest, int32_t flags, double* energy,
                            void* face_E, void* grad, rxg_bcsr* hess, void* stream);

/*
 * Generic per-face energy terms (DiffScalarProblem::add_term<Op::FV,
 * ProjectHess>(lambda), diff/diff_scalar_problem.h:127-194): an energy of
 * the D components of each face's three vertices (D = 2, e.g. uv, or 3).
 * A term is evaluated face by face into records of
 * 1 + 3D + 3D(3D+1)/2 values of dtype each (E, the gradient in the order
 * corner 0 components, corner 1, corner 2 -- the face's vertices in input
 * order -- then the Hessian's upper triangle, row-major), nf records in face
 * linear order, by the library's built-in terms or by an application's own
 * kernel (include/rxg/diff.cuh: Scalar<T, K, Hess>, face_term_kernel).
 * rxg_face_term_gather assembles them: energy (host or device double, may
 * be NULL) = the sum of the face energies, face_E (nf of dtype, may be
 * NULL), grad (nv*D, may be NULL) and hess (D x D blocks, D*D*nnzb values,
 * over the [diagonal, one-ring] pattern of rxg_mcf_pattern_size; may be
 * NULL).  RXG_TERM_ACCUMULATE adds into grad and hess (the sum of several
 * terms) instead of overwriting them.  Needs a manifold mesh.
 */
enum { RXG_TERM_ACCUMULATE = 1, RXG_TERM_PROJECT_HESSIAN = 2 };
rxg_status rxg_face_term_gather(const rxg_mesh* m, int32_t dtype, int32_t dim, const void* records,
                                int32_t flags, double* energy, void* face_E, void* grad,
                                rxg_bcsr* hess, void* stream);
/*
 * Generic per-edge and per-vertex terms (add_term<Op::EV> and add_term<Op::V>
 * of diff/diff_scalar_problem.h:127-194), assembled like
 * rxg_face_term_gather.  An edge term's records hold 1 + 2D + 2D(2D+1)/2
 * values (E, the gradient for the edge's two vertices in EV order, the
 * packed upper Hessian), ne records in edge linear order; a vertex term's
 * 1 + D + D(D+1)/2 values, nv records in vertex linear order
 * (include/rxg/diff.cuh: edge_term_kernel, vertex_term_kernel).  edge_E /
 * vertex_E: the per-element energies (ne or nv of dtype, may be NULL).
 * Without RXG_TERM_ACCUMULATE the gradient and the whole Hessian are
 * overwritten (a vertex term's off-diagonal blocks cleared).  Needs a
 * manifold mesh (the Hessian's one-ring pattern).
 */
rxg_status rxg_edge_term_gather(const rxg_mesh* m, int32_t dtype, int32_t dim, const void* records,
                                int32_t flags, double* energy, void* edge_E, void* grad,
                                rxg_bcsr* hess, void* stream);
rxg_status rxg_vertex_term_gather(const rxg_mesh* m, int32_t dtype, int32_t dim, const void* records,
                                  int32_t flags, double* energy, void* vertex_E, void* grad,
                                  rxg_bcsr* hess, void* stream);

/*
 * The symmetric Dirichlet energy of Param (apps/Param/param.cu:146-183), a
 * built-in term with D = 2: per face E = A (|J|_F^2 + |J^-1|_F^2), J = M
 * Mr^-1, M = [b - a, c - a] of the uv positions (uv: nv*2 of dtype, linear
 * order), rest = Mr^-1 per face (nf*4, rxg_arap_rest), A = det(Mr) / 2; a
 * face with det(M) <= 0 gets the largest finite value and no derivatives,
 * as the reference's energy returns.  flags: RXG_TERM_PROJECT_HESSIAN (each
 * face's 6x6 Hessian made positive definite, project_positive_definite),
 * RXG_TERM_ACCUMULATE.  Outputs as rxg_face_term_gather (hess: 2x2 blocks).
 */
rxg_status rxg_symdir_eval(const rxg_mesh* m, int32_t dtype, const void* uv, const void* rest,
                           int32_t flags, double* energy, void* face_E, void* grad, rxg_bcsr* hess,
                           void* stream);

/*
 * Inertia term of a mass-spring system (add_inertia_term of
 * tests/RXMesh_test/test_hess.cu:13-29, a per-vertex Op::V term): E =
 * sum_v mass/2 |x_v - x_target_v|^2; gradient mass (x - x_target); Hessian
 * mass I on every diagonal block.  x, x_target: nv*dim of dtype (dim 2 or
 * 3), linear order, device.  Without RXG_TERM_ACCUMULATE grad and the whole
 * Hessian are overwritten; with it, added to.  energy: host or device
 * double, may be NULL.
 */
rxg_status rxg_inertia_eval(const rxg_mesh* m, int32_t dtype, int32_t dim, const void* x,
                            const void* x_target, double mass, int32_t flags, double* energy,
                            void* grad, rxg_bcsr* hess, void* stream);

/*
 * Scalar CSR (3n x 3n) of a 3x3-block CSR, the form the reference's
 * CG/PCG solvers work on for a Hessian (HessianSparseMatrix,
 * diff/hessian_sparse_matrix.h:16-137): scalar row 3i+a lists, block by
 * block in the block row's order, the entries 3j+0..2 of block (i,j).
 * out->row_ptr (3n+1), out->col and out->val (9*nnzb) are caller-allocated
 * device arrays; n, nnz and dtype are set.  Feeds rxg_cg_solve (nc = 1).
 */
rxg_status rxg_bcsr_to_csr(const rxg_bcsr* H, rxg_csr* out, void* stream);

/*
 * Dense vector operations of DenseMatrix (matrix/dense_matrix.h:284-334,
 * 446-640) on device arrays of n values of dtype: y = a*x + b*y
 * (axpy: b = 1; multiply by a scalar: x = NULL, a = 0; copy: b = 0; with
 * a = 0 or b = 0 that term is dropped, not multiplied), and the dot product
 * of x and y (FP64 accumulation, deterministic) into *out, a host or device
 * double (a host *out synchronises the stream).
 */
rxg_status rxg_dense_axpby(int64_t n, int32_t dtype, double a, const void* x, double b,
                           void* y, void* stream);
rxg_status rxg_dense_dot(int64_t n, int32_t dtype, const void* x, const void* y,
                         double* out, void* stream);
/*
 * Zero the rows i of a row-major n x ncols array x (dtype) whose mask[i]
 * is non-zero: the gradient half of NewtonSolver::apply_bc when there is no
 * assembled Hessian (diff/newton_solver.h).  Device arrays; enqueues only.
 */
rxg_status rxg_dense_zero_rows(int64_t n, int32_t ncols, int32_t dtype, const int8_t* mask,
                               void* x, void* stream);

/*
 * apply_bc of NewtonSolver (diff/newton_solver.h): for every vertex i with
 * bc[i] != 0, block row i gets the identity as its diagonal block and zero
 * off-diagonal blocks, every block (j, i) is zeroed, and row i of grad
 * (n*3, H's dtype, may be NULL) is zeroed.  Device arrays.
 */
rxg_status rxg_bcsr_apply_bc(rxg_bcsr* H, const int8_t* bc, void* grad, void* stream);

/*
 * Hessian-vector product without an assembled Hessian (the reference's
 * DiffScalarProblem::eval_matvec, diff/diff_query_kernel.cuh:26-148):
 * y = H(x) v for the ARAP term at positions x (nv*3, linear order), v, y
 * nv*3 of dtype; flags as rxg_arap_eval_ex (RXG_ARAP_PROJECT_HESSIAN).  bc
 * (nv int8, may be NULL): constrained vertices get identity rows and zero
 * columns, the Hessian that apply_bc would leave.  Device arrays.
 */
rxg_status rxg_arap_hvp(const rxg_mesh* m, int32_t dtype, const void* x,
                        const void* rest, int32_t flags, const int8_t* bc,
                        const void* v, void* y, void* stream);

/*
 * Matrix-free CG on H(x) X = B (CGMatFreeSolver, matrix/cg_mat_free_solver.h,
 * un-preconditioned: opts->precond must be 0), H as in rxg_arap_hvp; each
 * face is evaluated once per call, then every iteration's product is a
 * per-vertex gather over the fan faces.  One cooperative launch; stops when
 * r.r < abs_tol or r.r / r0.r0 < rel_tol, or after max_iter iterations
 * (RXG_ERR_NOT_CONVERGED).  B, X: nv*3 of dtype, X is the initial guess.
 */
rxg_status rxg_arap_cg_matfree(const rxg_mesh* m, int32_t dtype, const void* x,
                               const void* rest, int32_t flags, const int8_t* bc,
                               const void* B, void* X, const rxg_solver_opts* opts,
                               rxg_solver_stats* stats, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* RXG_H */
