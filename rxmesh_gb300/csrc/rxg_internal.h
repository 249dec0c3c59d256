// Internal structures shared by the translation units of librxg.so.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <string>
#include <vector>

#include "../../include/rxg.h"

namespace rxg {

// Per-patch header, one per CTA of a patch-parallel kernel.  Local ids are
// 16-bit: owned elements first, then ribbon (not-owned) elements.
struct PatchHdr
{
    int32_t nVo, nVl;  // owned / local vertices
    int32_t nEo, nEl;  // owned / local edges
    int32_t nFo, nFl;  // owned / local faces
    int32_t v_base;    // linear id of owned vertex 0
    int32_t e_base;
    int32_t f_base;
    int32_t vv_base;   // first VV/VE value of this patch's owned rows
    int32_t vf_base;   // first VF value of this patch's owned rows
    int32_t ev_off;    // arena word offsets (16-byte aligned slices)
    int32_t fe_off;
    int32_t rv_off;    // ribbon vertex -> linear id
    int32_t re_off;    // ribbon edge   -> linear id
    int32_t rf_off;    // ribbon face   -> linear id
};
static_assert(sizeof(PatchHdr) == 64, "PatchHdr is one 64-byte line");

// Device-resident topology (owned by Mesh).
struct DeviceTopo
{
    PatchHdr* hdr   = nullptr;
    uint32_t* arena = nullptr;  // words: ev (u16 pairs), fe (u16 triples), ribbon tables
    int64_t   arena_words = 0;
    // permutations, linear -> input (device copies for rxg_permute)
    int32_t* v_l2i = nullptr;
    int32_t* e_l2i = nullptr;
    int32_t* f_l2i = nullptr;
    // face -> 3 linear vertex ids (face linear order), used by per-face kernels
    int32_t* fv_lin = nullptr;
    // per-patch incidence blocks of the vertex-normal kernel (see Mesh::nrm)
    uint32_t* nrm     = nullptr;
    int32_t*  nrm_off = nullptr;
    // ef_base (np+1) then ff_base (np+1), see Mesh::ef_base
    int32_t* qbase = nullptr;
};

// An explicit partition in input ids (a saved RXMesh patcher, or the
// caller's own): face -> patch, and optionally the owner patch of each vertex
// and edge.  Without owners, a vertex or edge goes to the lowest-numbered
// patch among its faces' patches (RXMesh's Patcher::assign_patch,
// patcher/patcher.cu:719-757).
struct Partition {
    const int32_t* face   = nullptr;  // nf entries
    const int32_t* vertex = nullptr;  // nv entries or NULL; ignored for vertices in no face
    const int32_t* edge   = nullptr;  // ne entries or NULL
    int64_t        ne     = -1;       // entries of edge
    int32_t        patch_size = 0;    // the patcher's nominal patch size (0: the largest patch)
};

struct Mesh
{
    int64_t nv = 0, ne = 0, nf = 0;
    int32_t patch_faces = 0;
    int32_t num_patches = 0;
    int32_t device      = 0;
    bool    closed = true, edge_manifold = true;
    bool    oriented = true;  // no edge traversed in the same direction by two of its faces
    int64_t max_valence = 0;
    int32_t max_vl = 0, max_el = 0, max_fl = 0, max_vo = 0, max_eo = 0, max_fo = 0;
    int64_t ribbon_v = 0, ribbon_f = 0;

    std::vector<int32_t> ev_in;  // input edge list (ne*2)
    std::vector<int32_t> v_l2i, e_l2i, f_l2i;
    std::vector<int32_t> v_i2l, e_i2l, f_i2l;
    std::vector<PatchHdr> hdr;
    std::vector<uint32_t> arena;
    // Per patch p, words [nrm_off[p], nrm_off[p+1]) of nrm (16-byte aligned):
    // offsets of the owned vertices' incidence lists (u32 x nVo+1, pad4) and
    // the lists (pad4): one word per incident face (input VF order), the
    // face's other two corners after the vertex in the face's cyclic order,
    // local vertex ids a | b << 16.  Static topology, built once with the
    // patches.
    std::vector<uint32_t> nrm;
    std::vector<int32_t>  nrm_off;
    // first EF / FF value of each patch's owned rows (np+1 each; the last
    // entry is the total): the CSR bases of the edge and face queries
    std::vector<int32_t> ef_base, ff_base;
    // the input faces (for rxg_mesh_save_patch_file), the patches that own
    // faces (the rest hold vertices in no face), face-connected components
    std::vector<int32_t> fv_in;
    std::vector<int8_t>  vbnd;  // 1 for a boundary vertex, linear order
    int32_t              num_face_patches = 0, num_components = 0;
    int32_t              lloyd_runs = 0;  // GPU patcher iterations (0: not used)
    int32_t              max_edge_faces = 0, max_face_faces = 0;

    DeviceTopo d;

    // lazily built device structures (guarded by the mesh's own mutex)
    void* lazy = nullptr;

    int64_t device_bytes = 0;
    size_t  smem_bytes[16] = {};  // per kernel kind (query ops 0-9; 11: oriented FF; 12, 13: normals), max over patches
    // rxg_query_sweep: by requested outputs (bit 0 normals, 1 VV, 2 VE, 3 VF,
    // 4 FV, 5 EV; only the slices those outputs read are counted), max over patches
    size_t  sweep_smem[64] = {};

    // calls with host arrays: a copy stream and events that overlap the
    // device-to-host copy of each slice of patches with the kernel of the next
    mutable std::mutex   stage_mu;
    mutable cudaStream_t copy_stream = nullptr;
    mutable cudaEvent_t  copy_ev[4]  = {nullptr, nullptr, nullptr, nullptr};
    // rxg_query_sweep_ex with host outputs: one stream per query kernel
    // (highest priority first) and their completion events, plus the
    // fork and join events (also under stage_mu)
    mutable cudaStream_t sweep_streams[6] = {};
    mutable cudaEvent_t  sweep_ev[8]      = {};
};

void compute_smem_table(Mesh& m);

// thread-local error message
void        set_error(const char* fmt, ...);
rxg_status  cuda_status(cudaError_t e, const char* what);

#define RXG_CUDA_TRY(call)                                   \
    do {                                                     \
        cudaError_t _e = (call);                             \
        if (_e != cudaSuccess) return cuda_status(_e, #call); \
    } while (0)

// Host/device pointer classification: true when p is device-accessible
// memory allocated by CUDA (device or managed).  Host memory (pageable,
// pinned or registered) returns false.
bool is_device_ptr(const void* p);

// Stream-ordered device scratch from the library's own pool (freed with
// cudaFreeAsync); freed blocks stay in the pool for later calls.
cudaError_t scratch_alloc(void** p, size_t bytes, cudaStream_t s);

// Mesh construction behind rxg_mesh_create_ex (part == NULL: the library's
// own BFS partition into patches of at most patch_faces faces) and the
// partitioned / patch-file constructors (rxg_mesh.cpp).
rxg_status create_mesh(const int32_t* fv, int64_t nf, int64_t nv, int32_t patch_faces,
                       int32_t flags, const Partition* part, rxg_mesh** out);

// Partition on the GPU (rxg_patcher.cu): Lloyd region growing on the face
// graph ff (CSR through shared edges) into regions of at most P faces; comp:
// per face, the smallest face id of its connected component.
rxg_status gpu_partition(int64_t nf, const std::vector<int32_t>& ff_off,
                         const std::vector<int32_t>& ff_val, const std::vector<int32_t>& comp,
                         int32_t P, std::vector<int32_t>& face_patch, int32_t& np,
                         int32_t& lloyd_runs);

// Lazily allocated per-mesh device scratch and the oriented ring.
struct Lazy;
Lazy* lazy_of(const Mesh* m);
void  lazy_free(Mesh* m);

// Query kernels entry (rxg_query.cu)
rxg_status launch_query(const Mesh* m, int op, int32_t* d_off, int32_t* d_val,
                        cudaStream_t s);

// Per-device caches are arrays indexed by the CUDA device ordinal.
constexpr int kMaxDevices = 64;

// device error word (bounded waits) of the current device; NULL when there
// is no current device
int* device_error_word();
// multiprocessor count of the current device (cached per device)
int device_sm_count();
// current device ordinal, clamped to [0, kMaxDevices)
int current_device();
rxg_status check_device_error(cudaStream_t s);

}  // namespace rxg

struct rxg_mesh
{
    rxg::Mesh m;
};
