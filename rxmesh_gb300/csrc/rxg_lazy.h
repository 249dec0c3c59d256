// Per-mesh structures built on first use: the oriented one-ring (with the
// face that follows each ring entry), the [diagonal, ring...] CSR pattern
// shared by the MCF matrix and the ARAP block Hessian, and solver scratch.
#pragma once

#include <mutex>
#include <vector>

#include "rxg_internal.h"

namespace rxg {

struct Lazy
{
    std::mutex mu;
    bool       ring_ready = false;
    int32_t*   ring_off   = nullptr;  // nv+1, linear ids
    int32_t*   ring       = nullptr;  // 2*ne
    int8_t*    bnd        = nullptr;  // nv
    int32_t*   ring_face  = nullptr;  // 2*ne: face between ring[i] and ring[i+1] (-1: none)
    int32_t*   ring_edge  = nullptr;  // 2*ne: 2 * (edge to ring[i]) + (the row vertex's end of it, 0 or 1)
    int32_t*   row_ptr    = nullptr;  // nv+1  (= ring_off + p)
    int32_t*   col        = nullptr;  // nnz   (diagonal first, then the ring)
    int64_t    nnz        = 0;
    // MCF step scratch (sized for this mesh)
    void*   buf      = nullptr;
    size_t  buf_size = 0;
    // row ranges of the on-chip mixed solver's CTAs, balanced by cost
    std::vector<int32_t> oc_bounds;             // G+1, host copy
    int32_t*             d_oc_bounds = nullptr;  // G+1, device
    int32_t              oc_cp       = 0;        // shared-memory stride (max rows, rounded to 32)
};

// Builds the ring and pattern once per mesh (thread-safe); needs a manifold mesh.
rxg_status ensure_pattern(const Mesh* m, cudaStream_t s, Lazy** out);

int grid_for_items(int64_t work);

// Mixed-precision MCF solve with the PCG state in shared memory
// (rxg_onchip.cu): one cooperative launch runs the FP64-residual refinement
// and its FP32 Jacobi-PCG sweeps for the FP32 packed matrix (Ent<float>),
// FP64 diagonal, FP64 B4 and X4 (4-wide rows); Z4 is n 4-wide FP32 rows of
// scratch.  mcf_onchip_fits says whether n rows of at most max_row entries
// fit on chip.
bool       mcf_onchip_fits(int64_t n, int64_t max_row);
size_t     mcf_onchip_scratch_bytes(int64_t n, int64_t max_row);
rxg_status mcf_onchip_solve(Lazy* z, int64_t n, int64_t max_row, const void* ent_f32,
                            const double* diag, const void* B4, void* X4, void* Z4, void* scratch,
                            double tol, int max_iter, cudaStream_t s);
rxg_status mcf_onchip_stats(const void* scratch, rxg_solver_stats* st, cudaStream_t s);

}  // namespace rxg
