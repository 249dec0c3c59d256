// Per-mesh structures built on first use: the oriented one-ring (with the
// face that follows each ring entry), the [diagonal, ring...] CSR pattern
// shared by the MCF matrix and the ARAP block Hessian, and solver scratch.
#pragma once

#include <mutex>

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
    int32_t*   row_ptr    = nullptr;  // nv+1  (= ring_off + p)
    int32_t*   col        = nullptr;  // nnz   (diagonal first, then the ring)
    int64_t    nnz        = 0;
    // MCF step scratch (sized for this mesh)
    void*   buf      = nullptr;
    size_t  buf_size = 0;
};

// Builds the ring and pattern once per mesh (thread-safe); needs a manifold mesh.
rxg_status ensure_pattern(const Mesh* m, cudaStream_t s, Lazy** out);

int grid_for_items(int64_t work);

}  // namespace rxg
