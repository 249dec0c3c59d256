// Compiles the reference's own cotangent and Voronoi-area routines
// (include/rxmesh/geometry_util.cuh:50-206: tri_area, clamp_cot,
// partial_voronoi_area, edge_cotan_weight), included from the reference
// tree by oracle/Makefile through the glm stand-ins in oracle/shim/, behind
// a C ABI for the pinning tests of the oracle's restatement.
// TEST INFRASTRUCTURE ONLY: the product path never loads oracle/_ref.
#define __host__
#define __device__
#define __inline__ inline
#define __forceinline__ inline
#include <algorithm>
#include <cassert>
#include <cmath>
#include <cstdint>
#include <limits>

// the reference calls isnan / isinf unqualified (CUDA's global overloads)
using std::isinf;
using std::isnan;

#include "rxmesh/geometry_util.cuh"

template <typename T>
static rxmesh::vec3<T> at(const T* p, int64_t i)
{
    return rxmesh::vec3<T>(p[3 * i], p[3 * i + 1], p[3 * i + 2]);
}

// out[i] = partial_voronoi_area(P[i], Q[i], R[i]) (p center, q before, r after)
extern "C" void ref_partial_voronoi_area_f64(int64_t n, const double* P, const double* Q,
                                             const double* R, double* out)
{
    for (int64_t i = 0; i < n; ++i)
        out[i] = rxmesh::partial_voronoi_area<double>(at(P, i), at(Q, i), at(R, i));
}

extern "C" void ref_partial_voronoi_area_f32(int64_t n, const float* P, const float* Q,
                                             const float* R, float* out)
{
    for (int64_t i = 0; i < n; ++i)
        out[i] = rxmesh::partial_voronoi_area<float>(at(P, i), at(Q, i), at(R, i));
}

// out[i] = edge_cotan_weight(P[i], R[i], Q[i], S[i]) (edge p-r, opposite q, s)
extern "C" void ref_edge_cotan_weight_f64(int64_t n, const double* P, const double* R,
                                          const double* Q, const double* S, double* out)
{
    for (int64_t i = 0; i < n; ++i)
        out[i] = rxmesh::edge_cotan_weight<double>(at(P, i), at(R, i), at(Q, i), at(S, i));
}

extern "C" void ref_edge_cotan_weight_f32(int64_t n, const float* P, const float* R,
                                          const float* Q, const float* S, float* out)
{
    for (int64_t i = 0; i < n; ++i)
        out[i] = rxmesh::edge_cotan_weight<float>(at(P, i), at(R, i), at(Q, i), at(S, i));
}

extern "C" void ref_tri_area_f64(int64_t n, const double* P, const double* Q, const double* R,
                                 double* out)
{
    for (int64_t i = 0; i < n; ++i) out[i] = rxmesh::tri_area<double>(at(P, i), at(Q, i), at(R, i));
}
