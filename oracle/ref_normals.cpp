// Compiles the reference's own serial vertex-normal routine
// (apps/VertexNormal/vertex_normal_ref.h:5-85, included from the reference
// tree by oracle/Makefile) behind a C ABI for the tests and the CPU baseline.
// TEST INFRASTRUCTURE ONLY: the product path never loads oracle/_ref.
#include <cstdint>
#include <cstring>
#include <vector>
#include "vertex_normal_ref.h"

template <typename T>
static void run(int64_t nv, int64_t nf, const int32_t* fv, const T* xyz, T* out)
{
    std::vector<std::vector<uint32_t>> faces(nf, std::vector<uint32_t>(3));
    for (int64_t f = 0; f < nf; ++f)
        for (int k = 0; k < 3; ++k) faces[f][k] = (uint32_t)fv[3 * f + k];
    std::vector<std::vector<T>> verts(nv, std::vector<T>(3));
    for (int64_t v = 0; v < nv; ++v)
        for (int k = 0; k < 3; ++k) verts[v][k] = xyz[3 * v + k];
    std::vector<T> vn(3 * nv);
    vertex_normal_ref(faces, verts, vn);
    std::memcpy(out, vn.data(), sizeof(T) * 3 * nv);
}

extern "C" void ref_vertex_normal_f32(int64_t nv, int64_t nf, const int32_t* fv,
                                      const float* xyz, float* out)
{
    run<float>(nv, nf, fv, xyz, out);
}

extern "C" void ref_vertex_normal_f64(int64_t nv, int64_t nf, const int32_t* fv,
                                      const double* xyz, double* out)
{
    run<double>(nv, nf, fv, xyz, out);
}
