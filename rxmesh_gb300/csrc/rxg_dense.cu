// Dense vector operations of DenseMatrix (include/rxmesh/matrix/dense_matrix.h:
// axpy, multiply by a scalar, copy, dot, norm2 -- 284-334, 446-640), for
// callers that hold device arrays without a tensor library: y = a x + b y in
// one pass, and a deterministic dot product (per-block FP64 partials summed
// in a fixed order by one block).
#include <algorithm>

#include "rxg_device.cuh"
#include "rxg_lazy.h"

namespace rxg {

template <typename T>
__global__ void k_axpby(int64_t n, T a, const T* __restrict__ x, T b, T* __restrict__ y)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        y[i] = (b == T(0) ? T(0) : b * y[i]) + (a == T(0) ? T(0) : a * x[i]);
}

template <typename T>
__global__ void k_zero_rows(int64_t n, int32_t nc, const int8_t* __restrict__ mask, T* __restrict__ x)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n * nc;
         i += (int64_t)gridDim.x * blockDim.x)
        if (mask[i / nc]) x[i] = T(0);
}

constexpr int kDotBlocks = 296, kDotThreads = 256;

template <typename T>
__global__ void __launch_bounds__(kDotThreads) k_dot_partial(int64_t n, const T* __restrict__ x,
                                                             const T* __restrict__ y,
                                                             double* __restrict__ part)
{
    __shared__ double s[kDotThreads];
    double            acc = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        acc += (double)x[i] * (double)y[i];
    s[threadIdx.x] = acc;
    __syncthreads();
    for (int o = kDotThreads / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = s[0];
}

__global__ void k_dot_final(const double* __restrict__ part, int n, double* __restrict__ out)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double t = 0.0;
        for (int i = 0; i < n; ++i) t += part[i];
        *out = t;
    }
}

}  // namespace rxg

using namespace rxg;

extern "C" {

rxg_status rxg_dense_axpby(int64_t n, int32_t dtype, double a, const void* x, double b, void* y,
                           void* stream)
{
    if (n < 0 || !y || (a != 0.0 && !x) || (dtype != RXG_F32 && dtype != RXG_F64)) {
        set_error("rxg_dense_axpby: bad argument");
        return RXG_ERR_INVALID;
    }
    if (!is_device_ptr(y) || (x && !is_device_ptr(x))) {
        set_error("rxg_dense_axpby: x and y must be device arrays");
        return RXG_ERR_INVALID;
    }
    if (n == 0) return RXG_OK;
    cudaStream_t s = (cudaStream_t)stream;
    const int    g = grid_for_items(n);
    if (dtype == RXG_F64)
        k_axpby<double><<<g, 256, 0, s>>>(n, a, (const double*)x, b, (double*)y);
    else
        k_axpby<float><<<g, 256, 0, s>>>(n, (float)a, (const float*)x, (float)b, (float*)y);
    RXG_CUDA_TRY(cudaGetLastError());
    return RXG_OK;
}

rxg_status rxg_dense_zero_rows(int64_t n, int32_t ncols, int32_t dtype, const int8_t* mask, void* x,
                               void* stream)
{
    if (n < 0 || ncols <= 0 || !mask || !x || (dtype != RXG_F32 && dtype != RXG_F64)) {
        set_error("rxg_dense_zero_rows: bad argument");
        return RXG_ERR_INVALID;
    }
    if (!is_device_ptr(mask) || !is_device_ptr(x)) {
        set_error("rxg_dense_zero_rows: mask and x must be device arrays");
        return RXG_ERR_INVALID;
    }
    if (n == 0) return RXG_OK;
    cudaStream_t s = (cudaStream_t)stream;
    const int    g = grid_for_items(n * ncols);
    if (dtype == RXG_F64)
        k_zero_rows<double><<<g, 256, 0, s>>>(n, ncols, mask, (double*)x);
    else
        k_zero_rows<float><<<g, 256, 0, s>>>(n, ncols, mask, (float*)x);
    RXG_CUDA_TRY(cudaGetLastError());
    return RXG_OK;
}

rxg_status rxg_dense_dot(int64_t n, int32_t dtype, const void* x, const void* y, double* out,
                         void* stream)
{
    if (n < 0 || !x || !y || !out || (dtype != RXG_F32 && dtype != RXG_F64)) {
        set_error("rxg_dense_dot: bad argument");
        return RXG_ERR_INVALID;
    }
    if (!is_device_ptr(x) || !is_device_ptr(y)) {
        set_error("rxg_dense_dot: x and y must be device arrays");
        return RXG_ERR_INVALID;
    }
    cudaStream_t s = (cudaStream_t)stream;
    double*      part;
    RXG_CUDA_TRY(scratch_alloc((void**)&part, sizeof(double) * (kDotBlocks + 1), s));
    if (dtype == RXG_F64)
        k_dot_partial<double><<<kDotBlocks, kDotThreads, 0, s>>>(n, (const double*)x,
                                                               (const double*)y, part);
    else
        k_dot_partial<float><<<kDotBlocks, kDotThreads, 0, s>>>(n, (const float*)x,
                                                              (const float*)y, part);
    k_dot_final<<<1, 32, 0, s>>>(part, kDotBlocks, part + kDotBlocks);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) {
        if (is_device_ptr(out)) {
            e = cudaMemcpyAsync(out, part + kDotBlocks, sizeof(double), cudaMemcpyDeviceToDevice, s);
        } else {
            e = cudaMemcpyAsync(out, part + kDotBlocks, sizeof(double), cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        }
    }
    cudaFreeAsync(part, s);
    if (e != cudaSuccess) return cuda_status(e, "rxg_dense_dot");
    return RXG_OK;
}

}  // extern "C"
