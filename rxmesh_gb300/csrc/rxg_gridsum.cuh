// Deterministic block- and grid-wide sums for persistent solver kernels.
//
// GB300 runs FP64 at about 1/64 of the FP32 rate, so a reduction in which
// every thread shuffles and adds doubles, or in which every thread then
// divides two doubles to get alpha and beta, costs microseconds per CG
// iteration.  Here per-thread FP32 partials are reduced in FP32 inside each
// warp; only the per-warp totals are summed in FP64, by one warp; and the
// scalar recurrence (alpha, beta, stopping tests) runs once per CTA in a
// caller-supplied `post` step on thread 0, which publishes FP32 scalars and
// flags through shared memory.
//
// Grid exchange: each CTA stores its FP64 partial, adds 1 to a ticket
// counter with release semantics and polls it with acquire loads until all
// G tickets of the round are in; then warp 0 of every CTA sums the G
// partials in the same fixed order, so every CTA gets the bit-identical
// total one round trip after the last arrival.  Partials are double-buffered
// by round parity (a CTA cannot reach round k+2 before every CTA has left
// round k).  Every poll is bounded: on timeout the CTA sets
// DEVERR_GRID_TIMEOUT and an abort word that the other CTAs poll, and all
// return false.
#pragma once

#include "rxg_device.cuh"

namespace rxg {

__device__ __forceinline__ void red_add_release(unsigned* p, unsigned v)
{
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Device state of one grid-sum sequence: bar[0] ticket counter, bar[1]
// abort word (both zeroed before the launch), part[2 * G] partials.
struct GridSum
{
    unsigned* bar;
    double*   part;
    int*      err;
    unsigned  G;      // CTAs taking part
    unsigned  round;  // sums done so far
    unsigned  slot;   // this CTA's partial slot, 0..G-1
};

// per-CTA shared scratch of the reductions
struct RedSmem
{
    double warp[32];
    int    ok;
};

// thread partials -> RedSmem::warp[] (FP32 butterfly inside each warp)
template <int BT>
__device__ __forceinline__ void warp_partials(float v, RedSmem& r)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) r.warp[threadIdx.x >> 5] = (double)v;
}

// FP64 thread partials (residual norms: rare, so the FP64 butterfly is fine)
template <int BT>
__device__ __forceinline__ void warp_partials(double v, RedSmem& r)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) r.warp[threadIdx.x >> 5] = v;
}

// FP64 sum of the CTA's warp totals, in warp 0, valid in every lane
template <int BT>
__device__ __forceinline__ double block_total_warp0(const RedSmem& r)
{
    const int lane = threadIdx.x & 31;
    double    t    = lane < BT / 32 ? r.warp[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    return t;
}

// Exchange of the CTA totals already in RedSmem::warp[0..NW) among the G CTAs
// of a grid or gang: thread 0 of each CTA runs post(total) before the CTA's
// threads continue.  Returns false on timeout.
template <int NW, typename Post>
__device__ __forceinline__ bool grid_sum_core(GridSum& g, RedSmem& r, Post post)
{
    __syncthreads();
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        double    t    = lane < NW ? r.warp[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        double* pk = g.part + (g.round & 1u) * g.G;
        int     ok = 1;
        if (g.G == 1) {  // a CTA on its own: no exchange
            if (lane == 0) {
                r.ok = 1;
                post(t);
            }
            goto done;
        }
        if (lane == 0) {
            __stcg(pk + g.slot, t);
            red_add_release(g.bar, 1u);
            const unsigned target = (g.round + 1u) * g.G;
            uint32_t       it     = 0;
            while ((int)(ld_acquire_u32(g.bar) - target) < 0) {
                ++it;
                if ((it & 1023u) == 0u && ld_acquire_u32(g.bar + 1) != 0u) {
                    ok = 0;  // another CTA gave up
                    break;
                }
                if (it > kWaitLimit) {
                    if (g.err) atomicOr(g.err, DEVERR_GRID_TIMEOUT);
                    atomicExch(g.bar + 1, 1u);
                    ok = 0;
                    break;
                }
            }
        }
        ok = __shfl_sync(0xffffffffu, ok, 0);
        __syncwarp();  // lane 0's acquire before the other lanes' loads
        double acc = 0.0;
        if (ok) {
            if (g.G <= 256) {
                double q[8];
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    const unsigned i = lane + 32u * k;
                    q[k]             = i < g.G ? __ldcg(pk + i) : 0.0;
                }
#pragma unroll
                for (int k = 0; k < 8; ++k) acc += q[k];
            } else {
                for (unsigned i = lane; i < g.G; i += 32) acc += __ldcg(pk + i);
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) {
            r.ok = ok;
            if (ok) post(acc);
        }
    }
done:
    __syncthreads();
    ++g.round;
    return r.ok != 0;
}

// Sum over the grid of every thread's partial v (FP32: reduced in FP32 per
// warp; FP64: FP64 warp butterfly, for rare reductions).
template <int BT, typename V, typename Post>
__device__ __forceinline__ bool grid_sum(V v, GridSum& g, RedSmem& r, Post post)
{
    warp_partials<BT>(v, r);
    return grid_sum_core<BT / 32>(g, r, post);
}

// FP64 partials of every iteration (the FP64 solver): staged in shared
// memory (s_part: BT doubles) and summed by warp 0, so the CTA does BT FP64
// adds instead of 5 BT.
template <int BT, typename Post>
__device__ __forceinline__ bool grid_sum_staged(double v, double* s_part, GridSum& g, RedSmem& r,
                                                Post post)
{
    s_part[threadIdx.x] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        double t = 0.0;
#pragma unroll 8
        for (int k = 0; k < BT / 32; ++k) t += s_part[threadIdx.x + 32 * k];
        r.warp[threadIdx.x] = t;
    }
    return grid_sum_core<32>(g, r, post);
}

// Same protocol within one CTA (no grid exchange): post(block total).
template <int BT, typename V, typename Post>
__device__ __forceinline__ void block_sum_post(V v, RedSmem& r, Post post)
{
    warp_partials<BT>(v, r);
    __syncthreads();
    if (threadIdx.x < 32) {
        const double t = block_total_warp0<BT>(r);
        if (threadIdx.x == 0) post(t);
    }
    __syncthreads();
}

}  // namespace rxg
