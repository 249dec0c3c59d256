// Device helpers shared by the kernels: TMA bulk copies into shared memory
// with an mbarrier, bounded waits that report through an error word instead
// of hanging, and block-wide scans/reductions.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "rxg_internal.h"

namespace rxg {

// error codes OR-ed into the device error word
enum : int {
    DEVERR_MBAR_TIMEOUT   = 1,
    DEVERR_GRID_TIMEOUT   = 2,
    DEVERR_SMEM_OVERFLOW  = 4,
    DEVERR_NONMANIFOLD    = 8,
};

// spin limit of every bounded wait; try_wait itself suspends for a
// hardware-defined interval per attempt, so this bounds a wait to well
// under a second on a healthy GPU while never hanging a faulty one.
constexpr uint32_t kWaitLimit = 1u << 22;

__device__ __forceinline__ uint32_t smem_addr(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
                 : "memory");
    // make the initialised barrier visible to the async (TMA) proxy
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
                 "r"(bytes)
                 : "memory");
}

// global -> shared bulk copy (TMA, non-tensor).  dst, src 16-byte aligned,
// bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
            "r"(smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait on phase `parity` of an mbarrier.  On timeout the error word
// gets DEVERR_MBAR_TIMEOUT, then the thread waits once more (bounded) for
// the copies still in flight and returns false.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, int* err)
{
    for (uint32_t i = 0; i < kWaitLimit; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    if (err) atomicOr(err, DEVERR_MBAR_TIMEOUT);
    for (uint32_t i = 0; i < kWaitLimit; ++i)
        if (mbar_try_wait(bar, parity)) break;
    return false;
}

// bytes of a slice of `words` 32-bit words padded to 16 bytes
__host__ __device__ __forceinline__ uint32_t pad16_bytes(int32_t words)
{
    return (uint32_t)(((words + 3) & ~3) * 4);
}

__host__ __device__ __forceinline__ int32_t pad4i(int32_t n) { return (n + 3) & ~3; }

// Exclusive scan of s[0..n) in place, returns the total.  256-thread blocks.
// Each thread scans a contiguous chunk, warps combine chunk totals with
// shuffles, and warp totals go through shared memory.  Deterministic.
// out (may be null): also written out[i] = base + the exclusive prefix of
// element i, in the same pass (CSR row offsets).
template <int BT>
__device__ __forceinline__ int32_t block_exclusive_scan(int32_t* s, int32_t n, int32_t* s_warp,
                                                        int32_t* __restrict__ out = nullptr, int32_t base = 0)
{
    const int tid   = threadIdx.x;
    const int chunk = (n + BT - 1) / BT;
    const int beg   = min(n, tid * chunk), end = min(n, beg + chunk);
    int32_t   sum   = 0;
    for (int i = beg; i < end; ++i) sum += s[i];
    // inclusive warp scan of per-thread sums
    int32_t x = sum;
    const int lane = tid & 31, warp = tid >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int32_t w = lane < BT / 32 ? s_warp[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < BT / 32) s_warp[lane] = w;  // inclusive warp totals
    }
    __syncthreads();
    int32_t run   = x - sum + (warp > 0 ? s_warp[warp - 1] : 0);
    int32_t total = s_warp[BT / 32 - 1];
    if (out) {
        for (int i = beg; i < end; ++i) {
            int32_t v = s[i];
            s[i]      = run;
            out[i]    = base + run;
            run += v;
        }
    } else {
        for (int i = beg; i < end; ++i) {
            int32_t v = s[i];
            s[i]      = run;
            run += v;
        }
    }
    __syncthreads();
    return total;
}

// Write n values to global dst[gbase .. gbase+n) from 16-bit local ids in
// shared memory (sbuf[j] <-> global (gbase & ~3) + j), each mapped to its
// 32-bit id by map(): 8-byte shared loads and 16-byte global stores in the
// aligned middle, scalar accesses at the ragged ends.  sbuf 8-byte aligned.
template <int BT, typename Map>
__device__ __forceinline__ void store_u16_mapped(int32_t* __restrict__ dst, int64_t gbase,
                                                 const uint16_t* sbuf, int32_t n, const Map& map)
{
    int32_t* const        d    = dst + gbase;           // 64-bit arithmetic once
    const uint16_t* const s    = sbuf + (gbase & 3);    // s[j] <-> d[j]
    const int32_t         lead = min(n, (int32_t)((4 - (gbase & 3)) & 3));
    const int32_t         body = (n - lead) & ~3;
    if ((int32_t)threadIdx.x < lead) d[threadIdx.x] = map(s[threadIdx.x]);
    for (int32_t j = lead + body + threadIdx.x; j < n; j += BT) d[j] = map(s[j]);
    const uint2* s4 = reinterpret_cast<const uint2*>(s + lead);  // 8-byte aligned
    int4*        d4 = reinterpret_cast<int4*>(d + lead);         // 16-byte aligned
    for (int32_t i = threadIdx.x; i < (body >> 2); i += BT) {
        const uint2 w = s4[i];
        int4        o;
        o.x   = map(w.x & 0xffffu);
        o.y   = map(w.x >> 16);
        o.z   = map(w.y & 0xffffu);
        o.w   = map(w.y >> 16);
        d4[i] = o;
    }
}

// Bounded wait on phase `parity` of an mbarrier that suspends the thread
// between attempts (try_wait with a time hint), so a waiting warp issues
// almost nothing.  Same error reporting as mbar_wait_bounded.
__device__ __forceinline__ bool mbar_try_wait_hint(uint64_t* bar, uint32_t parity, uint32_t ns)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity), "r"(ns)
        : "memory");
    return ok != 0;
}

constexpr uint32_t kHintNs         = 20000;  // 20 us per attempt
constexpr uint32_t kHintedAttempts = 25000;  // ~0.5 s in all

__device__ __forceinline__ bool mbar_wait_hinted(uint64_t* bar, uint32_t parity, int* err)
{
    for (uint32_t i = 0; i < kHintedAttempts; ++i)
        if (mbar_try_wait_hint(bar, parity, kHintNs)) return true;
    if (err) atomicOr(err, DEVERR_MBAR_TIMEOUT);
    for (uint32_t i = 0; i < kHintedAttempts; ++i)
        if (mbar_try_wait_hint(bar, parity, kHintNs)) break;
    return false;
}

}  // namespace rxg
