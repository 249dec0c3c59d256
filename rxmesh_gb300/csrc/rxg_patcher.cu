// Patch partition on the GPU: Lloyd iterations of multi-source region growing
// on the face graph, the scheme of RXMesh's patcher (Patcher::run_lloyd,
// include/rxmesh/patcher/patcher.cu:828-960; kernels in patcher_kernel.cuh):
//
//   seeds (random faces, at least one per connected component, about
//   nf / P in all) -> grow every seed's region one face-ring per level until
//   every face is claimed -> mark faces next to another region (boundary) ->
//   new seed of each region = its face deepest from the region's boundary
//   -> repeat, splitting regions over P faces every fifth iteration with an
//   extra seed on their boundary, until no region holds more than P faces.
//
// Unlike the reference, every step is deterministic: a face reached by
// several regions in the same level goes to the lowest region id (an atomicMin
// claim, then a commit pass), and ties in depth go to the lowest face id, so
// one mesh always gives one partition.  All loops are driven from the host
// with bounded trip counts; no kernel waits on another.
#include <algorithm>
#include <cstdint>
#include <vector>

#include "rxg_device.cuh"

namespace rxg {
namespace {

constexpr int32_t kFree    = -1;
constexpr int32_t kFar     = INT32_MAX;
constexpr int     kThreads = 256;

int grid_of(int64_t n)
{
    return (int)std::max<int64_t>(1, std::min<int64_t>((n + kThreads - 1) / kThreads, 152 * 16));
}

__global__ void k_fill(int32_t* __restrict__ a, int64_t n, int32_t v)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        a[i] = v;
}

// seed p claims its own face and starts the first frontier
__global__ void k_place_seeds(const int32_t* __restrict__ seeds, int32_t np,
                              int32_t* __restrict__ fpatch, int32_t* __restrict__ front,
                              int32_t* __restrict__ psize)
{
    for (int32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        fpatch[seeds[p]] = p;
        front[p]         = seeds[p];
        psize[p]         = 1;
    }
}

// one level of region growing, pass 1: every free neighbour of a frontier
// face records the lowest region that reaches it
__global__ void k_grow_claim(const int32_t* __restrict__ front, int32_t nfront,
                             const int32_t* __restrict__ ff_off, const int32_t* __restrict__ ff_val,
                             const int32_t* __restrict__ fpatch, int32_t* __restrict__ claim)
{
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nfront;
         i += gridDim.x * blockDim.x) {
        const int32_t f = front[i], p = fpatch[f];
        for (int32_t t = ff_off[f]; t < ff_off[f + 1]; ++t) {
            const int32_t g = ff_val[t];
            if (fpatch[g] == kFree) atomicMin(&claim[g], p);
        }
    }
}

// pass 2: each claimed free face joins its region once and enters the next
// frontier
__global__ void k_grow_commit(const int32_t* __restrict__ front, int32_t nfront,
                              const int32_t* __restrict__ ff_off,
                              const int32_t* __restrict__ ff_val, int32_t* __restrict__ fpatch,
                              const int32_t* __restrict__ claim, int32_t* __restrict__ next,
                              int32_t* __restrict__ nnext, int32_t* __restrict__ psize)
{
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nfront;
         i += gridDim.x * blockDim.x) {
        const int32_t f = front[i];
        for (int32_t t = ff_off[f]; t < ff_off[f + 1]; ++t) {
            const int32_t g = ff_val[t];
            const int32_t c = claim[g];
            if (c != kFar && atomicCAS(&fpatch[g], kFree, c) == kFree) {
                next[atomicAdd(nnext, 1)] = g;
                atomicAdd(&psize[c], 1);
            }
        }
    }
}

// faces with a neighbour in another region start the depth search (depth 0)
__global__ void k_boundary(int64_t nf, const int32_t* __restrict__ ff_off,
                           const int32_t* __restrict__ ff_val, const int32_t* __restrict__ fpatch,
                           int32_t* __restrict__ depth, int32_t* __restrict__ front,
                           int32_t* __restrict__ nfront, int32_t* __restrict__ max_bnd)
{
    for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < nf;
         f += (int64_t)gridDim.x * blockDim.x) {
        const int32_t p = fpatch[f];
        bool          b = false;
        for (int32_t t = ff_off[f]; t < ff_off[f + 1]; ++t) b |= fpatch[ff_val[t]] != p;
        depth[f] = b ? 0 : kFar;
        if (b) {
            front[atomicAdd(nfront, 1)] = (int32_t)f;
            atomicMax(&max_bnd[p], (int32_t)f);
        }
    }
}

// one level of the inward search: region-internal neighbours one deeper
__global__ void k_depth_level(const int32_t* __restrict__ front, int32_t nfront,
                              const int32_t* __restrict__ ff_off,
                              const int32_t* __restrict__ ff_val,
                              const int32_t* __restrict__ fpatch, int32_t* __restrict__ depth,
                              int32_t level, int32_t* __restrict__ next, int32_t* __restrict__ nnext)
{
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nfront;
         i += gridDim.x * blockDim.x) {
        const int32_t f = front[i], p = fpatch[f];
        for (int32_t t = ff_off[f]; t < ff_off[f + 1]; ++t) {
            const int32_t g = ff_val[t];
            if (fpatch[g] == p && atomicCAS(&depth[g], kFar, level + 1) == kFar)
                next[atomicAdd(nnext, 1)] = g;
        }
    }
}

// deepest face of each region (lowest id among equals): key = depth << 32 |
// ~face, maximised
__global__ void k_deepest(int64_t nf, const int32_t* __restrict__ fpatch,
                          const int32_t* __restrict__ depth,
                          unsigned long long* __restrict__ best)
{
    for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < nf;
         f += (int64_t)gridDim.x * blockDim.x) {
        const int32_t d = depth[f];
        if (d == kFar) continue;
        const unsigned long long key =
            ((unsigned long long)(uint32_t)d << 32) | (unsigned long long)(~(uint32_t)f);
        atomicMax(&best[fpatch[f]], key);
    }
}

// new seeds: the deepest face; a region with no boundary (a whole
// component) keeps its seed
__global__ void k_reseed(int32_t np, const unsigned long long* __restrict__ best,
                         int32_t* __restrict__ seeds)
{
    for (int32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x)
        if (best[p] != 0ull) seeds[p] = (int32_t)(~(uint32_t)(best[p] & 0xFFFFFFFFull));
}

// largest face id of each region (a split seed for a region without boundary)
__global__ void k_max_face(int64_t nf, const int32_t* __restrict__ fpatch,
                           int32_t* __restrict__ max_face)
{
    for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < nf;
         f += (int64_t)gridDim.x * blockDim.x)
        atomicMax(&max_face[fpatch[f]], (int32_t)f);
}

uint64_t splitmix(uint64_t& s)
{
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z          = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z          = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

struct DevBuf {
    void* p = nullptr;
    ~DevBuf()
    {
        if (p) cudaFree(p);
    }
};

}  // namespace

rxg_status gpu_partition(int64_t nf, const std::vector<int32_t>& ff_off,
                         const std::vector<int32_t>& ff_val, const std::vector<int32_t>& comp,
                         int32_t P, std::vector<int32_t>& face_patch, int32_t& np_out,
                         int32_t& lloyd_runs)
{
    // ---- initial seeds: pseudo-random faces (fixed generator), at least one
    // per component, about nf / P in all, shared by component size
    //      (Patcher::initialize_random_seeds, patcher.cu:431-535)
    std::vector<int32_t> seeds;
    {
        std::vector<int32_t> count(nf, 0), start(nf + 1, 0), members(nf);
        for (int64_t f = 0; f < nf; ++f) ++count[comp[f]];
        for (int64_t f = 0; f < nf; ++f) start[f + 1] = start[f] + count[f];
        std::vector<int32_t> cur(start.begin(), start.end() - 1);
        for (int64_t f = 0; f < nf; ++f) members[cur[comp[f]]++] = (int32_t)f;
        const int64_t total = (nf + P - 1) / P;
        uint64_t      rng   = 0x5EED5EEDull;
        for (int64_t r = 0; r < nf; ++r) {
            const int32_t n = count[r];
            if (n == 0) continue;  // r is not a component root
            int64_t k = std::max<int64_t>(1, (int64_t)((double)n * (double)total / (double)nf + 0.5));
            k = std::min<int64_t>(k, n);
            // partial Fisher-Yates over the component's faces
            int32_t* m = members.data() + start[r];
            for (int64_t i = 0; i < k; ++i) {
                const int64_t j = i + (int64_t)(splitmix(rng) % (uint64_t)(n - i));
                std::swap(m[i], m[j]);
                seeds.push_back(m[i]);
            }
        }
    }
    const int64_t nnz    = (int64_t)ff_val.size();
    const int32_t max_np = (int32_t)std::min<int64_t>(nf, 2 * (int64_t)seeds.size() + 4 * (nf / P) + 64);

    DevBuf b_off, b_val, b_fpatch, b_claim, b_front, b_next, b_depth, b_seeds, b_psize, b_best,
        b_aux, b_cnt;
    auto alloc = [](DevBuf& b, size_t bytes) { return cudaMalloc(&b.p, std::max<size_t>(bytes, 16)); };
    cudaError_t e = cudaSuccess;
    for (auto pr : {std::make_pair(&b_off, (size_t)(nf + 1) * 4), std::make_pair(&b_val, (size_t)nnz * 4),
                    std::make_pair(&b_fpatch, (size_t)nf * 4), std::make_pair(&b_claim, (size_t)nf * 4),
                    std::make_pair(&b_front, (size_t)nf * 4), std::make_pair(&b_next, (size_t)nf * 4),
                    std::make_pair(&b_depth, (size_t)nf * 4), std::make_pair(&b_seeds, (size_t)max_np * 4),
                    std::make_pair(&b_psize, (size_t)max_np * 4),
                    std::make_pair(&b_best, (size_t)max_np * 8),
                    std::make_pair(&b_aux, (size_t)max_np * 4), std::make_pair(&b_cnt, (size_t)16)})
        if (e == cudaSuccess) e = alloc(*pr.first, pr.second);
    if (e != cudaSuccess) return cuda_status(e, "gpu patcher: cudaMalloc");
    int32_t* d_off    = (int32_t*)b_off.p;
    int32_t* d_val    = (int32_t*)b_val.p;
    int32_t* d_fpatch = (int32_t*)b_fpatch.p;
    int32_t* d_claim  = (int32_t*)b_claim.p;
    int32_t* d_front  = (int32_t*)b_front.p;
    int32_t* d_next   = (int32_t*)b_next.p;
    int32_t* d_depth  = (int32_t*)b_depth.p;
    int32_t* d_seeds  = (int32_t*)b_seeds.p;
    int32_t* d_psize  = (int32_t*)b_psize.p;
    int32_t* d_aux    = (int32_t*)b_aux.p;
    int32_t* d_cnt    = (int32_t*)b_cnt.p;
    auto*    d_best   = (unsigned long long*)b_best.p;
    RXG_CUDA_TRY(cudaMemcpy(d_off, ff_off.data(), (size_t)(nf + 1) * 4, cudaMemcpyHostToDevice));
    if (nnz) RXG_CUDA_TRY(cudaMemcpy(d_val, ff_val.data(), (size_t)nnz * 4, cudaMemcpyHostToDevice));

    int32_t              np = (int32_t)seeds.size();
    std::vector<int32_t> psize;
    const int            gf = grid_of(nf);
    constexpr int        kMaxRuns = 200;
    for (lloyd_runs = 1; lloyd_runs <= kMaxRuns; ++lloyd_runs) {
        RXG_CUDA_TRY(cudaMemcpy(d_seeds, seeds.data(), (size_t)np * 4, cudaMemcpyHostToDevice));
        // ---- grow all regions from their seeds, one face ring per level
        k_fill<<<gf, kThreads>>>(d_fpatch, nf, kFree);
        k_fill<<<gf, kThreads>>>(d_claim, nf, kFar);
        k_place_seeds<<<grid_of(np), kThreads>>>(d_seeds, np, d_fpatch, d_front, d_psize);
        int32_t nfront = np, reached = np;
        for (int64_t level = 0; nfront > 0 && level < nf; ++level) {
            RXG_CUDA_TRY(cudaMemsetAsync(d_cnt, 0, 4));
            k_grow_claim<<<grid_of(nfront), kThreads>>>(d_front, nfront, d_off, d_val, d_fpatch,
                                                        d_claim);
            k_grow_commit<<<grid_of(nfront), kThreads>>>(d_front, nfront, d_off, d_val, d_fpatch,
                                                         d_claim, d_next, d_cnt, d_psize);
            RXG_CUDA_TRY(cudaMemcpy(&nfront, d_cnt, 4, cudaMemcpyDeviceToHost));
            std::swap(d_front, d_next);
            reached += nfront;
        }
        RXG_CUDA_TRY(cudaGetLastError());
        if (reached != nf) {
            set_error("gpu patcher: %lld of %lld faces reached from the seeds", (long long)reached,
                      (long long)nf);
            return RXG_ERR_INVALID;
        }
        psize.resize(np);
        RXG_CUDA_TRY(cudaMemcpy(psize.data(), d_psize, (size_t)np * 4, cudaMemcpyDeviceToHost));
        const int32_t largest = *std::max_element(psize.begin(), psize.end());
        if (largest <= P) break;

        // ---- move every seed to its region's deepest face
        RXG_CUDA_TRY(cudaMemsetAsync(d_cnt, 0, 4));
        k_fill<<<grid_of(np), kThreads>>>(d_aux, np, -1);
        k_boundary<<<gf, kThreads>>>(nf, d_off, d_val, d_fpatch, d_depth, d_front, d_cnt, d_aux);
        RXG_CUDA_TRY(cudaMemcpy(&nfront, d_cnt, 4, cudaMemcpyDeviceToHost));
        for (int32_t level = 0; nfront > 0 && level < nf; ++level) {
            RXG_CUDA_TRY(cudaMemsetAsync(d_cnt, 0, 4));
            k_depth_level<<<grid_of(nfront), kThreads>>>(d_front, nfront, d_off, d_val, d_fpatch,
                                                         d_depth, level, d_next, d_cnt);
            RXG_CUDA_TRY(cudaMemcpy(&nfront, d_cnt, 4, cudaMemcpyDeviceToHost));
            std::swap(d_front, d_next);
        }
        RXG_CUDA_TRY(cudaMemsetAsync(d_best, 0, (size_t)np * 8));
        k_deepest<<<gf, kThreads>>>(nf, d_fpatch, d_depth, d_best);
        k_reseed<<<grid_of(np), kThreads>>>(np, d_best, d_seeds);
        RXG_CUDA_TRY(cudaGetLastError());
        std::vector<int32_t> max_bnd(np);
        RXG_CUDA_TRY(cudaMemcpy(max_bnd.data(), d_aux, (size_t)np * 4, cudaMemcpyDeviceToHost));
        RXG_CUDA_TRY(cudaMemcpy(seeds.data(), d_seeds, (size_t)np * 4, cudaMemcpyDeviceToHost));

        // ---- every fifth run, one more seed in each region over P faces:
        // its largest-id boundary face, or its largest face when it has no
        // boundary (Patcher's add_more_seeds, patcher_kernel.cuh:256-300)
        if (lloyd_runs % 5 == 0) {
            std::vector<int32_t> max_face;
            const int32_t        np0 = np;
            for (int32_t p = 0; p < np0; ++p) {
                if (psize[p] <= P) continue;
                int32_t s = max_bnd[p];
                if (s < 0) {
                    if (max_face.empty()) {
                        k_fill<<<grid_of(np0), kThreads>>>(d_aux, np0, -1);
                        k_max_face<<<gf, kThreads>>>(nf, d_fpatch, d_aux);
                        max_face.resize(np0);
                        RXG_CUDA_TRY(cudaMemcpy(max_face.data(), d_aux, (size_t)np0 * 4,
                                                cudaMemcpyDeviceToHost));
                    }
                    s = max_face[p];
                }
                if (s == seeds[p]) continue;  // a one-face boundary region (P >= 16 rules it out)
                if (np == max_np) {
                    set_error("gpu patcher: more than %d patches", max_np);
                    return RXG_ERR_INVALID;
                }
                seeds.push_back(s);
                ++np;
            }
        }
    }
    if (lloyd_runs > kMaxRuns) {
        set_error("gpu patcher: regions still above %d faces after %d Lloyd runs", P, kMaxRuns);
        return RXG_ERR_NOT_CONVERGED;
    }
    face_patch.resize(nf);
    RXG_CUDA_TRY(cudaMemcpy(face_patch.data(), d_fpatch, (size_t)nf * 4, cudaMemcpyDeviceToHost));
    np_out = np;
    return RXG_OK;
}

}  // namespace rxg
