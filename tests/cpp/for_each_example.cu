// Device-side queries through the facade (include/rxg/rxmesh.hpp +
// rxg/query.cuh), written as an RXMesh application writes them:
// RXMeshStatic::for_each<Op, blockThreads>(device lambda), attributes read
// and written through handles, for_each_vertex on the host and the device,
// and run_kernel with a kernel of its own that drives Query<blockThreads>
// (dispatch with an active set, compute_vertex_valence).
//
//   for_each_example <mesh.obj> <patch_size> <out_dir>
// Writes one binary int32 (or float64) file per result into out_dir for the
// test to compare with the oracle, prints "OK" and exits 0; prints the
// failing check and exits 1 otherwise.
//   for_each_example torus <n> <patch_size>
// Times, on an n x n torus, for_each<Op::VV> with a lambda that writes each
// vertex's valence and the sum of its neighbours' ids, against rxg_query VV
// into preallocated device buffers (CUDA events, 20 runs after 3 warm-ups).
#include <cstdio>
#include <string>
#include <vector>

#include "rxg/rxmesh.hpp"

using namespace rxg;

#define REQUIRE(c)                                               \
    do {                                                         \
        if (!(c)) {                                              \
            std::printf("FAILED: %s (line %d)\n", #c, __LINE__); \
            return 1;                                            \
        }                                                        \
    } while (0)

template <typename T>
static void dump(const std::string& path, const T* p, size_t n)
{
    std::FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) throw Error(RXG_ERR_INVALID, "cannot write " + path);
    std::fwrite(p, sizeof(T), n, f);
    std::fclose(f);
}

// an int32 attribute of k values per element of the handle's kind
template <typename H>
static std::shared_ptr<Attribute<int32_t, H>> add_attr(RXMeshStatic& rx, const std::string& n, uint32_t k)
{
    if constexpr (H::kElem == RXG_ELEM_VERTEX)
        return rx.add_vertex_attribute<int32_t>(n, k);
    else if constexpr (H::kElem == RXG_ELEM_EDGE)
        return rx.add_edge_attribute<int32_t>(n, k);
    else
        return rx.add_face_attribute<int32_t>(n, k);
}

// every source element's row of query OP, as linear ids, W slots per row
// (-1 past the row's end), and the row's size
template <Op OP, typename SrcH, typename OutH, int W>
static void run_op(RXMeshStatic& rx, const std::string& dir, const char* name, bool oriented = false)
{
    auto cnt = add_attr<SrcH>(rx, std::string(name) + "_cnt", 1u);
    auto val = add_attr<SrcH>(rx, std::string(name) + "_val", (uint32_t)W);
    cnt->reset(-1, LOCATION_ALL);
    val->reset(-1, LOCATION_ALL);
    Attribute<int32_t, SrcH> c = *cnt, v = *val;
    rx.for_each<OP, 256>(
        [c, v] __device__(const SrcH& h, const Iterator<OutH>& it) {
            c(h) = it.size();
            for (int k = 0; k < it.size() && k < W; ++k) v(h, k) = it[k].linear_id();
        },
        oriented);
    check_cuda(cudaDeviceSynchronize(), "for_each");
    cnt->move(DEVICE, HOST);
    val->move(DEVICE, HOST);
    dump(dir + "/" + name + "_cnt.bin", cnt->data(HOST), (size_t)cnt->size());
    dump(dir + "/" + name + "_val.bin", val->data(HOST), (size_t)val->size() * W);
}

// A kernel of the application's own (run_kernel): the valence of every
// owned vertex and, for even linear ids only (the active set), the VV row
// size; odd vertices keep -1.
template <uint32_t blockThreads>
__global__ void k_active_valence(Context ctx, VertexAttribute<int32_t> out)
{
    auto           block = cooperative_groups::this_thread_block();
    ShmemAllocator shrd_alloc;
    Query<blockThreads> query(ctx);
    query.compute_vertex_valence(block, shrd_alloc);
    query.template dispatch<Op::VV>(
        block, shrd_alloc,
        [&](const VertexHandle& vh, const VertexIterator& it) {
            out(vh) = 1000 * it.size() + query.vertex_valence(vh);
        },
        [](const VertexHandle& vh) { return (vh.linear_id() & 1) == 0; });
}

// Query::prologue / run_compute / epilogue spelled out: per face, the sum of
// its vertices' linear ids
template <uint32_t blockThreads>
__global__ void k_face_sum(Context ctx, FaceAttribute<int32_t> out)
{
    auto           block = cooperative_groups::this_thread_block();
    ShmemAllocator shrd_alloc;
    Query<blockThreads> query(ctx);
    query.template prologue<Op::FV>(block, shrd_alloc);
    query.run_compute(block, [&](const FaceHandle& fh, const VertexIterator& it) {
        out(fh) = it[0].linear_id() + it[1].linear_id() + it[2].linear_id();
    });
    query.epilogue(block, shrd_alloc);
}

static int time_torus(int n, int patch)
{
    std::vector<std::vector<uint32_t>> fv;
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            const uint32_t a = i * n + j, b = ((i + 1) % n) * n + j, c = ((i + 1) % n) * n + (j + 1) % n,
                           d = i * n + (j + 1) % n;
            fv.push_back({a, b, c});
            fv.push_back({a, c, d});
        }
    RXMeshStatic rx(fv, "", (uint32_t)patch);
    auto         V = rx.add_vertex_attribute<int32_t>("valence", 1, DEVICE);
    auto         S = rx.add_vertex_attribute<int32_t>("nsum", 1, DEVICE);
    VertexAttribute<int32_t> val = *V, sum = *S;
    auto run = [&]() {
        rx.for_each<Op::VV, 256>([val, sum] __device__(const VertexHandle& vh, const VertexIterator& it) {
            int32_t s = 0;
            for (uint16_t k = 0; k < it.size(); ++k) s += it[k].linear_id();
            val(vh) = it.size();
            sum(vh) = s;
        });
    };
    int64_t rows = 0, nval = 0;
    check(rxg_query_size(rx.handle(), RXG_OP_VV, &rows, &nval));
    DeviceArray<int32_t> off((size_t)rows + 1), vals((size_t)nval);
    auto q = [&]() { check(rxg_query(rx.handle(), RXG_OP_VV, off.data(), vals.data(), nullptr)); };
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    float t[2];
    for (int w = 0; w < 2; ++w) {
        for (int i = 0; i < 3; ++i) w ? q() : run();
        cudaEventRecord(a);
        for (int i = 0; i < 20; ++i) w ? q() : run();
        cudaEventRecord(b);
        check_cuda(cudaEventSynchronize(b), "timing");
        cudaEventElapsedTime(&t[w], a, b);
    }
    std::printf("torus %d x %d, %u patches: for_each<VV> %.2f us, rxg_query VV %.2f us per call\n", n, n,
                rx.get_num_patches(), 1e3 * t[0] / 20, 1e3 * t[1] / 20);
    std::printf("OK\n");
    return 0;
}

int main(int argc, char** argv)
{
    if (argc >= 4 && std::string(argv[1]) == "torus") {
        try {
            return time_torus(std::stoi(argv[2]), std::stoi(argv[3]));
        } catch (const std::exception& e) {
            std::printf("FAILED: %s\n", e.what());
            return 1;
        }
    }
    if (argc < 4) {
        std::printf("usage: for_each_example <mesh.obj> <patch_size> <out_dir>\n");
        return 2;
    }
    try {
        const std::string dir = argv[3];
        RXMeshStatic      rx(argv[1], "", (uint32_t)std::stoi(argv[2]));
        const uint32_t    nv = rx.get_num_vertices(), nf = rx.get_num_faces();

        run_op<Op::VV, VertexHandle, VertexHandle, 16>(rx, dir, "vv");
        run_op<Op::VV, VertexHandle, VertexHandle, 16>(rx, dir, "vvo", true);
        run_op<Op::VE, VertexHandle, EdgeHandle, 16>(rx, dir, "ve");
        run_op<Op::VF, VertexHandle, FaceHandle, 16>(rx, dir, "vf");
        run_op<Op::FV, FaceHandle, VertexHandle, 3>(rx, dir, "fv");
        run_op<Op::FE, FaceHandle, EdgeHandle, 3>(rx, dir, "fe");
        run_op<Op::FF, FaceHandle, FaceHandle, 16>(rx, dir, "ff");
        run_op<Op::EV, EdgeHandle, VertexHandle, 2>(rx, dir, "ev");
        run_op<Op::EF, EdgeHandle, FaceHandle, 8>(rx, dir, "ef");
        run_op<Op::EVDiamond, EdgeHandle, VertexHandle, 4>(rx, dir, "evd");
        run_op<Op::EE, EdgeHandle, EdgeHandle, 4>(rx, dir, "ee");

        // attributes through handles: the umbrella operator
        // sum_{u in VV(v)} (x_u - x_v) on the input coordinates
        auto X = rx.add_vertex_attribute<double>("x", 3);
        check_cuda(cudaMemcpy(X->data(DEVICE), rx.get_input_vertex_coordinates().data(),
                              sizeof(double) * 3 * nv, cudaMemcpyDeviceToDevice),
                   "cudaMemcpy");
        auto                    Lp = rx.add_vertex_attribute<double>("lap", 3);
        VertexAttribute<double> x = *X, lap = *Lp;
        rx.for_each<Op::VV, 256>([x, lap] __device__(const VertexHandle& vh, const VertexIterator& it) {
            for (int c = 0; c < 3; ++c) {
                double s = 0.0;
                for (uint16_t k = 0; k < it.size(); ++k) s += x(it[k], c) - x(vh, c);
                lap(vh, c) = s;
            }
        });
        Lp->move(DEVICE, HOST);
        dump(dir + "/lap.bin", Lp->data(HOST), (size_t)3 * nv);

        // for_each_vertex / for_each_face on the device and on the host
        auto D = rx.add_vertex_attribute<int32_t>("twice", 1);
        D->reset(-1, LOCATION_ALL);
        VertexAttribute<int32_t> d = *D;
        rx.for_each_vertex(DEVICE, [d] __device__(const VertexHandle vh) { d(vh) = 2 * vh.linear_id(); });
        D->move(DEVICE, HOST);
        for (uint32_t i = 0; i < nv; ++i) REQUIRE(D->data(HOST)[i] == 2 * (int32_t)i);
        D->reset(-1, HOST);
        rx.for_each_vertex(HOST, [d](const VertexHandle vh) { d(vh) = 3 * vh.linear_id(); });
        for (uint32_t i = 0; i < nv; ++i) REQUIRE(D->data(HOST)[i] == 3 * (int32_t)i);
        auto F = rx.add_face_attribute<int32_t>("fid", 1, DEVICE);
        FaceAttribute<int32_t> fa = *F;
        rx.for_each_face(DEVICE, [fa] __device__(const FaceHandle fh) { fa(fh) = fh.linear_id(); });
        std::vector<int32_t> hf(nf);
        check_cuda(cudaMemcpy(hf.data(), F->data(DEVICE), 4 * (size_t)nf, cudaMemcpyDeviceToHost), "copy");
        for (uint32_t i = 0; i < nf; ++i) REQUIRE(hf[i] == (int32_t)i);
        REQUIRE(rx.does_attribute_exist("fid") && rx.get_face_attribute<int32_t>("fid")->size() == nf);
        rx.remove_attribute("fid");
        REQUIRE(!rx.does_attribute_exist("fid"));

        // run_kernel with the application's own kernels
        auto A = rx.add_vertex_attribute<int32_t>("active", 1);
        A->reset(-1, LOCATION_ALL);
        LaunchBox<256> lb;
        rx.prepare_launch_box({Op::VV}, lb, (const void*)k_active_valence<256>, false, true);
        REQUIRE(lb.blocks == rx.get_num_patches() && lb.smem_bytes_dyn > 0);
        rx.run_kernel(lb, k_active_valence<256>, rx.get_context(), *A);
        check_cuda(cudaDeviceSynchronize(), "k_active_valence");
        A->move(DEVICE, HOST);
        dump(dir + "/active.bin", A->data(HOST), (size_t)nv);
        auto S = rx.add_face_attribute<int32_t>("fsum", 1);
        rx.run_kernel<256>({Op::FV}, k_face_sum<256>, rx.get_context(), *S);
        check_cuda(cudaDeviceSynchronize(), "k_face_sum");
        S->move(DEVICE, HOST);
        dump(dir + "/fsum.bin", S->data(HOST), (size_t)nf);

        // the numbering the test maps linear ids back with
        for (int e = 0; e < 3; ++e) {
            const std::vector<int32_t> l2i = rx.linear_to_input(e);
            dump(dir + "/l2i_" + std::to_string(e) + ".bin", l2i.data(), l2i.size());
        }
    } catch (const std::exception& e) {
        std::printf("FAILED: %s\n", e.what());
        return 1;
    }
    std::printf("OK\n");
    return 0;
}
