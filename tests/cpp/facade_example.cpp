// C++ use of the rxg facade (include/rxg/rxmesh.hpp), written the way an
// RXMesh application drives the same path: build an RXMeshStatic, run
// queries, assemble the MCF system, solve it with PCGSolver, take MCF steps,
// evaluate the ARAP term, and run a small batch.
//
//   facade_example host [dir] -- mesh build and numbering only (no GPU
//                                needed); with dir, a patcher-file round trip
//   facade_example gpu    -- the whole path on the current GPU
// Prints "OK" and exits 0 when every check passes; prints the failing check
// and exits 1 otherwise.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <set>
#include <vector>

#include "rxg/rxmesh.hpp"

using namespace rxg;

#define REQUIRE(c)                                                 \
    do {                                                           \
        if (!(c)) {                                                \
            std::printf("FAILED: %s (line %d)\n", #c, __LINE__);   \
            return 1;                                              \
        }                                                          \
    } while (0)

// closed torus on an n x m (u, v) grid, two triangles per cell
static void torus(int n, int m, std::vector<std::vector<uint32_t>>& fv,
                  std::vector<std::vector<double>>& xyz)
{
    const double R = 1.0, r = 0.3, pi = 3.14159265358979323846;
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < m; ++j) {
            const double u = 2 * pi * i / n, v = 2 * pi * j / m;
            xyz.push_back({(R + r * std::cos(v)) * std::cos(u), (R + r * std::cos(v)) * std::sin(u),
                           r * std::sin(v)});
            const uint32_t a = i * m + j, b = ((i + 1) % n) * m + j, c = ((i + 1) % n) * m + (j + 1) % m,
                           d = i * m + (j + 1) % m;
            fv.push_back({a, b, c});
            fv.push_back({a, c, d});
        }
}

// open k x k grid in the plane z = 0, spacing 1
static void grid(int k, std::vector<int32_t>& fv, std::vector<double>& xyz)
{
    for (int i = 0; i < k; ++i)
        for (int j = 0; j < k; ++j) {
            xyz.push_back(j);
            xyz.push_back(i);
            xyz.push_back(0.0);
        }
    for (int i = 0; i + 1 < k; ++i)
        for (int j = 0; j + 1 < k; ++j) {
            const int a = i * k + j, b = a + 1, c = a + k + 1, d = a + k;
            const int t[6] = {a, b, c, a, c, d};
            fv.insert(fv.end(), t, t + 6);
        }
}

static int host_checks(const char* dir)
{
    std::vector<std::vector<uint32_t>> fv;
    std::vector<std::vector<double>>   xyz;
    torus(48, 32, fv, xyz);
    RXMeshStatic rx(fv, "", 128, /*host_only=*/true);
    REQUIRE(rx.get_num_vertices() == 48 * 32);
    REQUIRE(rx.get_num_faces() == 2 * 48 * 32);
    REQUIRE(rx.get_num_edges() == 3 * 48 * 32);
    REQUIRE(rx.is_closed() && rx.is_edge_manifold());
    REQUIRE(rx.get_num_patches() >= 24);
    const std::vector<int32_t> l2i = rx.linear_to_input(RXG_ELEM_VERTEX);
    std::set<int32_t>          seen(l2i.begin(), l2i.end());
    REQUIRE(seen.size() == l2i.size() && *seen.begin() == 0);
    const std::vector<int8_t> bnd = rx.get_boundary_vertices();  // closed torus: none
    REQUIRE(bnd.size() == l2i.size() && std::count(bnd.begin(), bnd.end(), 1) == 0);
    bool threw = false;
    try {
        std::vector<std::vector<uint32_t>> bad = {{0, 1}};
        RXMeshStatic                       r2(bad, "", 128, true);
    } catch (const Error& e) {
        threw = e.status == RXG_ERR_INVALID;
    }
    REQUIRE(threw);
    {
        // a given partition: two halves of the faces by input order
        std::vector<int32_t> half(fv.size());
        for (size_t f = 0; f < fv.size(); ++f) half[f] = f < fv.size() / 2 ? 0 : 1;
        RXMeshStatic         two(fv, half, true);
        std::vector<int32_t> fp, vp, ep;
        two.partition(fp, vp, ep);
        REQUIRE(two.get_num_patches() == 2 && fp == half);
    }
    if (dir) {
        // save the partition, load it back: the same patches and numbering
        const std::string path = std::string(dir) + "/torus_patches";
        rx.save(path);
        RXMeshStatic back(fv, path, 512, true);
        REQUIRE(back.get_num_patches() == rx.get_num_patches());
        std::vector<int32_t> fp0, vp0, ep0, fp1, vp1, ep1;
        rx.partition(fp0, vp0, ep0);
        back.partition(fp1, vp1, ep1);
        REQUIRE(fp0 == fp1 && vp0 == vp1 && ep0 == ep1);
        REQUIRE((int64_t)fp0.size() == rx.get_num_faces());
        REQUIRE(back.linear_to_input(RXG_ELEM_VERTEX) == l2i);
        REQUIRE(back.linear_to_input(RXG_ELEM_EDGE) == rx.linear_to_input(RXG_ELEM_EDGE));
        threw = false;
        try {
            RXMeshStatic r3(fv, std::string(dir) + "/missing_patches", 512, true);
        } catch (const Error& e) {
            threw = e.status == RXG_ERR_INVALID;
        }
        REQUIRE(threw);

        // OBJ constructor: a quad (fanned), a triangle in v/t/n form, a
        // relative index; the same mesh as its face list
        const std::string obj = std::string(dir) + "/quad.obj";
        std::FILE*        fp  = std::fopen(obj.c_str(), "w");
        REQUIRE(fp != nullptr);
        std::fputs("# two faces\nv 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nv 2 0 0\n"
                   "vt 0 0\nvn 0 0 1\nf 1 2 3 4\nf 2/1/1 -1/1/1 3/1/1\n",
                   fp);
        std::fclose(fp);
        RXMeshStatic from_obj(obj, "", 512, true);
        REQUIRE(from_obj.get_num_vertices() == 5 && from_obj.get_num_faces() == 3);
        REQUIRE(from_obj.get_num_edges() == 7);
        std::vector<std::vector<uint32_t>> qf = {{0, 1, 2}, {0, 2, 3}, {1, 4, 2}};
        RXMeshStatic                       from_fv(qf, "", 512, true);
        REQUIRE(from_obj.linear_to_input(RXG_ELEM_EDGE) == from_fv.linear_to_input(RXG_ELEM_EDGE));
        // two files, two regions
        const std::string tri = std::string(dir) + "/tri.obj";
        fp                    = std::fopen(tri.c_str(), "w");
        REQUIRE(fp != nullptr);
        std::fputs("v 0 0 1\nv 1 0 1\nv 0 1 1\nf 1 2 3\n", fp);
        std::fclose(fp);
        RXMeshStatic both(std::vector<std::string>{obj, tri}, 512, true);
        REQUIRE(both.get_num_regions() == 2 && both.get_num_faces() == 4);
        REQUIRE((both.get_region_label(RXG_ELEM_FACE) == std::vector<int32_t>{0, 0, 0, 1}));
        const std::vector<int32_t> el = both.get_region_label(RXG_ELEM_EDGE);
        REQUIRE(std::count(el.begin(), el.end(), 1) == 3 && el.size() == 10);
        threw = false;
        try {
            RXMeshStatic r4(std::string(dir) + "/missing.obj", "", 512, true);
        } catch (const Error& e) {
            threw = e.status == RXG_ERR_INVALID;
        }
        REQUIRE(threw);
    }
    return 0;
}

static int gpu_checks(const char* dir)
{
    std::vector<std::vector<uint32_t>> fv;
    std::vector<std::vector<double>>   xyz;
    torus(96, 64, fv, xyz);
    RXMeshStatic rx(fv);
    rx.add_vertex_coordinates(xyz);
    const uint32_t nv = rx.get_num_vertices();
    const std::vector<int32_t> vl2i = rx.linear_to_input(RXG_ELEM_VERTEX);

    // VV: every torus vertex has valence 6 and adjacency is symmetric
    QueryResult                vv  = rx.query(Op::VV);
    const std::vector<int32_t> off = vv.offsets.to_host(), val = vv.values.to_host();
    REQUIRE((int64_t)off.size() == nv + 1);
    std::set<std::pair<int32_t, int32_t>> adj;
    for (uint32_t v = 0; v < nv; ++v) {
        REQUIRE(off[v + 1] - off[v] == 6);
        for (int32_t k = off[v]; k < off[v + 1]; ++k) adj.insert({(int32_t)v, val[k]});
    }
    for (const auto& e : adj) REQUIRE(adj.count({e.second, e.first}) == 1);

    // FV maps back to the input faces (up to rotation)
    QueryResult                fvq  = rx.query(Op::FV);
    const std::vector<int32_t> fval = fvq.values.to_host();
    const std::vector<int32_t> fl2i = rx.linear_to_input(RXG_ELEM_FACE);
    for (size_t f = 0; f < fl2i.size(); ++f) {
        const auto& in = fv[(size_t)fl2i[f]];
        int         a = vl2i[fval[3 * f]], b = vl2i[fval[3 * f + 1]], c = vl2i[fval[3 * f + 2]];
        bool        same = false;
        for (int r = 0; r < 3; ++r) {
            same |= (int)in[r] == a && (int)in[(r + 1) % 3] == b && (int)in[(r + 2) % 3] == c;
        }
        REQUIRE(same);
    }

    // FF on the closed torus: every face has three edge neighbours; EVDiamond:
    // every edge has both opposite vertices, distinct from its endpoints
    QueryResult                ffq   = rx.query(Op::FF);
    const std::vector<int32_t> ffoff = ffq.offsets.to_host();
    for (size_t f = 0; f + 1 < ffoff.size(); ++f) REQUIRE(ffoff[f + 1] - ffoff[f] == 3);
    QueryResult                dq = rx.query(Op::EVDiamond);
    const std::vector<int32_t> dv = dq.values.to_host();
    REQUIRE(dv.size() == 4 * (size_t)rx.get_num_edges());
    for (size_t e = 0; e < dv.size() / 4; ++e) {
        const int32_t* d = &dv[4 * e];
        REQUIRE(d[1] >= 0 && d[3] >= 0 && d[1] != d[3]);
        REQUIRE(d[1] != d[0] && d[1] != d[2] && d[3] != d[0] && d[3] != d[2]);
    }

    // input order -> linear order on the device: the coordinates that
    // add_vertex_coordinates placed; and back
    {
        std::vector<double> hin;
        for (const auto& p : xyz) hin.insert(hin.end(), p.begin(), p.end());
        DenseMatrix<double> xin(nv, 3), xlin(nv, 3), xback(nv, 3);
        xin.from_host(hin);
        rx.to_linear(RXG_ELEM_VERTEX, xin, xlin);
        rx.to_input(RXG_ELEM_VERTEX, xlin, xback);
        device_check();
        REQUIRE(xlin.to_host() == rx.get_input_vertex_coordinates().to_host());
        REQUIRE(xback.to_host() == hin);
    }

    // export_obj, read back: the same mesh in linear numbering
    if (dir) {
        const std::string path = std::string(dir) + "/torus_out.obj";
        rx.export_obj(path, rx.get_input_vertex_coordinates());
        RXMeshStatic back(path, "", 512, true);
        REQUIRE(back.get_num_vertices() == nv && back.get_num_faces() == rx.get_num_faces());
        REQUIRE(back.get_num_edges() == rx.get_num_edges() && back.is_closed());
    }

    // MCF system + Jacobi PCG: |A X - B| / |B| small
    const double        dt = 1e-3;
    SparseMatrix<double> A(rx);
    DenseMatrix<double>  B(rx, nv, 3), X(rx, nv, 3), AX(nv, 3);  // both constructor forms
    mcf_assemble(rx, dt, rx.get_input_vertex_coordinates(), A, B);
    PCGSolver<double> solver(A, 3, 2000, 1e-20, 0.0);
    solver.pre_solve(B, X);
    solver.solve(B, X);
    REQUIRE(solver.iter_taken() > 0 && solver.converged());
    REQUIRE(A(0, 0) > 0.0 && A(0, (int64_t)nv + 5) == 0.0);  // diagonal; no such column
    A.multiply(X, AX);
    const std::vector<double> hb = B.to_host(), hax = AX.to_host();
    double                    num = 0, den = 0;
    for (size_t i = 0; i < hb.size(); ++i) {
        num += (hax[i] - hb[i]) * (hax[i] - hb[i]);
        den += hb[i] * hb[i];
    }
    REQUIRE(std::sqrt(num / den) < 1e-8);

    // the same solve through the entry point that allocates nothing (6,144
    // rows, inside its fixed scratch): the same iterations and solution
    {
        DenseMatrix<double> Xn(nv, 3);
        PCGSolver<double>   s2(A, 3, 2000, 1e-20, 0.0);
        s2.solve_noalloc(B, Xn);
        REQUIRE(s2.converged() && s2.iter_taken() == solver.iter_taken());
        const std::vector<double> hx = X.to_host(), hn = Xn.to_host();
        double                    d = 0, mx = 0;
        for (size_t i = 0; i < hx.size(); ++i) {
            d  = std::max(d, std::fabs(hx[i] - hn[i]));
            mx = std::max(mx, std::fabs(hx[i]));
        }
        REQUIRE(d <= 1e-12 * mx);
    }

    // mcf_step: plain FP64 against mixed precision
    DenseMatrix<double> x64(nv, 3), x32(nv, 3);
    const std::vector<double> x0 = rx.get_input_vertex_coordinates().to_host();
    x64.from_host(x0);
    x32.from_host(x0);
    mcf_step(rx, x64, dt, 3, RXG_F64, 1e-8);
    mcf_step(rx, x32, dt, 3, RXG_F32, 1e-8);
    const std::vector<double> h64 = x64.to_host(), h32 = x32.to_host();
    num = den = 0;
    for (size_t i = 0; i < h64.size(); ++i) {
        num += (h64[i] - h32[i]) * (h64[i] - h32[i]);
        den += h64[i] * h64[i];
    }
    REQUIRE(std::sqrt(num / den) < 1e-6);

    // ARAP: zero energy and gradient at rest, positive after a stretch
    std::vector<int32_t> gfv;
    std::vector<double>  gx;
    grid(24, gfv, gx);
    std::vector<std::vector<uint32_t>> gf;
    for (size_t t = 0; t < gfv.size(); t += 3)
        gf.push_back({(uint32_t)gfv[t], (uint32_t)gfv[t + 1], (uint32_t)gfv[t + 2]});
    RXMeshStatic gr(gf);
    std::vector<std::vector<double>> gxyz;
    for (size_t i = 0; i < gx.size(); i += 3) gxyz.push_back({gx[i], gx[i + 1], gx[i + 2]});
    gr.add_vertex_coordinates(gxyz);
    DiffScalarProblem<double> prob(gr);
    prob.add_arap_term(gr.get_input_vertex_coordinates());
    prob.eval_terms(gr.get_input_vertex_coordinates());
    REQUIRE(std::fabs(prob.get_current_loss()) < 1e-12);
    const std::vector<double> g0 = prob.grad.to_host();
    for (double g : g0) REQUIRE(std::fabs(g) < 1e-10);
    std::vector<double> stretched = gr.get_input_vertex_coordinates().to_host();
    for (size_t i = 0; i < stretched.size(); i += 3) stretched[i] *= 1.1;
    DenseMatrix<double> xs(gr.get_num_vertices(), 3);
    xs.from_host(stretched);
    prob.eval_terms(xs);
    REQUIRE(prob.get_current_loss() > 1e-3);
    REQUIRE(prob.hess && prob.hess->non_zero_blocks() > 0);

    // DenseMatrix vector operations against the same arithmetic on the host
    {
        const int64_t       n = gr.get_num_vertices();
        std::vector<double> ha(3 * n), hb(3 * n);
        for (int64_t i = 0; i < 3 * n; ++i) {
            ha[i] = std::sin(0.37 * (double)i);
            hb[i] = std::cos(0.11 * (double)i) - 0.25;
        }
        DenseMatrix<double> a(n, 3), b(n, 3), c(n, 3);
        a.from_host(ha);
        b.from_host(hb);
        double dot = 0, nrm = 0;
        for (int64_t i = 0; i < 3 * n; ++i) {
            dot += ha[i] * hb[i];
            nrm += ha[i] * ha[i];
        }
        REQUIRE(std::fabs(a.dot(b) - dot) <= 1e-12 * std::fabs(dot) + 1e-12);
        REQUIRE(std::fabs(a.norm2() - std::sqrt(nrm)) <= 1e-12 * std::sqrt(nrm));
        c.copy_from(a);
        c.multiply(2.5);
        c.axpy(b, -0.5);
        const std::vector<double> hc = c.to_host();
        for (int64_t i = 0; i < 3 * n; ++i) REQUIRE(std::fabs(hc[i] - (2.5 * ha[i] - 0.5 * hb[i])) <= 1e-14);
        DenseMatrix<float>  fa(n, 3);
        std::vector<float>  hf(ha.begin(), ha.end());
        fa.from_host(hf);
        double fdot = 0;
        for (float v : hf) fdot += (double)v * (double)v;
        REQUIRE(std::fabs((double)fa.dot(fa) - fdot) <= 1e-6 * fdot);
    }

    // Newton with the corners fixed (NewtonSolver): the energy drops, the
    // corners stay put, and the assembled-PCG and matrix-free paths agree
    {
        const int64_t       n = gr.get_num_vertices();
        const std::vector<int32_t> gl2i = gr.linear_to_input(RXG_ELEM_VERTEX);
        std::vector<int8_t> hbc((size_t)n, 0);
        for (int64_t l = 0; l < n; ++l) {
            const int32_t v = gl2i[(size_t)l];
            if (v == 0 || v == 23 || v == 24 * 23 || v == 24 * 24 - 1) hbc[(size_t)l] = 1;
        }
        DeviceArray<int8_t> bc((size_t)n);
        bc.upload(hbc.data(), hbc.size());
        std::vector<double> bent = gr.get_input_vertex_coordinates().to_host();
        for (int64_t l = 0; l < n; ++l) {
            const double u = bent[3 * l], w = bent[3 * l + 1];
            bent[3 * l + 2] = 0.2 * std::sin(3.0 * u) * std::cos(2.0 * w);
            if (hbc[(size_t)l]) bent[3 * l] *= 1.2;
        }
        double last[2] = {0, 0};
        for (int k = 0; k < 2; ++k) {
            DiffScalarProblem<double> p(gr, k == 0);
            p.add_arap_term(gr.get_input_vertex_coordinates(), nullptr, true);
            DenseMatrix<double> x(n, 3);
            x.from_host(bent);
            NewtonSolver<double> newton(p, x, k == 0 ? NewtonSolver<double>::PCG
                                                     : NewtonSolver<double>::CG_MATFREE,
                                        5000, 0.0, 1e-24);
            double first = 0;
            for (int it = 0; it < 4; ++it) {
                p.eval_terms(x);
                if (it == 0) first = p.get_current_loss();
                newton.apply_bc(bc);
                newton.compute_direction();
                REQUIRE(newton.iter_taken() > 0);
                REQUIRE(newton.line_search());
            }
            last[k] = p.get_current_loss();
            REQUIRE(last[k] < 0.5 * first);
            const std::vector<double> hx = x.to_host();
            for (int64_t l = 0; l < n; ++l)
                if (hbc[(size_t)l])
                    for (int d = 0; d < 3; ++d) REQUIRE(hx[3 * l + d] == bent[3 * l + d]);
        }
        REQUIRE(std::fabs(last[0] - last[1]) <= 1e-8 * std::fabs(last[0]) + 1e-14);
    }

    // batch: two meshes, one launch
    std::vector<int32_t> t1;
    for (const auto& f : fv)
        for (uint32_t v : f) t1.push_back((int32_t)v);
    std::vector<std::pair<std::vector<int32_t>, int64_t>> meshes = {{t1, (int64_t)nv},
                                                                    {gfv, (int64_t)gxyz.size()}};
    MeshBatch batch(meshes);
    std::vector<double> bx;
    for (const auto& p : xyz) bx.insert(bx.end(), p.begin(), p.end());
    bx.insert(bx.end(), gx.begin(), gx.end());
    DenseMatrix<double> dbx((int64_t)bx.size() / 3, 3);
    dbx.from_host(bx);
    batch.mcf(dbx, dt, 2, 1e-6);
    std::vector<int32_t> iters, conv;
    batch.stats(iters, conv);
    REQUIRE(iters.size() == 2 && conv[0] && conv[1]);
    return 0;
}

int main(int argc, char** argv)
{
    const bool gpu = argc > 1 && std::strcmp(argv[1], "gpu") == 0;
    try {
        const char* dir = argc > 2 ? argv[2] : nullptr;
        const int   rc  = gpu ? gpu_checks(dir) : host_checks(dir);
        if (rc) return rc;
    } catch (const Error& e) {
        std::printf("FAILED: exception %s\n", e.what());
        return 1;
    }
    std::printf("OK\n");
    return 0;
}
