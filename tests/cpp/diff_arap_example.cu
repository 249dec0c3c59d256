// DiffARAP (apps/DiffARAP/diff_arap.cu:14-229, apps/DiffARAP/arap_kernels.h)
// written on the facade the way the reference application is written:
//   - cotangent edge weights from for_each<Op::EVDiamond> (the reference's
//     calc_edge_weights_mat), one per edge, clamped at zero;
//   - per-vertex rotations from for_each<Op::VE> (calculate_rotation_matrix):
//     S_i = sum_j w_ij (p_i - p_j)(p'_i - p'_j)^T = U Sigma V^T, R_i = V U^T
//     with the reflection removed;
//   - the energy as a per-edge term, add_term<Op::EV, ProjectHess = true>:
//     E = sum_e w_e |(p'_i - p'_j) - R_i (p_i - p_j)|^2, i, j the edge's
//     vertices in EV order;
//   - Newton with the constrained vertices held (apply_bc), PCG on the
//     assembled Hessian (the reference uses a Cholesky solver), Armijo line
//     search, stopping on the Newton decrement.
// The mesh is a torus: vertices with x < -1 are fixed, those with x > 1.1
// are moved by the user displacement each step.
//   diff_arap_example: prints the checks' results and "OK" (exit 0), or the
//   failing check (exit 1).
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "rxg/diff.cuh"
#include "rxg/rxmesh.hpp"

using namespace rxg;

#define REQUIRE(c)                                               \
    do {                                                         \
        if (!(c)) {                                              \
            std::printf("FAILED: %s (line %d)\n", #c, __LINE__); \
            return 1;                                            \
        }                                                        \
    } while (0)

// R = V U^T for S = U Sigma V^T (3x3, row-major), without reflection: the
// eigenvectors V of S^T S by cyclic Jacobi rotations, u_k = S v_k / sigma_k
// for the two largest singular values, u_3 = u_1 x u_2, and when det V < 0
// the column of the smallest singular value flipped.
__device__ void arap_rotation(const double S[9], float R[9])
{
    double A[9], V[9];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            double s = 0;
            for (int k = 0; k < 3; ++k) s += S[3 * k + r] * S[3 * k + c];
            A[3 * r + c] = s;
        }
    term_jacobi<double, 3>(A, V);
    int o[3] = {0, 1, 2};  // eigenvalues in decreasing order
    for (int i = 0; i < 3; ++i)
        for (int j = i + 1; j < 3; ++j)
            if (A[4 * o[j]] > A[4 * o[i]]) {
                const int t = o[i];
                o[i]        = o[j];
                o[j]        = t;
            }
    double v[3][3], u[3][3];
    for (int k = 0; k < 3; ++k)
        for (int r = 0; r < 3; ++r) v[k][r] = V[3 * r + o[k]];
    for (int k = 0; k < 2; ++k) {
        double n = 0;
        for (int r = 0; r < 3; ++r) {
            u[k][r] = S[3 * r] * v[k][0] + S[3 * r + 1] * v[k][1] + S[3 * r + 2] * v[k][2];
            n += u[k][r] * u[k][r];
        }
        n = ::sqrt(n);
        if (n < 1e-30) {  // rank-deficient: any unit vector orthogonal to u_0
            const double* a = u[0];
            const double  e[3] = {::fabs(a[0]) < 0.9 ? 1.0 : 0.0, ::fabs(a[0]) < 0.9 ? 0.0 : 1.0, 0.0};
            u[k][0] = a[1] * e[2] - a[2] * e[1];
            u[k][1] = a[2] * e[0] - a[0] * e[2];
            u[k][2] = a[0] * e[1] - a[1] * e[0];
            n       = ::sqrt(u[k][0] * u[k][0] + u[k][1] * u[k][1] + u[k][2] * u[k][2]);
        }
        for (int r = 0; r < 3; ++r) u[k][r] /= n;
    }
    u[2][0] = u[0][1] * u[1][2] - u[0][2] * u[1][1];
    u[2][1] = u[0][2] * u[1][0] - u[0][0] * u[1][2];
    u[2][2] = u[0][0] * u[1][1] - u[0][1] * u[1][0];
    const double detv = v[0][0] * (v[1][1] * v[2][2] - v[1][2] * v[2][1]) -
                        v[0][1] * (v[1][0] * v[2][2] - v[1][2] * v[2][0]) +
                        v[0][2] * (v[1][0] * v[2][1] - v[1][1] * v[2][0]);
    if (detv < 0)
        for (int r = 0; r < 3; ++r) u[2][r] = -u[2][r];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c)
            R[3 * r + c] = (float)(v[0][r] * u[0][c] + v[1][r] * u[1][c] + v[2][r] * u[2][c]);
}

static double cot_at(const double* a, const double* b, const double* q)
{
    const double e1[3] = {a[0] - q[0], a[1] - q[1], a[2] - q[2]}, e2[3] = {b[0] - q[0], b[1] - q[1], b[2] - q[2]};
    const double cr[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
    return (e1[0] * e2[0] + e1[1] * e2[1] + e1[2] * e2[2]) /
           std::sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
}

int main()
{
    try {
        // torus, 64 x 24 vertices, major radius 1, minor 0.35
        const int                          nu = 64, nw = 24;
        std::vector<std::vector<uint32_t>> fv;
        std::vector<std::vector<double>>   xyz;
        for (int i = 0; i < nu; ++i)
            for (int j = 0; j < nw; ++j) {
                const double u = 2 * M_PI * i / nu, w = 2 * M_PI * j / nw;
                xyz.push_back({(1.0 + 0.35 * std::cos(w)) * std::cos(u), (1.0 + 0.35 * std::cos(w)) * std::sin(u),
                               0.35 * std::sin(w)});
                const uint32_t a = i * nw + j, b = ((i + 1) % nu) * nw + j, c = ((i + 1) % nu) * nw + (j + 1) % nw,
                               d = i * nw + (j + 1) % nw;
                fv.push_back({a, b, c});
                fv.push_back({a, c, d});
            }
        RXMeshStatic   rx(fv, "", 128);
        const int64_t  nv = rx.get_num_vertices(), ne = rx.get_num_edges();
        const std::vector<int32_t> l2i = rx.linear_to_input(RXG_ELEM_VERTEX);
        auto                       Pa  = rx.add_vertex_attribute(xyz, "P");  // FP64 rest positions
        auto                       Pf  = rx.add_vertex_attribute<float>("Pf", 3);
        auto                       Ca  = rx.add_vertex_attribute<int32_t>("constraints", 1);
        auto                       Wa  = rx.add_edge_attribute<float>("weights", 1);
        auto                       Ra  = rx.add_vertex_attribute<float>("rotations", 9);
        VertexAttribute<double>    P   = *Pa;
        VertexAttribute<float>     Pr  = *Pf, R = *Ra;
        VertexAttribute<int32_t>   C   = *Ca;
        EdgeAttribute<float>       W   = *Wa;
        Wa->reset(0.f, LOCATION_ALL);
        DeviceArray<int8_t> bc((size_t)nv);
        int8_t*             bcp = bc.data();

        // constraints: 2 fixed, 1 user-displaced, 0 free
        rx.for_each_vertex(DEVICE, [=] __device__(const VertexHandle& vh) {
            for (int c = 0; c < 3; ++c) Pr(vh, c) = (float)P(vh, c);
            const double x = P(vh, 0);
            C(vh)          = x < -1.0 ? 2 : (x > 1.1 ? 1 : 0);
            bcp[vh.linear_id()] = C(vh) != 0;
        });

        // cotangent weights (calc_edge_weights_mat): the edge p-r, q and s opposite
        rx.for_each<Op::EVDiamond, 256>([=] __device__(const EdgeHandle& eh, const VertexIterator& it) {
            const VertexHandle p = it[0], q = it[1], r = it[2], s = it[3];
            if (!p.is_valid() || !q.is_valid() || !r.is_valid() || !s.is_valid()) return;
            float w = 0;
            for (const VertexHandle o : {q, s}) {
                float e1[3], e2[3];
                for (int c = 0; c < 3; ++c) {
                    e1[c] = Pr(p, c) - Pr(o, c);
                    e2[c] = Pr(r, c) - Pr(o, c);
                }
                const float cx = e1[1] * e2[2] - e1[2] * e2[1], cy = e1[2] * e2[0] - e1[0] * e2[2],
                            cz = e1[0] * e2[1] - e1[1] * e2[0];
                w += (e1[0] * e2[0] + e1[1] * e2[1] + e1[2] * e2[2]) / sqrtf(cx * cx + cy * cy + cz * cz);
            }
            W(eh) = fmaxf(0.f, 0.5f * w);
        });
        Wa->move(DEVICE, HOST);
        // the weights against the same formula on the host, from the EVD query
        {
            const std::vector<int32_t> evd = rx.query(Op::EVDiamond).values.to_host();
            std::vector<double>        hp(3 * nv);
            for (int64_t l = 0; l < nv; ++l)
                for (int c = 0; c < 3; ++c) hp[3 * l + c] = xyz[l2i[l]][c];
            double maxd = 0, maxw = 0;
            for (int64_t e = 0; e < ne; ++e) {
                const int32_t* d = &evd[4 * e];
                const double   w = std::max(0.0, 0.5 * (cot_at(&hp[3 * d[0]], &hp[3 * d[2]], &hp[3 * d[1]]) +
                                                      cot_at(&hp[3 * d[0]], &hp[3 * d[2]], &hp[3 * d[3]])));
                maxd = std::max(maxd, std::fabs(w - (double)Wa->data(HOST)[e]));
                maxw = std::max(maxw, w);
            }
            std::printf("edge weights: max |w - host| = %.3g (max w %.3g)\n", maxd, maxw);
            REQUIRE(maxd <= 1e-5 * maxw);
        }

        const QueryResult          evq  = rx.query(Op::EV);
        const std::vector<int32_t> ev_h = evq.values.to_host();
        const int32_t*             ev   = evq.values.data();

        // P' (the optimisation variable) starts at P
        DenseMatrix<float> X(nv, 3);
        check_cuda(cudaMemcpy(X.data(), Pr.data(DEVICE), sizeof(float) * 3 * nv, cudaMemcpyDeviceToDevice),
                   "cudaMemcpy");
        float* xp = X.data();

        // rotations (calculate_rotation_matrix), over the vertex's edges
        auto rotate = [&]() {
            rx.for_each<Op::VE, 256>([=] __device__(const VertexHandle& vh, const Iterator<EdgeHandle>& it) {
                const int32_t i = vh.linear_id();
                double        S[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
                for (uint16_t k = 0; k < it.size(); ++k) {
                    const int32_t e = it[k].linear_id();
                    const int32_t j = ev[2 * e] == i ? ev[2 * e + 1] : ev[2 * e];
                    const double  w = W(it[k]);
                    for (int r = 0; r < 3; ++r)
                        for (int c = 0; c < 3; ++c)
                            S[3 * r + c] += w * (double)(Pr(vh, r) - Pr(VertexHandle(j), r)) *
                                            (double)(xp[3 * i + c] - xp[3 * j + c]);
                }
                float Ri[9];
                arap_rotation(S, Ri);
                for (int t = 0; t < 9; ++t) R(vh, t) = Ri[t];
            });
        };
        auto max_rot_err = [&](bool identity) {
            Ra->move(DEVICE, HOST);
            const float* r  = Ra->data(HOST);
            double       mx = 0;
            for (int64_t l = 0; l < nv; ++l) {
                const float* m = r + 9 * l;
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b) {
                        double d = 0;
                        for (int k = 0; k < 3; ++k) d += m[3 * k + a] * m[3 * k + b];
                        mx = std::max(mx, std::fabs(d - (a == b)));
                        if (identity) mx = std::max(mx, std::fabs((double)m[3 * a + b] - (a == b)));
                    }
                const double det = m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) +
                                   m[2] * (m[3] * m[7] - m[4] * m[6]);
                mx = std::max(mx, std::fabs(det - 1.0));
            }
            return mx;
        };
        rotate();
        const double e0 = max_rot_err(true);
        std::printf("undeformed: rotations within %.3g of I\n", e0);
        REQUIRE(e0 <= 1e-4);

        // the energy: add_term<Op::EV, ProjectHess = true>
        DiffScalarProblem<float, 3> problem(rx);
        const float*                rot = R.data(DEVICE);
        const float*                wts = W.data(DEVICE);
        const float*                pr  = Pr.data(DEVICE);
        problem.add_term<Op::EV, true>([=] __device__(int32_t e, const Scalar<float, 6, true>* v) {
            using S          = Scalar<float, 6, true>;
            const int32_t a  = ev[2 * e], b = ev[2 * e + 1];
            const float*  ri = rot + 9 * a;
            const float   d[3] = {pr[3 * a] - pr[3 * b], pr[3 * a + 1] - pr[3 * b + 1], pr[3 * a + 2] - pr[3 * b + 2]};
            S             E(0.f);
            for (int r = 0; r < 3; ++r) E += sqr(v[r] - v[3 + r] - (ri[3 * r] * d[0] + ri[3 * r + 1] * d[1] + ri[3 * r + 2] * d[2]));
            return E * wts[e];
        });
        NewtonSolver<float> newton(problem, X, NewtonSolver<float>::PCG, 4000, 0.f, 1e-6f);

        // host energy from the final state, for the check
        auto host_energy = [&]() {
            Ra->move(DEVICE, HOST);
            const std::vector<float> x = X.to_host();
            const float*             r = Ra->data(HOST);
            double                   E = 0;
            for (int64_t e = 0; e < ne; ++e) {
                const int32_t a = ev_h[2 * e], b = ev_h[2 * e + 1];
                double        s = 0;
                for (int i = 0; i < 3; ++i) {
                    double rd = 0;
                    for (int k = 0; k < 3; ++k)
                        rd += (double)r[9 * a + 3 * i + k] * ((double)(float)xyz[l2i[a]][k] - (double)(float)xyz[l2i[b]][k]);
                    const double t = (double)x[3 * a + i] - x[3 * b + i] - rd;
                    s += t * t;
                }
                E += (double)Wa->data(HOST)[e] * s;
            }
            return E;
        };

        const float disp[3] = {0.0f, 0.0f, 0.08f};
        double      prev    = 0;
        for (int step = 0; step < 4; ++step) {
            // the first two steps move the handles, the last two only iterate
            // local (rotations) and global (Newton) steps: the energy must not grow
            if (step < 2)
                rx.for_each_vertex(DEVICE, [=] __device__(const VertexHandle& vh) {
                    if (C(vh) == 1)
                        for (int c = 0; c < 3; ++c) xp[3 * vh.linear_id() + c] += disp[c];
                });
            rotate();
            problem.eval_terms(X);
            const double e_start = problem.get_current_loss();
            int          it      = 0;
            double       dec     = 0;
            for (; it < 30; ++it) {
                problem.eval_terms(X);
                newton.apply_bc(bc);
                newton.compute_direction();
                dec = 0.5 * (double)problem.grad.dot(newton.dir);
                if (dec < 1e-9) break;
                newton.line_search();
            }
            problem.eval_terms(X);
            const double e_end = problem.get_current_loss(), eh = host_energy();
            const double rerr  = max_rot_err(false);
            std::printf("step %d: energy %.6g -> %.6g (host %.6g), %d Newton iterations, decrement %.3g, "
                        "rotation error %.3g\n",
                        step, e_start, e_end, eh, it, dec, rerr);
            REQUIRE(it < 30);
            REQUIRE(e_end <= e_start * (1 + 1e-5) + 1e-9);
            REQUIRE(std::fabs(e_end - eh) <= 1e-3 * std::max(eh, 1e-6));
            REQUIRE(rerr <= 1e-4);
            if (step >= 2) REQUIRE(e_end <= prev * (1 + 1e-4) + 1e-9);
            prev = e_end;
        }
        // the constrained vertices: fixed ones unmoved, handles moved by 2 displacements
        {
            const std::vector<float> x = X.to_host();
            Ca->move(DEVICE, HOST);
            int    nfixed = 0, nhandle = 0;
            double mx     = 0;
            for (int64_t l = 0; l < nv; ++l) {
                const int c = Ca->data(HOST)[l];
                if (!c) continue;
                (c == 2 ? nfixed : nhandle)++;
                for (int k = 0; k < 3; ++k)
                    mx = std::max(mx, std::fabs((double)x[3 * l + k] -
                                                ((double)(float)xyz[l2i[l]][k] + (c == 1 ? 2.0 * disp[k] : 0.0))));
            }
            std::printf("constraints: %d fixed, %d moved, max deviation %.3g\n", nfixed, nhandle, mx);
            REQUIRE(nfixed > 0 && nhandle > 0);
            REQUIRE(mx <= 1e-6);
        }
    } catch (const std::exception& e) {
        std::printf("FAILED: %s\n", e.what());
        return 1;
    }
    std::printf("OK\n");
    return 0;
}
