// Energies written by the application (include/rxg/diff.cuh), the way an
// RXMesh application writes DiffScalarProblem::add_term<Op::FV>(lambda):
//   1. Param's symmetric Dirichlet energy as a __device__ lambda over the
//      forward-mode Scalar (D = 2), against the library's built-in term
//      (rxg_symdir_eval): energy, gradient and 2x2-block Hessian;
//   2. a spring energy sum_{edges (i,j) of f} k/2 |x_i - x_j|^2 (D = 3),
//      a quadratic, so its gradient must equal H x;
//   3. both summed in one problem (terms accumulate);
//   4. the spring energy per edge, add_term<Op::EV> (D = 3): gradient and
//      Hessian against the host sums over EV, and an edge term summed with
//      a face term;
//   5. Diff.SmoothingNewton (tests/RXMesh_test/test_grad.h:14-105): the
//      edge term |x_0 - x_1|^2 in FP32 minimised by Newton steps, which
//      must bring every vertex to one position;
//   6. Diff.WhileLoop (tests/RXMesh_test/test_grad.h:107-211): a vertex
//      term, add_term<Op::V> with D = 1, computing sqrt(a) with a Newton
//      loop inside the lambda; its gradient must be 1 / (2 sqrt(a));
//   7. NeoHookean's per-face cloth energy (apps/NeoHookean/
//      neo_hookean_energy.h:25-69): zero with zero gradient at rest, the
//      host's value when deformed, gradient and Hessian against central
//      differences, unchanged by a rigid motion;
//   8. the per-face ARAP energy written with the forward-mode Scalar
//      (E = A (s - 2 sqrt(s + 2 |j1 x j2|) + 2), the DiffScalar way) against
//      the library's analytic ARAP term: energy, gradient and Hessian.
//   term_example <out_dir>: writes the spring gradient, positions and the
//   numbering for the test, prints "OK" and exits 0, or the failing check.
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

template <typename T>
static void dump(const std::string& path, const std::vector<T>& v)
{
    std::FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) throw Error(RXG_ERR_INVALID, "cannot write " + path);
    std::fwrite(v.data(), sizeof(T), v.size(), f);
    std::fclose(f);
}

// NeoHookean energy density of one face (apps/NeoHookean/
// neo_hookean_energy.h:25-69) for T a Scalar or double: with e0 = x2 - x0,
// e1 = x1 - x0, n their unit normal, F = [e0 e1 n] ib (ib the inverse of the
// same matrix at rest), J = det F,
//   E = vol h^2 (mu/2 (tr(F^T F) - 3) - mu ln J + lam/2 (ln J)^2).
struct NeoHookeanParams
{
    double mu, lam, h2;
};
template <typename S>
__host__ __device__ S neo_hookean(const S* v, const double* ib, double vol, NeoHookeanParams q)
{
    S e0[3], e1[3], n[3];
    for (int c = 0; c < 3; ++c) {
        e0[c] = v[6 + c] - v[c];
        e1[c] = v[3 + c] - v[c];
    }
    n[0]       = e0[1] * e1[2] - e0[2] * e1[1];
    n[1]       = e0[2] * e1[0] - e0[0] * e1[2];
    n[2]       = e0[0] * e1[1] - e0[1] * e1[0];
    const S nn = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    for (int c = 0; c < 3; ++c) n[c] = n[c] / nn;
    S F[9];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) F[3 * r + c] = e0[r] * ib[c] + e1[r] * ib[3 + c] + n[r] * ib[6 + c];
    const S J   = F[0] * (F[4] * F[8] - F[5] * F[7]) - F[1] * (F[3] * F[8] - F[5] * F[6]) +
                F[2] * (F[3] * F[7] - F[4] * F[6]);
    const S lnJ = log(J);
    S       tr  = F[0] * F[0];
    for (int i = 1; i < 9; ++i) tr = tr + F[i] * F[i];
    const S psi = (tr - 3.0) * (0.5 * q.mu) - lnJ * q.mu + lnJ * lnJ * (0.5 * q.lam);
    return psi * (vol * q.h2);
}

static double max_abs_diff(const std::vector<double>& a, const std::vector<double>& b, double* scale)
{
    double d = 0, s = 0;
    for (size_t i = 0; i < a.size(); ++i) {
        d = std::max(d, std::fabs(a[i] - b[i]));
        s = std::max(s, std::fabs(b[i]));
    }
    *scale = s;
    return d;
}

int main(int argc, char** argv)
{
    if (argc < 2) {
        std::printf("usage: term_example <out_dir>\n");
        return 2;
    }
    try {
        const std::string dir = argv[1];
        // a 14 x 14 grid bent out of its plane (rest), uv = the flat grid
        const int                          n = 14;
        std::vector<std::vector<uint32_t>> fv;
        std::vector<std::vector<double>>   rest, uv;
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                const double u = j / double(n - 1), v = i / double(n - 1);
                rest.push_back({u, v, 0.25 * std::sin(2.0 * u) * std::cos(1.5 * v)});
                uv.push_back({1.2 * u + 0.01 * std::sin(37.0 * i + j), 0.9 * v + 0.01 * std::cos(11.0 * j + i)});
            }
        for (int i = 0; i + 1 < n; ++i)
            for (int j = 0; j + 1 < n; ++j) {
                const uint32_t a = i * n + j, b = a + 1, c = a + n + 1, d = a + n;
                fv.push_back({a, b, c});
                fv.push_back({a, c, d});
            }
        RXMeshStatic   rx(fv, "", 64);
        const uint32_t nv = rx.get_num_vertices(), nf = rx.get_num_faces();
        const std::vector<int32_t> l2i = rx.linear_to_input(RXG_ELEM_VERTEX);
        std::vector<double>        hr(3 * nv), hu(2 * nv);
        for (uint32_t l = 0; l < nv; ++l) {
            for (int c = 0; c < 3; ++c) hr[3 * l + c] = rest[l2i[l]][c];
            for (int c = 0; c < 2; ++c) hu[2 * l + c] = uv[l2i[l]][c];
        }
        DenseMatrix<double> R(nv, 3), U(nv, 2);
        R.from_host(hr);
        U.from_host(hu);
        DeviceArray<double> minv(4 * (size_t)nf);
        check(rxg_arap_rest(rx.handle(), R.data(), RXG_F64, minv.data(), nullptr));

        // 1. symmetric Dirichlet as the application's own lambda
        DiffScalarProblem<double, 2> sd(rx);
        const double*                mi = minv.data();
        sd.add_term<Op::FV, false>([mi] __device__(int32_t f, const Scalar<double, 6, true>* v) {
            using S          = Scalar<double, 6, true>;
            const Vec2<S> a{v[0], v[1]}, b{v[2], v[3]}, c{v[4], v[5]};
            const Mat2<S> M = col_mat(b - a, c - a);
            if (det(M).val <= 0.0) return S(DBL_MAX);
            const Mat2<double> r{mi[4 * f], mi[4 * f + 1], mi[4 * f + 2], mi[4 * f + 3]};
            const double       A = 0.5 / (r.a * r.d - r.b * r.c);
            const Mat2<S>      J = mul(M, r);
            return (squared_norm(J) + squared_norm(inverse(J))) * A;
        });
        sd.eval_terms(U);
        // the built-in term on the same input
        DenseMatrix<double>       g_ref(nv, 2);
        BlockSparseMatrix<double> H_ref(sd.hess->rows(), sd.hess->non_zero_blocks(), 2);
        rxg_bcsr                  hb = H_ref.bcsr();
        double                    e_ref = 0;
        check(rxg_symdir_eval(rx.handle(), RXG_F64, U.data(), minv.data(), 0, &e_ref, nullptr,
                              g_ref.data(), &hb, nullptr));
        REQUIRE(std::fabs(sd.get_current_loss() - e_ref) <= 1e-12 * e_ref);
        double sc = 0;
        REQUIRE(max_abs_diff(sd.grad.to_host(), g_ref.to_host(), &sc) <= 1e-12 * sc);
        REQUIRE(max_abs_diff(sd.hess->values().to_host(), H_ref.values().to_host(), &sc) <= 1e-12 * sc);
        // projected variant through the template flag: positive diagonal blocks
        DiffScalarProblem<double, 2> sdp(rx);
        sdp.add_term<Op::FV, true>([mi] __device__(int32_t f, const Scalar<double, 6, true>* v) {
            using S          = Scalar<double, 6, true>;
            const Vec2<S> a{v[0], v[1]}, b{v[2], v[3]}, c{v[4], v[5]};
            const Mat2<double> r{mi[4 * f], mi[4 * f + 1], mi[4 * f + 2], mi[4 * f + 3]};
            const Mat2<S>      J = mul(col_mat(b - a, c - a), r);
            return (squared_norm(J) + squared_norm(inverse(J))) * (0.5 / (r.a * r.d - r.b * r.c));
        });
        sdp.eval_terms(U);
        REQUIRE(std::fabs(sdp.get_current_loss() - e_ref) <= 1e-12 * e_ref);
        // Newton on it with 2x2 blocks (NewtonSolver<double, 2>): a stretched
        // uv relaxes, the energy falling at every step
        {
            std::vector<double> hs = hu;
            for (uint32_t l = 0; l < nv; ++l) {
                hs[2 * l] *= 1.3;
                hs[2 * l + 1] *= 0.8;
            }
            DenseMatrix<double> Us(nv, 2);
            Us.from_host(hs);
            NewtonSolver<double, 2> nt(sdp, Us, NewtonSolver<double, 2>::PCG, 2000, 0.0, 1e-12);
            sdp.eval_terms(Us);
            const double e0 = sdp.get_current_loss();
            double       ep = e0;
            for (int it = 0; it < 4; ++it) {
                sdp.eval_terms(Us);
                nt.compute_direction();
                REQUIRE(nt.line_search());
                sdp.eval_terms(Us);
                REQUIRE(sdp.get_current_loss() <= ep * (1 + 1e-12));
                ep = sdp.get_current_loss();
            }
            std::printf("symmetric Dirichlet Newton (2x2 blocks): %.6g -> %.6g\n", e0, ep);
            REQUIRE(ep < 0.9 * e0);
        }

        // 2. spring energy on the 3-D rest positions (quadratic: grad = H x)
        const double                 k = 2.5;
        DiffScalarProblem<double, 3> sp(rx);
        sp.add_term<Op::FV>([k] __device__(int32_t, const Scalar<double, 9, true>* v) {
            Scalar<double, 9, true> e(0.0);
            for (int i = 0; i < 3; ++i) {
                const int j = (i + 1) % 3;
                for (int c = 0; c < 3; ++c) e += sqr(v[3 * i + c] - v[3 * j + c]) * (0.5 * k);
            }
            return e;
        });
        sp.eval_terms(R);
        const std::vector<double> g  = sp.grad.to_host();
        const std::vector<double> hv = sp.hess->values().to_host();
        const std::vector<int32_t> rp = sp.hess->row_ptr().to_host(), col = sp.hess->col_idx().to_host();
        std::vector<double>        Hx(3 * nv, 0.0);
        for (uint32_t i = 0; i < nv; ++i)
            for (int32_t t = rp[i]; t < rp[i + 1]; ++t)
                for (int a = 0; a < 3; ++a)
                    for (int c = 0; c < 3; ++c) Hx[3 * i + a] += hv[9 * t + 3 * a + c] * hr[3 * col[t] + c];
        REQUIRE(max_abs_diff(Hx, g, &sc) <= 1e-12 * sc);
        dump(dir + "/spring_grad.bin", g);
        dump(dir + "/rest.bin", hr);
        dump(dir + "/l2i.bin", l2i);
        std::vector<int32_t> fl;
        for (const auto& f : fv)
            for (uint32_t v : f) fl.push_back((int32_t)v);
        dump(dir + "/fv.bin", fl);

        // 3. two terms in one problem add up
        DiffScalarProblem<double, 3> both(rx);
        for (int t = 0; t < 2; ++t)
            both.add_term<Op::FV>([k] __device__(int32_t, const Scalar<double, 9, true>* v) {
                Scalar<double, 9, true> e(0.0);
                for (int i = 0; i < 3; ++i)
                    for (int c = 0; c < 3; ++c) e += sqr(v[3 * i + c] - v[3 * ((i + 1) % 3) + c]) * (0.5 * k);
                return e;
            });
        both.eval_terms(R);
        REQUIRE(std::fabs(both.get_current_loss() - 2.0 * sp.get_current_loss()) <= 1e-12 * sp.get_current_loss());
        std::vector<double> g2 = both.grad.to_host();
        for (double& x : g2) x *= 0.5;
        REQUIRE(max_abs_diff(g2, g, &sc) <= 1e-12 * sc);

        // 4. spring energy per edge (each edge once)
        DiffScalarProblem<double, 3> es(rx);
        es.add_term<Op::EV>([k] __device__(int32_t, const Scalar<double, 6, true>* v) {
            Scalar<double, 6, true> e(0.0);
            for (int c = 0; c < 3; ++c) e += sqr(v[c] - v[3 + c]) * (0.5 * k);
            return e;
        });
        es.eval_terms(R);
        {
            const std::vector<int32_t> ev = rx.query(Op::EV).values.to_host();
            const size_t               ne = ev.size() / 2;
            std::vector<double>        want(3 * nv, 0.0);
            double                     ew = 0.0;
            for (size_t e = 0; e < ne; ++e) {
                const int32_t a = ev[2 * e], b = ev[2 * e + 1];
                for (int c = 0; c < 3; ++c) {
                    const double d = hr[3 * a + c] - hr[3 * b + c];
                    ew += 0.5 * k * d * d;
                    want[3 * a + c] += k * d;
                    want[3 * b + c] -= k * d;
                }
            }
            REQUIRE(std::fabs(es.get_current_loss() - ew) <= 1e-12 * ew);
            const std::vector<double> ge = es.grad.to_host();
            REQUIRE(max_abs_diff(ge, want, &sc) <= 1e-12 * sc);
            // Hessian: k (degree) I on the diagonal blocks, -k I per ring block
            const std::vector<double>  he  = es.hess->values().to_host();
            const std::vector<int32_t> erp = es.hess->row_ptr().to_host();
            for (uint32_t i = 0; i < nv; ++i) {
                const double deg = erp[i + 1] - erp[i] - 1;
                for (int32_t t = erp[i]; t < erp[i + 1]; ++t)
                    for (int a = 0; a < 3; ++a)
                        for (int c = 0; c < 3; ++c) {
                            const double w = a != c ? 0.0 : (t == erp[i] ? k * deg : -k);
                            REQUIRE(std::fabs(he[9 * t + 3 * a + c] - w) <= 1e-12 * k * 8);
                        }
            }
            // a face term and an edge term in one problem
            DiffScalarProblem<double, 3> fe(rx);
            fe.add_term<Op::FV>([k] __device__(int32_t, const Scalar<double, 9, true>* v) {
                Scalar<double, 9, true> e(0.0);
                for (int i = 0; i < 3; ++i)
                    for (int c = 0; c < 3; ++c) e += sqr(v[3 * i + c] - v[3 * ((i + 1) % 3) + c]) * (0.5 * k);
                return e;
            });
            fe.add_term<Op::EV>([k] __device__(int32_t, const Scalar<double, 6, true>* v) {
                Scalar<double, 6, true> e(0.0);
                for (int c = 0; c < 3; ++c) e += sqr(v[c] - v[3 + c]) * (0.5 * k);
                return e;
            });
            fe.eval_terms(R);
            std::vector<double> gs = g;
            for (size_t i = 0; i < gs.size(); ++i) gs[i] += ge[i];
            REQUIRE(max_abs_diff(fe.grad.to_host(), gs, &sc) <= 1e-12 * sc);
            const std::vector<double> hfe = fe.hess->values().to_host();
            std::vector<double>       hs  = hv;
            for (size_t i = 0; i < hs.size(); ++i) hs[i] += he[i];
            REQUIRE(max_abs_diff(hfe, hs, &sc) <= 1e-12 * sc);
        }

        // 5. Diff.SmoothingNewton: sum over edges |x_0 - x_1|^2, FP32
        {
            DiffScalarProblem<float, 3> sm(rx);
            sm.add_term<Op::EV>([] __device__(int32_t, const Scalar<float, 6, true>* v) {
                Scalar<float, 6, true> d(0.0f);
                for (int c = 0; c < 3; ++c) d += sqr(v[c] - v[3 + c]);
                return d;
            });
            std::vector<float> xf(hr.begin(), hr.end());
            DenseMatrix<float> X(nv, 3);
            X.from_host(xf);
            NewtonSolver<float> newton(sm, X, NewtonSolver<float>::PCG, 2000, 0.0f, 1e-6f);
            int                 it = 0;
            for (; it < 100; ++it) {
                sm.eval_terms(X);
                newton.compute_direction();
                if (0.5f * sm.grad.dot(newton.dir) < 1e-2f) break;
                newton.line_search();
            }
            REQUIRE(it < 100);
            const std::vector<float> xs = X.to_host();
            for (uint32_t i = 0; i < nv; ++i)
                for (int c = 0; c < 3; ++c) REQUIRE(std::fabs(xs[3 * i + c] - xs[c]) <= 1e-3f);
            std::printf("smoothing newton: %d iterations, energy %g\n", it, (double)sm.get_current_loss());
        }

        // 6. Diff.WhileLoop: a = x^2 per vertex, the term is sqrt(a) by a
        // Newton loop (bounded here: at most 64 rounds), its value also
        // written to root[] from inside the lambda
        {
            const float         tol = FLT_EPSILON;
            std::vector<float>  ha(nv), px(nv);
            for (uint32_t l = 0; l < nv; ++l) {
                px[l] = (float)(rest[l2i[l]][0] - 0.37);
                ha[l] = px[l] * px[l];
            }
            DenseMatrix<float>           A(nv, 1);
            A.from_host(ha);
            DeviceArray<float>           root(nv);
            float*                       rt = root.data();
            DiffScalarProblem<float, 1>  wl(rx, false);
            wl.add_term<Op::V>([tol, rt] __device__(int32_t vid, const Scalar<float, 1, true>* v) {
                using S = Scalar<float, 1, true>;
                const S a = v[0];
                S       y = a;
                if (a.val > tol) {
                    int rounds = 0;
                    do {
                        y = (y + a / y) * 0.5f;
                    } while (fabsf(y.val * y.val - a.val) > tol && ++rounds < 64);
                } else {
                    y = S(0.0f);
                }
                rt[vid] = y.val;
                return y;
            });
            wl.eval_terms(A);
            const std::vector<float> r  = root.to_host();
            const std::vector<float> gw = wl.grad.to_host();
            int                      checked = 0;
            for (uint32_t l = 0; l < nv; ++l) {
                const float s = std::fabs(px[l]);
                if (s > 0.001f) {
                    REQUIRE(std::fabs(r[l] - s) <= 0.001f);
                    REQUIRE(std::fabs(gw[l] - 1.0f / (2.0f * s)) <= 0.001f);
                    ++checked;
                }
            }
            REQUIRE(checked > (int)nv / 2);
        }

        // 7. NeoHookean: rest = the bent grid R, rest frames on the host
        {
            const NeoHookeanParams q{2.0, 5.0, 1e-2};
            const std::vector<int32_t> fvl = rx.query(Op::FV).values.to_host();
            std::vector<double>        ib(9 * (size_t)nf), vol(nf);
            for (uint32_t f = 0; f < nf; ++f) {
                const double* x0 = &hr[3 * fvl[3 * f]];
                const double* x1 = &hr[3 * fvl[3 * f + 1]];
                const double* x2 = &hr[3 * fvl[3 * f + 2]];
                double        e0[3], e1[3], n[3];
                for (int c = 0; c < 3; ++c) {
                    e0[c] = x2[c] - x0[c];
                    e1[c] = x1[c] - x0[c];
                }
                n[0]            = e0[1] * e1[2] - e0[2] * e1[1];
                n[1]            = e0[2] * e1[0] - e0[0] * e1[2];
                n[2]            = e0[0] * e1[1] - e0[1] * e1[0];
                const double nn = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
                vol[f]          = 0.5 * nn;
                const double B[9] = {e0[0], e1[0], n[0] / nn, e0[1], e1[1], n[1] / nn, e0[2], e1[2], n[2] / nn};
                const double d    = B[0] * (B[4] * B[8] - B[5] * B[7]) - B[1] * (B[3] * B[8] - B[5] * B[6]) +
                                 B[2] * (B[3] * B[7] - B[4] * B[6]);
                double* o = &ib[9 * (size_t)f];  // the inverse: adjugate / det
                o[0]      = (B[4] * B[8] - B[5] * B[7]) / d;
                o[1]      = (B[2] * B[7] - B[1] * B[8]) / d;
                o[2]      = (B[1] * B[5] - B[2] * B[4]) / d;
                o[3]      = (B[5] * B[6] - B[3] * B[8]) / d;
                o[4]      = (B[0] * B[8] - B[2] * B[6]) / d;
                o[5]      = (B[2] * B[3] - B[0] * B[5]) / d;
                o[6]      = (B[3] * B[7] - B[4] * B[6]) / d;
                o[7]      = (B[1] * B[6] - B[0] * B[7]) / d;
                o[8]      = (B[0] * B[4] - B[1] * B[3]) / d;
            }
            DenseMatrix<double> IB(nf, 9), VOL(nf, 1);
            IB.from_host(ib);
            VOL.from_host(vol);
            const double* ibd = IB.data();
            const double* vd  = VOL.data();
            DiffScalarProblem<double, 3> nh(rx);
            nh.add_term<Op::FV>([ibd, vd, q] __device__(int32_t f, const Scalar<double, 9, true>* v) {
                return neo_hookean(v, ibd + 9 * f, vd[f], q);
            });
            // at rest: zero energy and gradient
            nh.eval_terms(R);
            REQUIRE(std::fabs(nh.get_current_loss()) <= 1e-12);
            const std::vector<double> g0 = nh.grad.to_host();
            double                    gm = 0;
            for (double x : g0) gm = std::max(gm, std::fabs(x));
            REQUIRE(gm <= 1e-10);
            // deformed: stretched, sheared and jittered
            std::vector<double> xd(3 * nv);
            for (uint32_t l = 0; l < nv; ++l) {
                const double* X = &hr[3 * l];
                xd[3 * l]       = 1.15 * X[0] + 0.1 * X[1] + 0.01 * std::sin(7.0 * l);
                xd[3 * l + 1]   = 0.92 * X[1] + 0.01 * std::cos(5.0 * l);
                xd[3 * l + 2]   = X[2] + 0.05 * X[0] * X[1];
            }
            auto host_energy = [&](const std::vector<double>& x) {
                double E = 0;
                for (uint32_t f = 0; f < nf; ++f) {
                    double v[9];
                    for (int k = 0; k < 3; ++k)
                        for (int c = 0; c < 3; ++c) v[3 * k + c] = x[3 * fvl[3 * f + k] + c];
                    E += neo_hookean<double>(v, &ib[9 * (size_t)f], vol[f], q);
                }
                return E;
            };
            DenseMatrix<double> XD(nv, 3);
            XD.from_host(xd);
            nh.eval_terms(XD);
            const double Ed = nh.get_current_loss(), Eh = host_energy(xd);
            std::printf("neo-hookean: E = %.12g (host %.12g)\n", Ed, Eh);
            REQUIRE(Ed > 0 && std::fabs(Ed - Eh) <= 1e-10 * Eh);
            const std::vector<double>  g   = nh.grad.to_host();
            const std::vector<double>  hv  = nh.hess->values().to_host();
            const std::vector<int32_t> rp  = nh.hess->row_ptr().to_host();
            const std::vector<int32_t> col = nh.hess->col_idx().to_host();
            // central differences along three directions
            for (int t = 0; t < 3; ++t) {
                std::vector<double> d(3 * nv), xp(xd), xm(xd);
                for (size_t i = 0; i < d.size(); ++i) d[i] = std::sin(1.7 * i + 3.1 * t);
                const double h = 1e-6;
                for (size_t i = 0; i < d.size(); ++i) {
                    xp[i] += h * d[i];
                    xm[i] -= h * d[i];
                }
                DenseMatrix<double> XP(nv, 3), XM(nv, 3);
                XP.from_host(xp);
                XM.from_host(xm);
                const double fd = (nh.eval_terms_passive(XP) - nh.eval_terms_passive(XM)) / (2 * h);
                double       gd = 0;
                for (size_t i = 0; i < d.size(); ++i) gd += g[i] * d[i];
                REQUIRE(std::fabs(fd - gd) <= 1e-6 * std::fabs(gd) + 1e-12);
                // H d against the difference of gradients
                nh.eval_terms(XP);
                const std::vector<double> gp = nh.grad.to_host();
                nh.eval_terms(XM);
                const std::vector<double> gmn = nh.grad.to_host();
                std::vector<double>       Hd(3 * nv, 0.0), dg(3 * nv);
                for (uint32_t i = 0; i < nv; ++i)
                    for (int32_t k = rp[i]; k < rp[i + 1]; ++k)
                        for (int a = 0; a < 3; ++a)
                            for (int c = 0; c < 3; ++c) Hd[3 * i + a] += hv[9 * k + 3 * a + c] * d[3 * col[k] + c];
                for (size_t i = 0; i < dg.size(); ++i) dg[i] = (gp[i] - gmn[i]) / (2 * h);
                double scale = 0;
                REQUIRE(max_abs_diff(Hd, dg, &scale) <= 1e-5 * scale);
            }
            // a rigid motion leaves the energy unchanged
            std::vector<double> xr(3 * nv);
            const double        ca = std::cos(0.7), sa = std::sin(0.7);
            for (uint32_t l = 0; l < nv; ++l) {
                const double* X = &xd[3 * l];
                xr[3 * l]       = ca * X[0] - sa * X[2] + 0.3;
                xr[3 * l + 1]   = X[1] - 1.0;
                xr[3 * l + 2]   = sa * X[0] + ca * X[2] + 2.0;
            }
            DenseMatrix<double> XR(nv, 3);
            XR.from_host(xr);
            REQUIRE(std::fabs(nh.eval_terms_passive(XR) - Ed) <= 1e-9 * Ed);
        }

        // 8. ARAP through the forward-mode Scalar against the analytic term
        {
            std::vector<double> xd(3 * nv);
            for (uint32_t l = 0; l < nv; ++l) {
                const double* X = &hr[3 * l];
                xd[3 * l]       = 1.12 * X[0] + 0.08 * X[1] + 0.02 * std::sin(5.0 * l);
                xd[3 * l + 1]   = 0.93 * X[1] + 0.02 * std::cos(3.0 * l);
                xd[3 * l + 2]   = X[2] + 0.1 * X[0] * X[1];
            }
            DenseMatrix<double> XD(nv, 3);
            XD.from_host(xd);
            DiffScalarProblem<double, 3> an(rx);
            an.add_arap_term(R);
            an.eval_terms(XD);
            DiffScalarProblem<double, 3> ad(rx);
            ad.add_term<Op::FV>([mi] __device__(int32_t f, const Scalar<double, 9, true>* v) {
                using S         = Scalar<double, 9, true>;
                const double* m = mi + 4 * f;  // the rest frame's inverse, row-major 2x2
                S             j1[3], j2[3];
                for (int c = 0; c < 3; ++c) {
                    const S e1 = v[3 + c] - v[c], e2 = v[6 + c] - v[c];
                    j1[c]      = e1 * m[0] + e2 * m[2];
                    j2[c]      = e1 * m[1] + e2 * m[3];
                }
                S sn(0.0);
                for (int c = 0; c < 3; ++c) sn += sqr(j1[c]) + sqr(j2[c]);
                const S w0 = j1[1] * j2[2] - j1[2] * j2[1], w1 = j1[2] * j2[0] - j1[0] * j2[2],
                        w2 = j1[0] * j2[1] - j1[1] * j2[0];
                const S      d = sqrt(sqr(w0) + sqr(w1) + sqr(w2));
                const double A = 0.5 / (m[0] * m[3] - m[1] * m[2]);
                return (sn - 2.0 * sqrt(sn + 2.0 * d) + 2.0) * A;
            });
            ad.eval_terms(XD);
            const double ea = an.get_current_loss(), eb = ad.get_current_loss();
            std::printf("arap: analytic %.15g, forward-mode %.15g\n", ea, eb);
            REQUIRE(ea > 0 && std::fabs(ea - eb) <= 1e-10 * ea);
            REQUIRE(max_abs_diff(ad.grad.to_host(), an.grad.to_host(), &sc) <= 1e-9 * sc);
            REQUIRE(max_abs_diff(ad.hess->values().to_host(), an.hess->values().to_host(), &sc) <= 1e-8 * sc);
        }
    } catch (const std::exception& e) {
        std::printf("FAILED: %s\n", e.what());
        return 1;
    }
    std::printf("OK\n");
    return 0;
}
