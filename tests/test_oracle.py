"""CPU checks that pin the oracle to the reference's own tests and code."""
import numpy as np
import pytest

from conftest import golden, kat_system as _kat_system, sorted_rows
from rxmesh_gb300 import meshgen


def brute_edges(fv):
    seen, ev = {}, []
    for f in fv:
        for k in range(3):
            a, b = int(f[k]), int(f[(k + 1) % 3])
            key = (max(a, b), min(a, b))
            if key not in seen:
                seen[key] = len(ev)
                ev.append((a, b))
    return np.array(ev, np.int32)


@pytest.mark.parametrize("name", ["sphere3", "cloth"])
def test_edge_numbering_matches_reference_rule(oracle, name):
    # rxmesh.cpp:565-600: first appearance over (face, (v0v1,v1v2,v2v0)), EV as encountered
    g = golden(name)
    ev, fe = oracle.edges(g["fv"])
    assert np.array_equal(ev, brute_edges(g["fv"]))
    for f in range(0, len(g["fv"]), 7):
        for k in range(3):
            a, b = g["fv"][f][k], g["fv"][f][(k + 1) % 3]
            assert set(ev[fe[f][k]]) == {a, b}


def test_vv_ve_vf_ground_truth_small(oracle):
    v, f = meshgen.icosphere(1)
    ev, _ = oracle.edges(f)
    nv = len(v)
    off, val = oracle.vv(nv, ev)
    want = [set() for _ in range(nv)]
    for a, b in ev:
        want[a].add(int(b)); want[b].add(int(a))
    assert sorted_rows(off, val) == [tuple(sorted(s)) for s in want]
    off, val = oracle.vv(nv, ev, want_edges=True)
    wante = [set() for _ in range(nv)]
    for e, (a, b) in enumerate(ev):
        wante[a].add(e); wante[b].add(e)
    assert sorted_rows(off, val) == [tuple(sorted(s)) for s in wante]
    off, val = oracle.vf(nv, f)
    wantf = [set() for _ in range(nv)]
    for i, t in enumerate(f):
        for x in t:
            wantf[x].add(i)
    assert sorted_rows(off, val) == [tuple(sorted(s)) for s in wantf]


def test_ef_fe_ff_ground_truth(oracle):
    """EF, FE and FF as the reference's verifier builds them
    (tests/RXMesh_test/rxmesh_test.h:290-330), on a closed and an open mesh."""
    for v, f in (meshgen.icosphere(2), meshgen.plane(7, 5)):
        ev, fe = oracle.edges(f)
        eoff, eval_ = oracle.ef(f)
        want_ef = [set() for _ in range(len(ev))]
        for i, t in enumerate(fe):
            for e in t:
                want_ef[e].add(i)
        assert sorted_rows(eoff, eval_) == [tuple(sorted(s)) for s in want_ef]
        foff, fval = oracle.ff(f)
        want_ff = [set() for _ in range(len(f))]
        for fs in want_ef:
            for a in fs:
                want_ff[a] |= fs - {a}
        assert sorted_rows(foff, fval) == [tuple(sorted(s)) for s in want_ff]
        # FE edge k joins corners k and k+1
        for i, t in enumerate(f):
            for k in range(3):
                assert set(ev[fe[i][k]]) == {t[k], t[(k + 1) % 3]}


def test_ev_diamond_reference_kat(oracle):
    """tests/RXMesh_test/test_ev_diamond.cu: on plane_5, every edge with four
    valid diamond vertices has tri_area(v0,v1,v2) + tri_area(v0,v2,v3) = 1."""
    g = golden("plane_5")
    x, f = g["xyz"], g["fv"]
    d = oracle.ev_diamond(f)
    ev, _ = oracle.edges(f)
    assert np.array_equal(d[:, 0], ev[:, 0]) and np.array_equal(d[:, 2], ev[:, 1])

    def area(a, b, c):
        return 0.5 * np.linalg.norm(np.cross(x[b] - x[a], x[c] - x[a]))

    full = (d >= 0).all(axis=1)
    assert full.sum() == 40  # the 40 interior edges of the 4 x 4 grid
    for r in d[full]:
        assert abs(area(r[0], r[1], r[2]) + area(r[0], r[2], r[3]) - 1.0) < 1e-5
    # slot 1 is opposite the edge in the face traversing v0 -> v1, slot 3 in the other
    for i, t in enumerate(f):
        for k in range(3):
            a, b, c = int(t[k]), int(t[(k + 1) % 3]), int(t[(k + 2) % 3])
            e = [j for j in range(len(ev)) if set(ev[j]) == {a, b}][0]
            assert d[e][1 if ev[e][0] == a else 3] == c


@pytest.mark.parametrize("name", ["sphere3", "torus", "cloth", "bunnyhead"])
def test_normals_match_reference_vertex_normal_ref(oracle, name):
    # fixtures hold the output of apps/VertexNormal/vertex_normal_ref.h itself
    g = golden(name)
    n = oracle.vertex_normals(g["fv"], g["xyz"], 0)
    ref = g["ref_normals_f64"]
    assert np.allclose(n, ref, rtol=1e-12, atol=1e-15)
    scale = np.linalg.norm(ref, axis=1).max()
    assert np.abs(n - g["ref_normals_f32"]).max() <= 1e-5 * scale


def test_normals_against_live_reference_build(oracle):
    # oracle/_ref is the reference's own routine compiled from its source (here only)
    if oracle.ref_lib() is None:
        pytest.skip("oracle/_ref not built (reference tree absent)")
    v, f = meshgen.icosphere(3)
    x = meshgen.radial_noise(v, 0.02, 3)
    ref = oracle.ref_vertex_normals(f, x, np.float64)
    assert np.allclose(oracle.vertex_normals(f, x, 0), ref, rtol=1e-12, atol=1e-15)


def test_oriented_ring_closed_and_open(oracle):
    for x, f in [meshgen.icosphere(2), meshgen.plane(6, 5)]:
        nv = len(x)
        off, ring, bnd = oracle.oriented_vv(nv, f)
        faces = {tuple(np.roll(t, -np.argmin(t))) for t in f.tolist()}

        def is_face(a, b, c):
            t = (a, b, c)
            return tuple(np.roll(t, -int(np.argmin(t)))) in faces

        ev, _ = oracle.edges(f)
        voff, vval = oracle.vv(nv, ev)
        for p in range(nv):
            r = ring[off[p]:off[p + 1]].tolist()
            assert sorted(r) == sorted(vval[voff[p]:voff[p + 1]].tolist())
            k = len(r)
            pairs = range(k) if not bnd[p] else range(k - 1)
            for i in pairs:
                assert is_face(p, r[i], r[(i + 1) % k])


def test_sparse_matrix_row_count_is_valence_plus_one(oracle):
    # tests/RXMesh_test/test_sparse_matrix.cu:111-173
    g = golden("bunnyhead")
    nv = len(g["xyz"])
    ev, _ = oracle.edges(g["fv"])
    voff, _ = oracle.vv(nv, ev)
    rp, col, val, B = oracle.mcf_system(g["fv"], g["xyz"], 0.01)
    assert np.array_equal(np.diff(rp), np.diff(voff) + 1)


@pytest.mark.parametrize("precond", [False, True])
def test_solver_kat(oracle, precond):
    # Solver.CG / Solver.PCG: sphere3, abs_tol 1e-7, 5000 iterations, |Ax-b| <= 1e-3
    rp, col, val, B, X0 = _kat_system(oracle, "sphere3")
    X, it, r0, r1, conv = oracle.cg(rp, col, val, B, X0, 5000, 1e-7, 0.0, precond)
    assert conv and it < 5000
    assert np.abs(oracle.spmm(rp, col, val, X) - B).max() <= 1e-3


def test_mcf_system_closed_symmetric_and_spd(oracle):
    import scipy.sparse as sp
    v, f = meshgen.icosphere(3)
    x = meshgen.radial_noise(v, 0.02, 7)
    rp, col, val, B = oracle.mcf_system(f, x, 0.01)
    A = sp.csr_matrix((val, col, rp), shape=(len(x), len(x)))
    assert abs(A - A.T).max() < 1e-15 * abs(A).max() * 10
    # diagonal = 2*area + sum of |off-diagonals|; off-diagonals <= 0
    off = A - sp.diags(A.diagonal())
    assert off.max() <= 0
    area = np.linalg.norm(B, axis=1) / np.linalg.norm(x, axis=1)
    assert np.allclose(A.diagonal(), area - np.asarray(off.sum(1)).ravel(), rtol=1e-12)
    # total lumped area ~ reference's Voronoi scaling (2x area in non-obtuse cases)
    assert area.sum() > 0


def test_mcf_cg_matches_direct_solve(oracle):
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl
    v, f = meshgen.icosphere(4)
    x = meshgen.radial_noise(v, 0.02, 1)
    rp, col, val, B = oracle.mcf_system(f, x, 0.01)
    A = sp.csr_matrix((val, col, rp), shape=(len(x), len(x))).tocsc()
    Xd = spl.spsolve(A, B)
    X, it, r0, r1, conv = oracle.cg(rp, col, val, B, x, 10000, 0.0, 1e-24, True)
    assert conv
    assert np.abs(X - Xd).max() < 1e-9


def test_arap_face_derivatives(oracle):
    rng = np.random.default_rng(5)
    rest = rng.normal(size=(3, 3))
    minv, area = oracle.rest_frame(np.array([[0, 1, 2]], np.int32), rest)
    x = rest + 0.3 * rng.normal(size=(3, 3))
    E, g, H = oracle.arap_face(x.ravel(), minv[0], area[0])
    h = 1e-6
    for i in range(9):
        d = np.zeros(9); d[i] = h
        Ep = oracle.arap_face(x.ravel() + d, minv[0], area[0])[0]
        Em = oracle.arap_face(x.ravel() - d, minv[0], area[0])[0]
        assert abs((Ep - Em) / (2 * h) - g[i]) < 1e-6 * max(1, abs(g).max())
        gp = oracle.arap_face(x.ravel() + d, minv[0], area[0])[1]
        gm = oracle.arap_face(x.ravel() - d, minv[0], area[0])[1]
        assert np.abs((gp - gm) / (2 * h) - H[i]).max() < 1e-5 * max(1, abs(H).max())
    assert np.allclose(H, H.T, atol=1e-12)
    # rest shape has zero energy
    assert abs(oracle.arap_face(rest.ravel(), minv[0], area[0])[0]) < 1e-12


def test_arap_against_torch_autograd(oracle):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(11)
    x0, f = meshgen.plane(4, 4, 0.3)
    minv, area = oracle.rest_frame(f, x0)
    x = x0 + 0.05 * rng.normal(size=x0.shape)
    ev, _ = oracle.edges(f)
    voff, vval = oracle.vv(len(x), ev)
    rp = np.zeros(len(x) + 1, np.int64); rp[1:] = np.cumsum(np.diff(voff) + 1)
    col = np.empty(rp[-1], np.int32)
    for p in range(len(x)):
        col[rp[p]] = p; col[rp[p] + 1:rp[p + 1]] = vval[voff[p]:voff[p + 1]]
    E, fE, g, Hb = oracle.arap_assemble(f, x, minv, area, rp, col)

    def energy(X):
        a, b, c = X[f[:, 0]], X[f[:, 1]], X[f[:, 2]]
        M = torch.stack([b - a, c - a], -1)
        J = M @ torch.as_tensor(minv)
        s = (J * J).sum((-1, -2))
        d = torch.linalg.norm(torch.cross(J[..., 0], J[..., 1], dim=-1), dim=-1)
        return (torch.as_tensor(area) * (s - 2 * torch.sqrt(s + 2 * d) + 2)).sum()

    X = torch.tensor(x, requires_grad=True)
    Et = energy(X)
    gt, = torch.autograd.grad(Et, X)
    assert abs(Et.item() - E) < 1e-12 * max(1, abs(E))
    assert np.abs(gt.numpy() - g).max() < 1e-10
    Ht = torch.autograd.functional.hessian(energy, torch.tensor(x)).reshape(len(x) * 3, -1).numpy()
    for p in range(len(x)):
        for t in range(rp[p], rp[p + 1]):
            q = col[t]
            assert np.abs(Ht[3 * p:3 * p + 3, 3 * q:3 * q + 3] - Hb[t]).max() < 1e-9


def test_project_pd_matches_eigh(oracle):
    """project_positive_definite (diff/hessian_projection.h:21-95) restated
    with a cyclic Jacobi eigensolver, against numpy's eigh: unchanged when
    positive diagonally dominant with margin eps or already >= eps,
    otherwise eigenvalues below eps raised to eps."""
    rng = np.random.default_rng(0)
    eps = 1e-9
    for k in (3, 6, 9):
        for t in range(150):
            m = rng.normal(size=(k, k))
            h = m + m.T
            if t % 3 == 0:
                h += 4 * k * np.eye(k)
            got = oracle.project_pd(h, eps)
            w, v = np.linalg.eigh(h)
            dd = all(h[i, i] >= np.abs(h[i]).sum() - abs(h[i, i]) + eps for i in range(k))
            want = h if (dd or w.min() >= eps) else (v * np.maximum(w, eps)) @ v.T
            assert np.abs(got - want).max() < 1e-10 * max(1.0, np.abs(h).max())
            assert np.linalg.eigvalsh(got).min() >= eps * (1 - 1e-6) - 1e-12



def test_cotan_and_voronoi_match_reference_geometry_util(oracle):
    """The oracle's partial_voronoi_area and edge_cotan_weight against the
    reference's own geometry_util.cuh compiled from its source (outputs kept
    in tests/golden/geometry_util.npz by make_golden.py) on every branch:
    generic, obtuse at each corner, within 1e-9 .. 1e-3 rad of a right angle,
    clamped cotangents of slivers, and zero-area triangles."""
    g = golden("geometry_util")
    vor = oracle.partial_voronoi_area(g["P"], g["Q"], g["R"])
    cot = oracle.edge_cotan_weight(g["P"], g["Q"], g["R"], g["S"])
    # scale: the triangle's area for Voronoi areas (|cot| <= 19.1 for weights)
    area = 0.5 * np.linalg.norm(np.cross(g["Q"] - g["P"], g["R"] - g["P"]), axis=1)
    assert np.all(np.abs(vor - g["voronoi_f64"]) <= 1e-12 * np.maximum(area, 1e-300) + 1e-300)
    assert np.all(np.abs(cot - g["cotan_f64"]) <= 1e-12 * np.maximum(np.abs(g["cotan_f64"]), 1.0))
    # every branch is exercised: degenerate (-1), obtuse at p (A/4), at q or r (A/8), clamped
    assert (g["voronoi_f64"] == -1).sum() >= 100
    assert np.isclose(vor, 0.25 * area, rtol=1e-12).sum() >= 100
    assert np.isclose(vor, 0.125 * area, rtol=1e-12).sum() >= 100
    assert (np.abs(g["cotan_f64"]) >= 19.1 - 1e-12).sum() >= 50


def test_cotan_and_voronoi_against_live_reference_build(oracle):
    """Same comparison against oracle/_ref built from the reference tree
    in this checkout (skipped where the tree is absent)."""
    G = oracle.ref_geometry()
    if G is None:
        pytest.skip("oracle/_ref/libref_geometry.so not built (no reference tree)")
    from rxmesh_gb300 import meshgen
    v, f = meshgen.icosphere(3)
    x = meshgen.radial_noise(v, 0.05, 1)
    P, Q, R = (np.ascontiguousarray(x[f[:, k]]) for k in range(3))
    S = np.ascontiguousarray(np.roll(R, 1, axis=0))
    n = len(P)
    out = np.empty(n)
    G.ref_partial_voronoi_area_f64(n, P, Q, R, out)
    assert np.abs(oracle.partial_voronoi_area(P, Q, R) - out).max() <= 1e-15
    G.ref_edge_cotan_weight_f64(n, P, Q, R, S, out)
    assert np.abs(oracle.edge_cotan_weight(P, Q, R, S) - out).max() <= 1e-13
