/*
 * rxg_oracle.c -- CPU restatement of RXMesh's hot-path arithmetic.
 *
 * TEST INFRASTRUCTURE ONLY.  The CUDA library in rxmesh_gb300/csrc is tested
 * for parity against this file.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / --impl reference legs of bench.py may load it.  The product
 * path never calls it and has no CPU fallback.
 *
 * Every function restates a reference function; the citation (path:line, path
 * inside the RXMesh project) is given beside it.  Indices are int32, sizes
 * int64, geometry is FP64 unless a function says otherwise.
 *
 * Pinning: the restatement is checked in tests/ against the reference's own
 * known-answer tests (solver KAT of tests/RXMesh_test/test_solver.cu:79-119,
 * sparse-matrix row counts of tests/RXMesh_test/test_sparse_matrix.cu:111-173,
 * edge-map ground truth of tests/RXMesh_test/rxmesh_test.h:65-340) and against
 * the reference's own apps/VertexNormal/vertex_normal_ref.h compiled from its
 * source into oracle/_ref (see oracle/Makefile).
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_OK 0
#define ORC_ERR_NONMANIFOLD 5
#define ORC_ERR_INVALID 2
#define ORC_ERR_NOMEM 3

/* ------------------------------------------------------------------------ */
/* Edge map                                                                  */
/* ------------------------------------------------------------------------ */

/*
 * Global edge numbering of RXMesh::build_supporting_structures
 * (include/rxmesh/rxmesh.cpp:518-620): faces are visited in input order, each
 * face's edges in the order (v0,v1),(v1,v2),(v2,v0); an edge gets the next id
 * the first time its unordered key (max,min) (util/util.h:410-416) is seen,
 * and its EV pair is stored as first encountered ({v0, v1}).
 *
 * ev_out must hold 2*3*nf ints, fe_out 3*nf ints (edge id of each face edge).
 * Returns the number of edges, or -1 on allocation failure.
 */
int64_t orc_build_edges(int64_t nf, const int32_t* fv, int32_t* ev_out,
                        int32_t* fe_out)
{
    uint64_t cap = 16;
    while (cap < (uint64_t)(nf * 3) * 2) cap <<= 1;
    uint64_t* keys = (uint64_t*)malloc(cap * sizeof(uint64_t));
    int32_t*  ids  = (int32_t*)malloc(cap * sizeof(int32_t));
    if (!keys || !ids) {
        free(keys);
        free(ids);
        return -1;
    }
    for (uint64_t i = 0; i < cap; ++i) keys[i] = UINT64_MAX;
    int64_t ne = 0;
    for (int64_t f = 0; f < nf; ++f) {
        for (int k = 0; k < 3; ++k) {
            uint32_t v0 = (uint32_t)fv[3 * f + k];
            uint32_t v1 = (uint32_t)fv[3 * f + (k + 1) % 3];
            uint32_t hi = v0 > v1 ? v0 : v1, lo = v0 > v1 ? v1 : v0;
            uint64_t key = ((uint64_t)hi << 32) | lo;
            uint64_t h   = key * 0x9E3779B97F4A7C15ull;
            uint64_t s   = (h >> 17) & (cap - 1);
            while (keys[s] != UINT64_MAX && keys[s] != key) s = (s + 1) & (cap - 1);
            if (keys[s] == UINT64_MAX) {
                keys[s]            = key;
                ids[s]             = (int32_t)ne;
                ev_out[2 * ne + 0] = (int32_t)v0;
                ev_out[2 * ne + 1] = (int32_t)v1;
                ++ne;
            }
            fe_out[3 * f + k] = ids[s];
        }
    }
    free(keys);
    free(ids);
    return ne;
}

/* ------------------------------------------------------------------------ */
/* Adjacency ground truth (sets)                                             */
/* ------------------------------------------------------------------------ */

static int cmp_i32(const void* a, const void* b)
{
    int32_t x = *(const int32_t*)a, y = *(const int32_t*)b;
    return (x > y) - (x < y);
}

static void sort_rows(int64_t n, const int64_t* off, int32_t* val)
{
    for (int64_t i = 0; i < n; ++i)
        qsort(val + off[i], (size_t)(off[i + 1] - off[i]), sizeof(int32_t), cmp_i32);
}

/*
 * VV and VE ground truth as in RXMeshTest::run_test
 * (tests/RXMesh_test/rxmesh_test.h:65-160): every edge (a,b) of the edge map
 * adds b to a's list and a to b's list (VE: the edge id to both).  Rows are
 * returned sorted, which is the set form the reference's verifier compares.
 * off has nv+1 entries, val 2*ne.  want_edges selects VE instead of VV.
 */
void orc_vv_ve(int64_t nv, int64_t ne, const int32_t* ev, int want_edges,
               int64_t* off, int32_t* val)
{
    memset(off, 0, sizeof(int64_t) * (size_t)(nv + 1));
    for (int64_t e = 0; e < ne; ++e) {
        off[ev[2 * e] + 1]++;
        off[ev[2 * e + 1] + 1]++;
    }
    for (int64_t v = 0; v < nv; ++v) off[v + 1] += off[v];
    int64_t* cur = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nv + 1));
    memcpy(cur, off, sizeof(int64_t) * (size_t)(nv + 1));
    for (int64_t e = 0; e < ne; ++e) {
        int32_t a = ev[2 * e], b = ev[2 * e + 1];
        val[cur[a]++] = want_edges ? (int32_t)e : b;
        val[cur[b]++] = want_edges ? (int32_t)e : a;
    }
    free(cur);
    sort_rows(nv, off, val);
}

/*
 * VF ground truth (tests/RXMesh_test/rxmesh_test.h:160-230): every face adds
 * itself to the lists of its three vertices.  off: nv+1, val: 3*nf, rows sorted.
 */
void orc_vf(int64_t nv, int64_t nf, const int32_t* fv, int64_t* off, int32_t* val)
{
    memset(off, 0, sizeof(int64_t) * (size_t)(nv + 1));
    for (int64_t i = 0; i < 3 * nf; ++i) off[fv[i] + 1]++;
    for (int64_t v = 0; v < nv; ++v) off[v + 1] += off[v];
    int64_t* cur = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nv + 1));
    memcpy(cur, off, sizeof(int64_t) * (size_t)(nv + 1));
    for (int64_t f = 0; f < nf; ++f)
        for (int k = 0; k < 3; ++k) val[cur[fv[3 * f + k]]++] = (int32_t)f;
    free(cur);
    sort_rows(nv, off, val);
}

/*
 * EF ground truth (the e_f lists of tests/RXMesh_test/rxmesh_test.h:297-315):
 * every face adds itself to the lists of its three edges (fe from
 * orc_build_edges).  off: ne+1, val: 3*nf, rows sorted.
 */
void orc_ef(int64_t ne, int64_t nf, const int32_t* fe, int64_t* off, int32_t* val)
{
    memset(off, 0, sizeof(int64_t) * (size_t)(ne + 1));
    for (int64_t i = 0; i < 3 * nf; ++i) off[fe[i] + 1]++;
    for (int64_t e = 0; e < ne; ++e) off[e + 1] += off[e];
    int64_t* cur = (int64_t*)malloc(sizeof(int64_t) * (size_t)(ne + 1));
    memcpy(cur, off, sizeof(int64_t) * (size_t)(ne + 1));
    for (int64_t f = 0; f < nf; ++f)
        for (int k = 0; k < 3; ++k) val[cur[fe[3 * f + k]]++] = (int32_t)f;
    free(cur);
    sort_rows(ne, off, val);
}

/*
 * FF ground truth (tests/RXMesh_test/rxmesh_test.h:290-330): for every edge,
 * each pair of its faces adds each face to the other's list.  ef_off/ef_val
 * from orc_ef.  With val == NULL only the row counts are written to off
 * (off[f+1] = count of face f, off[0] = 0, then prefix-summed) and the total
 * is returned; otherwise the rows are filled (sorted) and the total returned.
 */
int64_t orc_ff(int64_t nf, int64_t ne, const int64_t* ef_off, const int32_t* ef_val,
               int64_t* off, int32_t* val)
{
    memset(off, 0, sizeof(int64_t) * (size_t)(nf + 1));
    for (int64_t e = 0; e < ne; ++e) {
        const int64_t k = ef_off[e + 1] - ef_off[e];
        for (int64_t i = ef_off[e]; i < ef_off[e + 1]; ++i) off[ef_val[i] + 1] += k - 1;
    }
    for (int64_t f = 0; f < nf; ++f) off[f + 1] += off[f];
    if (val == NULL) return off[nf];
    int64_t* cur = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nf + 1));
    memcpy(cur, off, sizeof(int64_t) * (size_t)(nf + 1));
    for (int64_t e = 0; e < ne; ++e)
        for (int64_t i = ef_off[e]; i < ef_off[e + 1]; ++i)
            for (int64_t j = i + 1; j < ef_off[e + 1]; ++j) {
                val[cur[ef_val[i]]++] = ef_val[j];
                val[cur[ef_val[j]]++] = ef_val[i];
            }
    free(cur);
    sort_rows(nf, off, val);
    return off[nf];
}

/*
 * EVDiamond of e_v_diamond (include/rxmesh/kernels/rxmesh_queries.cuh:197-262):
 * four vertices per edge, out[4e+0] = ev[e][0], out[4e+2] = ev[e][1], and in
 * slot 1 (slot 3) the vertex opposite the edge in the face that traverses
 * it from ev[e][0] to ev[e][1] (from ev[e][1] to ev[e][0]); -1 where there is
 * no such face (boundary).  Face f's edge k runs from corner k to corner
 * k+1, so its opposite vertex is corner k+2.  Edge-manifold meshes.
 */
void orc_ev_diamond(int64_t ne, int64_t nf, const int32_t* fv, const int32_t* ev,
                    const int32_t* fe, int32_t* out)
{
    for (int64_t e = 0; e < ne; ++e) {
        out[4 * e + 0] = ev[2 * e];
        out[4 * e + 1] = -1;
        out[4 * e + 2] = ev[2 * e + 1];
        out[4 * e + 3] = -1;
    }
    for (int64_t f = 0; f < nf; ++f)
        for (int k = 0; k < 3; ++k) {
            const int32_t e   = fe[3 * f + k];
            const int     dir = ev[2 * e] == fv[3 * f + k] ? 0 : 1;
            out[4 * e + 1 + 2 * dir] = fv[3 * f + (k + 2) % 3];
        }
}

/* ------------------------------------------------------------------------ */
/* Vertex normals                                                            */
/* ------------------------------------------------------------------------ */

/*
 * weighting 0: Max (1999) weights, apps/VertexNormal/vertex_normal_ref.h:5-85
 * (and the GPU kernel apps/VertexNormal/vertex_normal_kernel.cuh:10-43): the
 * unnormalised face normal n = (c1-c0)x(c2-c0) is added to vertex i scaled by
 * 1/(|e_i|^2 + |e_{i+2}|^2), e_0=v0v1, e_1=v1v2, e_2=v2v0.  Not normalised.
 * weighting 1: area weights, the unnormalised cross product n (= 2*A*n_hat)
 * added to each vertex of the face.
 * out: nv*3, FP64.
 */
void orc_vertex_normals(int64_t nv, int64_t nf, const int32_t* fv,
                        const double* xyz, int weighting, double* out)
{
    memset(out, 0, sizeof(double) * (size_t)(3 * nv));
    for (int64_t f = 0; f < nf; ++f) {
        int32_t      v[3] = {fv[3 * f], fv[3 * f + 1], fv[3 * f + 2]};
        const double* p0  = xyz + 3 * v[0];
        const double* p1  = xyz + 3 * v[1];
        const double* p2  = xyz + 3 * v[2];
        double        u[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
        double        w[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
        double        n[3] = {u[1] * w[2] - u[2] * w[1], u[2] * w[0] - u[0] * w[2],
                              u[0] * w[1] - u[1] * w[0]};
        double        l[3];
        for (int i = 0; i < 3; ++i) {
            const double* a = xyz + 3 * v[i];
            const double* b = xyz + 3 * v[(i + 1) % 3];
            double        d0 = a[0] - b[0], d1 = a[1] - b[1], d2 = a[2] - b[2];
            l[i]             = d0 * d0 + d1 * d1 + d2 * d2;
        }
        for (int i = 0; i < 3; ++i) {
            int    k   = (i + 2) % 3;
            double inv = weighting == 0 ? 1.0 / (l[i] + l[k]) : 1.0;
            for (int c = 0; c < 3; ++c) out[3 * v[i] + c] += n[c] * inv;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Oriented one-ring                                                         */
/* ------------------------------------------------------------------------ */

/*
 * Oriented VV, the ordering that orient_edges_around_vertices
 * (include/rxmesh/kernels/rxmesh_queries.cuh:376-499) produces for interior
 * vertices of a manifold: neighbours in the rotational order of the incident
 * faces, face (p,a,b) followed by face (p,b,c).  For a boundary vertex the
 * list starts at the neighbour whose edge has no face on one side and walks
 * the fan to the other boundary neighbour (k faces, k+1 neighbours), and
 * bnd[v] = 1.  Interior rows start at the lowest-index incident face.
 *
 * vf_off/vf_val: the VF CSR (any order).  off: nv+1, val: 2*ne.
 * Returns ORC_ERR_NONMANIFOLD when a fan is not a single disk or half-disk.
 */
int orc_oriented_vv(int64_t nv, const int32_t* fv, const int64_t* vf_off,
                    const int32_t* vf_val, int64_t* off, int32_t* val, int8_t* bnd)
{
    off[0] = 0;
    int64_t pos = 0;
    for (int64_t p = 0; p < nv; ++p) {
        int64_t s = vf_off[p], e = vf_off[p + 1], k = e - s;
        bnd[p]    = 0;
        if (k == 0) {
            off[p + 1] = pos;
            continue;
        }
        /* (a,b) = the two other vertices of each incident face, in face order */
        int32_t* A    = (int32_t*)malloc(sizeof(int32_t) * (size_t)(2 * k));
        int32_t* B    = A + k;
        int32_t  fmin = INT32_MAX;
        int64_t  imin = 0;
        for (int64_t i = 0; i < k; ++i) {
            int32_t f = vf_val[s + i];
            int     c = fv[3 * f] == p ? 0 : (fv[3 * f + 1] == p ? 1 : 2);
            A[i]      = fv[3 * f + (c + 1) % 3];
            B[i]      = fv[3 * f + (c + 2) % 3];
            if (f < fmin) {
                fmin = f;
                imin = i;
            }
        }
        /* boundary start: a face whose 'a' is no face's 'b' */
        int64_t start = -1;
        for (int64_t i = 0; i < k && start < 0; ++i) {
            int found = 0;
            for (int64_t j = 0; j < k; ++j)
                if (B[j] == A[i]) {
                    found = 1;
                    break;
                }
            if (!found) start = i;
        }
        int is_b = start >= 0;
        if (!is_b) start = imin;
        int64_t cur = start, nvis = 0;
        val[pos++]  = A[cur];
        while (1) {
            ++nvis;
            int32_t b = B[cur];
            int64_t nxt = -1;
            for (int64_t j = 0; j < k; ++j)
                if (A[j] == b) {
                    nxt = j;
                    break;
                }
            if (nxt < 0 || nxt == start) {
                if (is_b) val[pos++] = b;
                break;
            }
            if (nvis >= k) { /* cycle not through start: non-manifold */
                free(A);
                return ORC_ERR_NONMANIFOLD;
            }
            val[pos++] = b;
            cur        = nxt;
        }
        free(A);
        if (nvis != k) return ORC_ERR_NONMANIFOLD;
        bnd[p]     = (int8_t)is_b;
        off[p + 1] = pos;
    }
    return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* Cotangent Laplacian + mass, MCF system                                    */
/* ------------------------------------------------------------------------ */

static double tri_area3(const double* p0, const double* p1, const double* p2)
{
    /* include/rxmesh/geometry_util.cuh:55-63: 0.5*|(p1-p0)x(p2-p0)| */
    double u[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
    double v[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
    double c[3] = {u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2],
                   u[0] * v[1] - u[1] * v[0]};
    return 0.5 * sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
}

static double clamp_cot(double v)
{
    /* geometry_util.cuh:107-115: clamp to [-19.1, 19.1] */
    const double bound = 19.1;
    return v < -bound ? -bound : (v > bound ? bound : v);
}

static double dot3(const double* a, const double* b)
{
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

/* geometry_util.cuh:117-167 partial_voronoi_area(p, q, r) */
double orc_partial_voronoi_area(const double* p, const double* q, const double* r)
{
    double pq[3] = {q[0] - p[0], q[1] - p[1], q[2] - p[2]};
    double qr[3] = {r[0] - q[0], r[1] - q[1], r[2] - q[2]};
    double pr[3] = {r[0] - p[0], r[1] - p[1], r[2] - p[2]};
    double A     = tri_area3(p, q, r);
    if (A <= DBL_MIN) return -1.0;
    double dotp = dot3(pq, pr);
    double dotq = -dot3(qr, pq);
    double dotr = dot3(qr, pr);
    if (dotp < 0.0) return 0.25 * A;
    if (dotq < 0.0 || dotr < 0.0) return 0.125 * A;
    double cotq = clamp_cot(dotq / A);
    double cotr = clamp_cot(dotr / A);
    return 0.125 * (dot3(pr, pr) * cotq + dot3(pq, pq) * cotr);
}

/* geometry_util.cuh:173-206 partial_weight inside edge_cotan_weight */
double orc_half_cot(const double* p, const double* r, const double* v)
{
    double d0[3] = {p[0] - v[0], p[1] - v[1], p[2] - v[2]};
    double d1[3] = {r[0] - v[0], r[1] - v[1], r[2] - v[2]};
    double A     = tri_area3(p, r, v);
    if (A > DBL_MIN) return clamp_cot(dot3(d0, d1) / A);
    return 0.0;
}

/*
 * MCF system of mcf_A_setup / mcf_B_setup (apps/MCF/mcf_kernels.cuh:302-426),
 * cotangent mode, on the oriented one-ring:
 *   w_pr   = max(0, halfcot(q) + halfcot(s)) * dt     (q,s: ring neighbours of r)
 *   area_p = sum over ring triangles (p, q, r) of max(0, partial_voronoi_area)
 *   A_pp   = 2*area_p + sum_r w_pr,  A_pr = -w_pr,  B_p = 2*area_p * x_p.
 * Interior rows wrap around the ring exactly as the reference does.  Boundary
 * rows (bnd[p]=1) use only the real triangles of the fan (the reference pairs
 * the last and first neighbours there; see the design notes).
 * CSR: row_ptr[p] = off[p] + p, diagonal first then ring order.
 * Outputs row_ptr (nv+1), col (nv + off[nv]), val (same), B (nv*3).
 */
void orc_mcf_assemble(int64_t nv, const int64_t* off, const int32_t* ring,
                      const int8_t* bnd, const double* xyz, double dt,
                      int64_t* row_ptr, int32_t* col, double* val, double* B)
{
    for (int64_t p = 0; p <= nv; ++p) row_ptr[p] = off[p] + p;
    for (int64_t p = 0; p < nv; ++p) {
        int64_t       s = off[p], k = off[p + 1] - off[p];
        int64_t       rp = row_ptr[p];
        const double* P  = xyz + 3 * p;
        double        area = 0.0, sum_w = 0.0;
        int           wrap = !bnd[p];
        col[rp]            = (int32_t)p;
        for (int64_t i = 0; i < k; ++i) {
            int32_t r  = ring[s + i];
            int     has_q = wrap || i > 0;
            int     has_s = wrap || i < k - 1;
            int32_t q  = ring[s + (i + k - 1) % k];
            int32_t sv = ring[s + (i + 1) % k];
            double  w  = 0.0;
            if (has_q) w += orc_half_cot(P, xyz + 3 * r, xyz + 3 * q);
            if (has_s) w += orc_half_cot(P, xyz + 3 * r, xyz + 3 * sv);
            w = (w >= 0.0 ? w : 0.0) * dt;
            sum_w += w;
            col[rp + 1 + i] = r;
            val[rp + 1 + i] = -w;
            if (has_q) {
                double a = orc_partial_voronoi_area(P, xyz + 3 * q, xyz + 3 * r);
                area += a > 0 ? a : 0.0;
            }
        }
        double vw = 0.5 / area;
        val[rp]   = 1.0 / vw + sum_w;
        for (int c = 0; c < 3; ++c) B[3 * p + c] = P[c] / vw;
    }
}

/* ------------------------------------------------------------------------ */
/* CG / Jacobi-PCG                                                           */
/* ------------------------------------------------------------------------ */

static void spmm(int64_t n, int nc, const int64_t* rp, const int32_t* col,
                 const double* val, const double* x, double* y)
{
    for (int64_t i = 0; i < n; ++i) {
        double acc[4] = {0, 0, 0, 0};
        for (int64_t j = rp[i]; j < rp[i + 1]; ++j)
            for (int c = 0; c < nc; ++c) acc[c] += val[j] * x[(int64_t)col[j] * nc + c];
        for (int c = 0; c < nc; ++c) y[i * nc + c] = acc[c];
    }
}

static double vdot(int64_t m, const double* a, const double* b)
{
    double s = 0;
    for (int64_t i = 0; i < m; ++i) s += a[i] * b[i];
    return s;
}

/*
 * CGSolver / PCGSolver (include/rxmesh/matrix/cg_solver.h:37-125,
 * pcg_solver.h:34-144, convergence iterative_solver.h:52-58).  All nc columns
 * form one long vector (one alpha, one beta).  delta is |r|^2 (CG) or r.z
 * (PCG, z = r / (A_ii + eps)); converged when delta < abs_tol or
 * delta/delta_0 < rel_tol.  iters counts completed iterations as the
 * reference's m_iter_taken does (not incremented on the converging one).
 * Vectors are row-major n x nc.  Returns 1 if converged, 0 otherwise.
 */
int orc_cg(int64_t n, int nc, const int64_t* rp, const int32_t* col,
           const double* val, const double* B, double* X, int max_iter,
           double abs_tol, double rel_tol, int precond, int* iters,
           double* start_res, double* final_res)
{
    int64_t m  = n * nc;
    double* S  = (double*)calloc((size_t)m, sizeof(double));
    double* P  = (double*)calloc((size_t)m, sizeof(double));
    double* R  = (double*)calloc((size_t)m, sizeof(double));
    double* Z  = (double*)calloc((size_t)m, sizeof(double));
    double* Di = (double*)calloc((size_t)n, sizeof(double));
    for (int64_t i = 0; i < n; ++i) {
        double d = 0;
        for (int64_t j = rp[i]; j < rp[i + 1]; ++j)
            if (col[j] == i) d = val[j];
        Di[i] = 1.0 / (d + DBL_EPSILON);
    }
    spmm(n, nc, rp, col, val, X, S);
    for (int64_t i = 0; i < m; ++i) R[i] = B[i] - S[i];
    double delta_new;
    if (precond) {
        for (int64_t i = 0; i < m; ++i) P[i] = Di[i / nc] * R[i];
        delta_new = vdot(m, R, P);
    } else {
        for (int64_t i = 0; i < m; ++i) P[i] = R[i];
        delta_new = vdot(m, R, R);
    }
    double d0 = delta_new;
    *start_res = d0;
    int it = 0, conv = 0;
#define CONVERGED(d) ((d) < abs_tol || (d) / d0 < rel_tol)
    if (CONVERGED(delta_new)) {
        conv = 1;
    } else {
        while (it < max_iter) {
            spmm(n, nc, rp, col, val, P, S);
            double alpha = delta_new / vdot(m, S, P);
            for (int64_t i = 0; i < m; ++i) X[i] += alpha * P[i];
            for (int64_t i = 0; i < m; ++i) R[i] -= alpha * S[i];
            double delta_old = delta_new;
            if (precond) {
                for (int64_t i = 0; i < m; ++i) Z[i] = Di[i / nc] * R[i];
                delta_new = vdot(m, R, Z);
            } else {
                delta_new = vdot(m, R, R);
            }
            if (CONVERGED(delta_new)) {
                conv = 1;
                break;
            }
            double beta = delta_new / delta_old;
            const double* src = precond ? Z : R;
            for (int64_t i = 0; i < m; ++i) P[i] = src[i] + beta * P[i];
            ++it;
        }
    }
#undef CONVERGED
    *iters     = it;
    *final_res = delta_new;
    free(S);
    free(P);
    free(R);
    free(Z);
    free(Di);
    return conv;
}

/* y = A x for a CSR matrix, nc columns row-major (used by tests) */
void orc_spmm(int64_t n, int nc, const int64_t* rp, const int32_t* col,
              const double* val, const double* x, double* y)
{
    spmm(n, nc, rp, col, val, x, y);
}

/* ------------------------------------------------------------------------ */
/* Per-face ARAP energy                                                      */
/* ------------------------------------------------------------------------ */

/*
 * Flat rest frame of a face, as apps/Param/param.cu:113-141 builds it:
 * b1 = normalize(b-a), b2 = normalize(((b-a)x(c-a)) x b1),
 * Mr = [[(b-a).b1, (c-a).b1], [0, (c-a).b2]] (edge vectors as columns).
 * Writes Mr^{-1} (row-major 2x2) and the rest area 0.5*det(Mr).
 */
void orc_rest_frame(int64_t nf, const int32_t* fv, const double* xyz,
                    double* minv, double* area)
{
    for (int64_t f = 0; f < nf; ++f) {
        const double* a  = xyz + 3 * fv[3 * f];
        const double* b  = xyz + 3 * fv[3 * f + 1];
        const double* c  = xyz + 3 * fv[3 * f + 2];
        double        e1[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
        double        e2[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
        double        n[3]  = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                               e1[0] * e2[1] - e1[1] * e2[0]};
        double        l1    = sqrt(dot3(e1, e1));
        double        b1[3] = {e1[0] / l1, e1[1] / l1, e1[2] / l1};
        double        t[3]  = {n[1] * b1[2] - n[2] * b1[1], n[2] * b1[0] - n[0] * b1[2],
                               n[0] * b1[1] - n[1] * b1[0]};
        double        lt    = sqrt(dot3(t, t));
        double        b2[3] = {t[0] / lt, t[1] / lt, t[2] / lt};
        double        m00 = dot3(e1, b1), m01 = dot3(e2, b1), m10 = 0.0, m11 = dot3(e2, b2);
        double        det = m00 * m11 - m01 * m10;
        minv[4 * f + 0]   = m11 / det;
        minv[4 * f + 1]   = -m01 / det;
        minv[4 * f + 2]   = -m10 / det;
        minv[4 * f + 3]   = m00 / det;
        area[f]           = 0.5 * det;
    }
}

/*
 * Per-face ARAP energy E = A * ||J - R(J)||_F^2, J = [b-a, c-a] * Mr^{-1}
 * (3x2), R(J) the polar factor.  With j1, j2 the columns of J the singular
 * values satisfy s1^2+s2^2 = |j1|^2+|j2|^2 =: s and s1*s2 = |j1 x j2| =: d, so
 *   E = A * (s - 2*sqrt(s + 2d) + 2)
 * which is differentiated analytically (gradient 9, Hessian 9x9 row-major,
 * variables ordered a.xyz, b.xyz, c.xyz).  Either output may be NULL.
 */
double orc_arap_face(const double* x9, const double* minv, double A,
                     double* grad, double* hess)
{
    double dcoef[3][2];
    for (int k = 0; k < 2; ++k) {
        dcoef[1][k] = minv[0 * 2 + k];
        dcoef[2][k] = minv[1 * 2 + k];
        dcoef[0][k] = -(dcoef[1][k] + dcoef[2][k]);
    }
    double u[6] = {0, 0, 0, 0, 0, 0};
    for (int k = 0; k < 2; ++k)
        for (int v = 0; v < 3; ++v)
            for (int c = 0; c < 3; ++c) u[3 * k + c] += dcoef[v][k] * x9[3 * v + c];
    const double* j1 = u;
    const double* j2 = u + 3;
    double        s  = dot3(j1, j1) + dot3(j2, j2);
    double        w[3] = {j1[1] * j2[2] - j1[2] * j2[1], j1[2] * j2[0] - j1[0] * j2[2],
                          j1[0] * j2[1] - j1[1] * j2[0]};
    double        d  = sqrt(dot3(w, w));
    double        q  = s + 2.0 * d;
    double        sq = sqrt(q);
    double        E  = A * (s - 2.0 * sq + 2.0);
    if (!grad && !hess) return E;

    /* W = dw/du = [ -[j2]x , [j1]x ] (3x6) */
    double W[3][6];
    {
        double cj2[3][3] = {{0, -j2[2], j2[1]}, {j2[2], 0, -j2[0]}, {-j2[1], j2[0], 0}};
        double cj1[3][3] = {{0, -j1[2], j1[1]}, {j1[2], 0, -j1[0]}, {-j1[1], j1[0], 0}};
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                W[i][j]     = -cj2[i][j];
                W[i][j + 3] = cj1[i][j];
            }
    }
    double wh[3] = {0, 0, 0};
    if (d > 0) {
        wh[0] = w[0] / d;
        wh[1] = w[1] / d;
        wh[2] = w[2] / d;
    }
    double gd[6], gq[6], gE[6];
    for (int i = 0; i < 6; ++i) {
        gd[i] = W[0][i] * wh[0] + W[1][i] * wh[1] + W[2][i] * wh[2];
        gq[i] = 2.0 * u[i] + 2.0 * gd[i];
        gE[i] = A * (2.0 * u[i] - gq[i] / sq);
    }
    if (grad)
        for (int v = 0; v < 3; ++v)
            for (int c = 0; c < 3; ++c)
                grad[3 * v + c] = dcoef[v][0] * gE[c] + dcoef[v][1] * gE[3 + c];
    if (!hess) return E;

    double Hd[6][6];
    memset(Hd, 0, sizeof(Hd));
    if (d > 0) {
        double P[3][3];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) P[i][j] = ((i == j) - wh[i] * wh[j]) / d;
        for (int a = 0; a < 6; ++a)
            for (int b = 0; b < 6; ++b) {
                double acc = 0;
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) acc += W[i][a] * P[i][j] * W[j][b];
                Hd[a][b] = acc;
            }
        /* sum_k wh_k Hess(w_k): top-right block -[wh]x, bottom-left [wh]x */
        double cw[3][3] = {{0, -wh[2], wh[1]}, {wh[2], 0, -wh[0]}, {-wh[1], wh[0], 0}};
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                Hd[i][3 + j] += -cw[i][j];
                Hd[3 + i][j] += cw[i][j];
            }
    }
    double Hu[6][6];
    for (int a = 0; a < 6; ++a)
        for (int b = 0; b < 6; ++b) {
            double hs = (a == b) ? 2.0 : 0.0;
            double hq = hs + 2.0 * Hd[a][b];
            Hu[a][b]  = A * (hs - hq / sq + gq[a] * gq[b] / (2.0 * q * sq));
        }
    for (int vi = 0; vi < 3; ++vi)
        for (int ci = 0; ci < 3; ++ci)
            for (int vj = 0; vj < 3; ++vj)
                for (int cj = 0; cj < 3; ++cj) {
                    double acc = 0;
                    for (int k = 0; k < 2; ++k)
                        for (int l = 0; l < 2; ++l)
                            acc += dcoef[vi][k] * dcoef[vj][l] * Hu[3 * k + ci][3 * l + cj];
                    hess[(3 * vi + ci) * 9 + 3 * vj + cj] = acc;
                }
    return E;
}

/*
 * ARAP assembly over a mesh, in the layout DiffScalarProblem produces
 * (diff/diff_query_kernel.cuh:265-314): per-face energy, gradient V x 3, and
 * the Hessian as 3x3 blocks (row-major) on a block-CSR pattern (rp, col)
 * that contains the diagonal and every edge.  Returns the total energy.
 */
/*
 * Cyclic Jacobi eigen-decomposition of a symmetric k x k matrix (k <= 9;
 * Golub and Van Loan, Matrix Computations, sec. 8.5): A (row-major) is
 * rotated until its off-diagonal part vanishes, leaving the eigenvalues on
 * its diagonal; V receives the eigenvectors as columns.  Each rotation
 * zeroes A[p][q] with t = sgn(th) / (|th| + sqrt(th^2 + 1)),
 * th = (A[q][q] - A[p][p]) / (2 A[p][q]), c = 1/sqrt(1 + t^2), s = t c.
 */
static void jacobi_eig(int k, double* A, double* V)
{
    for (int i = 0; i < k * k; ++i) V[i] = (i % (k + 1)) == 0 ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 50; ++sweep) {
        double off = 0, all = 0;
        for (int i = 0; i < k; ++i)
            for (int j = 0; j < k; ++j) {
                all += A[i * k + j] * A[i * k + j];
                if (i != j) off += A[i * k + j] * A[i * k + j];
            }
        if (off <= 1e-30 * all) break;
        for (int p = 0; p < k - 1; ++p)
            for (int q = p + 1; q < k; ++q) {
                const double apq = A[p * k + q];
                if (apq == 0.0) continue;
                const double th = (A[q * k + q] - A[p * k + p]) / (2.0 * apq);
                const double t  = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
                const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                for (int r = 0; r < k; ++r) {
                    const double arp = A[r * k + p], arq = A[r * k + q];
                    A[r * k + p] = c * arp - s * arq;
                    A[r * k + q] = s * arp + c * arq;
                }
                for (int r = 0; r < k; ++r) {
                    const double apr = A[p * k + r], aqr = A[q * k + r];
                    A[p * k + r] = c * apr - s * aqr;
                    A[q * k + r] = s * apr + c * aqr;
                }
                for (int r = 0; r < k; ++r) {
                    const double vrp = V[r * k + p], vrq = V[r * k + q];
                    V[r * k + p] = c * vrp - s * vrq;
                    V[r * k + q] = s * vrp + c * vrq;
                }
            }
    }
}

/*
 * project_positive_definite (include/rxmesh/diff/hessian_projection.h:21-95):
 * a symmetric k x k H (k <= 9) that is positive diagonally dominant with
 * margin eps (H_ii >= sum_j!=i |H_ij| + eps for every i) is left alone;
 * otherwise its eigenvalues below eps are raised to eps and, if any was,
 * H = V diag(lambda) V^T.  eps: 1e-9 (FP64) / 1e-6 (FP32) in the reference.
 */
void orc_project_pd(int k, double* H, double eps)
{
    int dd = 1;
    for (int i = 0; i < k && dd; ++i) {
        double off = 0;
        for (int j = 0; j < k; ++j)
            if (j != i) off += fabs(H[i * k + j]);
        if (H[i * k + i] < off + eps) dd = 0;
    }
    if (dd) return;
    double A[81], V[81], lam[9];
    memcpy(A, H, sizeof(double) * (size_t)(k * k));
    jacobi_eig(k, A, V);
    int clamped = 0;
    for (int i = 0; i < k; ++i) {
        lam[i] = A[i * k + i];
        if (lam[i] < eps) {
            lam[i]  = eps;
            clamped = 1;
        }
    }
    if (!clamped) return;
    for (int i = 0; i < k; ++i)
        for (int j = 0; j < k; ++j) {
            double v = 0;
            for (int m = 0; m < k; ++m) v += V[i * k + m] * lam[m] * V[j * k + m];
            H[i * k + j] = v;
        }
}

/* orc_arap_assemble with each face's 9x9 Hessian projected (project != 0,
 * the reference's add_term<Op::FV, ProjectHess = true>) before the scatter. */
double orc_arap_assemble_ex(int64_t nv, int64_t nf, const int32_t* fv,
                            const double* x, const double* minv, const double* area,
                            const int64_t* rp, const int32_t* col, double* face_E,
                            double* grad, double* hblk, int project, double eps);

double orc_arap_assemble(int64_t nv, int64_t nf, const int32_t* fv,
                         const double* x, const double* minv, const double* area,
                         const int64_t* rp, const int32_t* col, double* face_E,
                         double* grad, double* hblk)
{
    return orc_arap_assemble_ex(nv, nf, fv, x, minv, area, rp, col, face_E, grad, hblk, 0, 0.0);
}

double orc_arap_assemble_ex(int64_t nv, int64_t nf, const int32_t* fv,
                         const double* x, const double* minv, const double* area,
                            const int64_t* rp, const int32_t* col, double* face_E,
                            double* grad, double* hblk, int project, double eps)
{
    double total = 0;
    if (grad) memset(grad, 0, sizeof(double) * (size_t)(3 * nv));
    if (hblk) memset(hblk, 0, sizeof(double) * (size_t)(9 * rp[nv]));
    for (int64_t f = 0; f < nf; ++f) {
        double  x9[9], g[9], H[81];
        int32_t v[3] = {fv[3 * f], fv[3 * f + 1], fv[3 * f + 2]};
        for (int i = 0; i < 3; ++i)
            for (int c = 0; c < 3; ++c) x9[3 * i + c] = x[3 * v[i] + c];
        double E = orc_arap_face(x9, minv + 4 * f, area[f], g, hblk ? H : NULL);
        if (hblk && project) orc_project_pd(9, H, eps);
        if (face_E) face_E[f] = E;
        total += E;
        if (grad)
            for (int i = 0; i < 3; ++i)
                for (int c = 0; c < 3; ++c) grad[3 * v[i] + c] += g[3 * i + c];
        if (hblk)
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) {
                    int64_t slot = -1;
                    for (int64_t t = rp[v[i]]; t < rp[v[i] + 1]; ++t)
                        if (col[t] == v[j]) {
                            slot = t;
                            break;
                        }
                    if (slot < 0) continue;
                    for (int a = 0; a < 3; ++a)
                        for (int b = 0; b < 3; ++b)
                            hblk[9 * slot + 3 * a + b] += H[(3 * i + a) * 9 + 3 * j + b];
                }
    }
    return total;
}
