// Host-side mesh build: edge map, patch partition, per-patch local topology
// and its upload to the device.  Restates the structure RXMesh builds in
// RXMesh::init / build / build_single_patch_ltog / build_single_patch_topology
// (include/rxmesh/rxmesh.cpp:86-225, 290-426, 754-996) with a different
// layout: one 16-byte-aligned arena of per-patch slices, and a dense
// ribbon -> linear-id table in place of RXMesh's LP hashtable
// (include/rxmesh/lp_hashtable.h:46-50).
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>

#include "rxg_internal.h"

namespace rxg {

static thread_local char g_msg[512] = "";

void set_error(const char* fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_msg, sizeof(g_msg), fmt, ap);
    va_end(ap);
}

rxg_status cuda_status(cudaError_t e, const char* what)
{
    set_error("%s: %s", what, cudaGetErrorString(e));
    if (e == cudaErrorMemoryAllocation) return RXG_ERR_NOMEM;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return RXG_ERR_NO_DEVICE;
    return RXG_ERR_CUDA;
}

// Stream-ordered scratch from a pool the library owns, one per device,
// created on first use.  Its release threshold keeps freed blocks for reuse,
// so a call that allocates and frees tens of MB (host-array staging, face
// records) does not map memory again after every synchronisation, as the
// device's default pool (release threshold 0) may.
cudaError_t scratch_alloc(void** p, size_t bytes, cudaStream_t s)
{
    static std::mutex       mu;
    static cudaMemPool_t    pools[64] = {};
    int                     dev       = 0;
    cudaError_t             e         = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaMallocAsync(p, bytes, s);
    cudaMemPool_t pool;
    {
        std::lock_guard<std::mutex> lk(mu);
        if (!pools[dev]) {
            cudaMemPoolProps props = {};
            props.allocType        = cudaMemAllocationTypePinned;
            props.location.type    = cudaMemLocationTypeDevice;
            props.location.id      = dev;
            if ((e = cudaMemPoolCreate(&pools[dev], &props)) != cudaSuccess) return e;
            uint64_t keep = UINT64_MAX;
            if ((e = cudaMemPoolSetAttribute(pools[dev], cudaMemPoolAttrReleaseThreshold, &keep)) !=
                cudaSuccess)
                return e;
        }
        pool = pools[dev];
    }
    return cudaMallocFromPoolAsync(p, bytes ? bytes : 16, pool, s);
}

bool is_device_ptr(const void* p)
{
    if (p == nullptr) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

namespace {

// Open-addressing map from an undirected edge key to its id, assigning ids in
// first-appearance order over (face, local edge), which is RXMesh's global
// edge numbering (rxmesh.cpp:565-600).
struct EdgeTable
{
    std::vector<uint64_t> keys;
    std::vector<int32_t>  ids;
    uint64_t              mask = 0;

    explicit EdgeTable(uint64_t expected)
    {
        uint64_t cap = 16;
        while (cap < expected * 2) cap <<= 1;
        keys.assign(cap, UINT64_MAX);
        ids.assign(cap, -1);
        mask = cap - 1;
    }
    // returns slot; *inserted tells whether the key was new
    uint64_t find_or_insert(uint64_t key, bool* inserted)
    {
        uint64_t s = ((key * 0x9E3779B97F4A7C15ull) >> 17) & mask;
        while (keys[s] != UINT64_MAX && keys[s] != key) s = (s + 1) & mask;
        *inserted = keys[s] == UINT64_MAX;
        if (*inserted) keys[s] = key;
        return s;
    }
};

inline int32_t pad4(int32_t words) { return (words + 3) & ~3; }

int32_t find_root(std::vector<int32_t>& up, int32_t x)
{
    while (up[x] != x) x = up[x] = up[up[x]];
    return x;
}

}  // namespace

static rxg_status build_host(Mesh& M, const int32_t* fv, int64_t nf, int64_t nv, int32_t P,
                             bool split_components, const Partition* part = nullptr,
                             bool gpu_patcher = false)
{
    M.nf          = nf;
    M.nv          = nv;
    M.patch_faces = P;
    M.fv_in.assign(fv, fv + 3 * nf);

    // ---- edge map ------------------------------------------------------
    EdgeTable            tab((uint64_t)nf * 3);
    std::vector<int32_t> fe(3 * nf), e_first_face;
    e_first_face.reserve(nf * 3 / 2 + 16);
    M.ev_in.reserve(nf * 3 + 32);
    for (int64_t f = 0; f < nf; ++f) {
        for (int k = 0; k < 3; ++k) {
            uint32_t v0 = (uint32_t)fv[3 * f + k], v1 = (uint32_t)fv[3 * f + (k + 1) % 3];
            uint32_t hi = std::max(v0, v1), lo = std::min(v0, v1);
            bool     ins;
            uint64_t s = tab.find_or_insert(((uint64_t)hi << 32) | lo, &ins);
            if (ins) {
                tab.ids[s] = (int32_t)(M.ev_in.size() / 2);
                M.ev_in.push_back((int32_t)v0);
                M.ev_in.push_back((int32_t)v1);
                e_first_face.push_back((int32_t)f);
            }
            fe[3 * f + k] = tab.ids[s];
        }
    }
    const int64_t ne = (int64_t)M.ev_in.size() / 2;
    M.ne             = ne;
    { std::vector<uint64_t>().swap(tab.keys); std::vector<int32_t>().swap(tab.ids); }

    // ---- edge -> faces, vertex -> faces, valences ----------------------
    std::vector<int32_t> ef_off(ne + 1, 0), ef_val(3 * nf);
    for (int64_t i = 0; i < 3 * nf; ++i) ef_off[fe[i] + 1]++;
    for (int64_t e = 0; e < ne; ++e) {
        int32_t c = ef_off[e + 1];
        if (c != 2) M.closed = false;
        if (c > 2) M.edge_manifold = false;
        ef_off[e + 1] += ef_off[e];
    }
    {
        std::vector<int32_t> cur(ef_off.begin(), ef_off.end() - 1);
        std::vector<uint8_t> dirs(ne, 0);  // bit 0 / 1: traversed from ev[0] / ev[1]
        for (int64_t f = 0; f < nf; ++f)
            for (int k = 0; k < 3; ++k) {
                const int32_t e = fe[3 * f + k];
                ef_val[cur[e]++] = (int32_t)f;
                const uint8_t bit = M.ev_in[2 * e] == fv[3 * f + k] ? 1 : 2;
                if (dirs[e] & bit) M.oriented = false;
                dirs[e] |= bit;
            }
    }
    std::vector<int32_t> vf_off(nv + 1, 0), vf_val(3 * nf), valence(nv, 0);
    for (int64_t i = 0; i < 3 * nf; ++i) vf_off[fv[i] + 1]++;
    for (int64_t v = 0; v < nv; ++v) vf_off[v + 1] += vf_off[v];
    {
        std::vector<int32_t> cur(vf_off.begin(), vf_off.end() - 1);
        for (int64_t f = 0; f < nf; ++f)
            for (int k = 0; k < 3; ++k) vf_val[cur[fv[3 * f + k]]++] = (int32_t)f;
    }
    for (int64_t e = 0; e < ne; ++e) {
        valence[M.ev_in[2 * e]]++;
        valence[M.ev_in[2 * e + 1]]++;
    }
    for (int64_t v = 0; v < nv; ++v) M.max_valence = std::max<int64_t>(M.max_valence, valence[v]);
    for (int64_t e = 0; e < ne; ++e) M.max_edge_faces = std::max(M.max_edge_faces, ef_off[e + 1] - ef_off[e]);
    for (int64_t f = 0; f < nf; ++f) {
        int32_t n = 0;
        for (int k = 0; k < 3; ++k) n += ef_off[fe[3 * f + k] + 1] - ef_off[fe[3 * f + k]] - 1;
        M.max_face_faces = std::max(M.max_face_faces, n);
    }

    // ---- face-connected components (through shared edges) -------------
    const bool           gpu_partitioning = gpu_patcher && !part;
    std::vector<int32_t> comp_of;  // smallest face id of each face's component
    {
        std::vector<int32_t> up(nf);
        for (int64_t f = 0; f < nf; ++f) up[f] = (int32_t)f;
        for (int64_t e = 0; e < ne; ++e)
            for (int32_t t = ef_off[e] + 1; t < ef_off[e + 1]; ++t) {
                const int32_t a = find_root(up, ef_val[ef_off[e]]), b = find_root(up, ef_val[t]);
                if (a != b) up[std::max(a, b)] = std::min(a, b);
            }
        M.num_components = 0;
        for (int64_t f = 0; f < nf; ++f) M.num_components += find_root(up, (int32_t)f) == f;
        if (gpu_partitioning) {
            comp_of.resize(nf);
            for (int64_t f = 0; f < nf; ++f) comp_of[f] = find_root(up, (int32_t)f);
        }
    }

    // ---- partition on the GPU (Lloyd region growing), then built like a
    // given partition
    Partition            gpart;
    std::vector<int32_t> gface;
    if (gpu_partitioning) {
        std::vector<int32_t> ff_off(nf + 1, 0), ff_val;
        for (int64_t f = 0; f < nf; ++f)
            for (int k = 0; k < 3; ++k) {
                const int32_t e = fe[3 * f + k];
                ff_off[f + 1] += ef_off[e + 1] - ef_off[e] - 1;
            }
        for (int64_t f = 0; f < nf; ++f) ff_off[f + 1] += ff_off[f];
        ff_val.resize(ff_off[nf]);
        for (int64_t f = 0; f < nf; ++f) {
            int32_t j = ff_off[f];
            for (int k = 0; k < 3; ++k) {
                const int32_t e = fe[3 * f + k];
                for (int32_t t = ef_off[e]; t < ef_off[e + 1]; ++t)
                    if (ef_val[t] != f) ff_val[j++] = ef_val[t];
            }
        }
        int32_t          gnp = 0;
        const rxg_status st  = gpu_partition(nf, ff_off, ff_val, comp_of, P, gface, gnp, M.lloyd_runs);
        if (st != RXG_OK) return st;
        gpart.face       = gface.data();
        gpart.patch_size = P;
        part             = &gpart;
    }

    // ---- patch partition: BFS region growing on the face graph ----------
    // (RXMesh uses GPU Lloyd k-means, patcher/patcher.cu:828-1035; the query
    //  engine needs only the <= P faces per patch contract.)
    std::vector<int32_t> fpatch(nf, -1);
    std::vector<int32_t> queue(part ? 0 : nf);
    int32_t              np = 0;
    int64_t              seed = 0;
    if (part) {
        // every patch id in [0, np) owns between 1 and 4096 faces
        int64_t hi = -1;
        for (int64_t f = 0; f < nf; ++f) {
            if (part->face[f] < 0) {
                set_error("face_patch[%lld] = %d is negative", (long long)f, part->face[f]);
                return RXG_ERR_INVALID;
            }
            hi = std::max<int64_t>(hi, part->face[f]);
        }
        if (hi >= nf) {
            set_error("face_patch names patch %lld, more patches than faces", (long long)hi);
            return RXG_ERR_INVALID;
        }
        np = (int32_t)hi + 1;
        std::vector<int32_t> cnt(np, 0);
        for (int64_t f = 0; f < nf; ++f) ++cnt[fpatch[f] = part->face[f]];
        int32_t largest = 0;
        for (int32_t p = 0; p < np; ++p) {
            if (cnt[p] == 0 || cnt[p] > 4096) {
                set_error("patch %d owns %d faces (every patch in [0, %d) must own 1 to 4096)", p,
                          cnt[p], np);
                return RXG_ERR_INVALID;
            }
            largest = std::max(largest, cnt[p]);
        }
        M.patch_faces = std::max(part->patch_size, largest);
        if (part->edge && part->ne != ne) {
            set_error("edge_patch has %lld entries, the mesh has %lld edges",
                      (long long)part->ne, (long long)ne);
            return RXG_ERR_INVALID;
        }
    }
    while (!part) {
        while (seed < nf && fpatch[seed] >= 0) ++seed;
        if (seed >= nf) break;
        int32_t p = np++;
        int64_t qh = 0, qt = 0, cnt = 0;
        fpatch[seed] = p;
        queue[qt++]  = (int32_t)seed;
        cnt          = 1;
        while (cnt < P) {
            if (qh == qt) {
                // a component is exhausted: close the patch, or keep filling it
                // from the next unassigned face (never across components when
                // split_components asks each component to keep its own patches)
                if (split_components || cnt >= P / 2) break;
                while (seed < nf && fpatch[seed] >= 0) ++seed;
                if (seed >= nf) break;
                fpatch[seed] = p;
                queue[qt++]  = (int32_t)seed;
                ++cnt;
                continue;
            }
            int32_t f = queue[qh++];
            for (int k = 0; k < 3 && cnt < P; ++k) {
                int32_t e = fe[3 * f + k];
                for (int32_t t = ef_off[e]; t < ef_off[e + 1] && cnt < P; ++t) {
                    int32_t g = ef_val[t];
                    if (fpatch[g] < 0) {
                        fpatch[g]   = p;
                        queue[qt++] = g;
                        ++cnt;
                    }
                }
            }
        }
    }
    const int32_t nfp = np;  // patches that own faces
    M.num_face_patches = nfp;
    // isolated vertices (in no face) go to extra face-less patches
    std::vector<int32_t> vpatch(nv, -1), epatch(ne);
    if (!part) {
        // the patch of the vertex's first face, of the edge's first face
        for (int64_t f = 0; f < nf; ++f)
            for (int k = 0; k < 3; ++k)
                if (vpatch[fv[3 * f + k]] < 0) vpatch[fv[3 * f + k]] = fpatch[f];
        for (int64_t e = 0; e < ne; ++e) epatch[e] = fpatch[e_first_face[e]];
    } else {
        // the given owner, which must be the patch of one of the element's
        // faces, else the lowest such patch
        auto owner = [&](const int32_t* given, int64_t i, const std::vector<int32_t>& off,
                         const std::vector<int32_t>& val, const char* what) -> int32_t {
            int32_t lo = INT32_MAX;
            bool    ok = false;
            for (int32_t t = off[i]; t < off[i + 1]; ++t) {
                lo = std::min(lo, fpatch[val[t]]);
                ok |= given && fpatch[val[t]] == given[i];
            }
            if (!given) return lo;
            if (!ok) {
                set_error("%s_patch[%lld] = %d is not the patch of any of its faces", what,
                          (long long)i, given[i]);
                return -1;
            }
            return given[i];
        };
        for (int64_t v = 0; v < nv; ++v)
            if (vf_off[v + 1] > vf_off[v] &&
                (vpatch[v] = owner(part->vertex, v, vf_off, vf_val, "vertex")) < 0)
                return RXG_ERR_INVALID;
        for (int64_t e = 0; e < ne; ++e)
            if ((epatch[e] = owner(part->edge, e, ef_off, ef_val, "edge")) < 0)
                return RXG_ERR_INVALID;
    }
    {
        int32_t extra = -1, fill = 0;
        for (int64_t v = 0; v < nv; ++v)
            if (vpatch[v] < 0) {
                if (extra < 0 || fill == 4096) {
                    extra = np++;
                    fill  = 0;
                }
                vpatch[v] = extra;
                ++fill;
            }
    }
    M.num_patches = np;

    // ---- owned lists (counting sort by patch, input order inside) -------
    auto bucket = [&](const std::vector<int32_t>& owner, int64_t n, std::vector<int32_t>& off,
                      std::vector<int32_t>& val) {
        off.assign(np + 1, 0);
        val.resize(n);
        for (int64_t i = 0; i < n; ++i) off[owner[i] + 1]++;
        for (int32_t p = 0; p < np; ++p) off[p + 1] += off[p];
        std::vector<int32_t> cur(off.begin(), off.end() - 1);
        for (int64_t i = 0; i < n; ++i) val[cur[owner[i]]++] = (int32_t)i;
    };
    std::vector<int32_t> pv_off, pv_val, pe_off, pe_val, pf_off, pf_val;
    bucket(vpatch, nv, pv_off, pv_val);
    bucket(epatch, ne, pe_off, pe_val);
    bucket(fpatch, nf, pf_off, pf_val);

    // linear ids: owned elements of patch 0, then patch 1, ...
    M.v_l2i = pv_val;
    M.e_l2i = pe_val;
    M.f_l2i = pf_val;
    M.v_i2l.resize(nv);
    M.e_i2l.resize(ne);
    M.f_i2l.resize(nf);
    for (int64_t i = 0; i < nv; ++i) M.v_i2l[M.v_l2i[i]] = (int32_t)i;
    // boundary vertices: the ends of edges with fewer than two faces
    M.vbnd.assign(nv, 0);
    for (int64_t e = 0; e < ne; ++e)
        if (ef_off[e + 1] - ef_off[e] < 2) {
            M.vbnd[M.v_i2l[M.ev_in[2 * e]]]     = 1;
            M.vbnd[M.v_i2l[M.ev_in[2 * e + 1]]] = 1;
        }
    for (int64_t i = 0; i < ne; ++i) M.e_i2l[M.e_l2i[i]] = (int32_t)i;
    for (int64_t i = 0; i < nf; ++i) M.f_i2l[M.f_l2i[i]] = (int32_t)i;

    // ---- per-patch local topology ---------------------------------------
    std::vector<int32_t> vstamp(nv, -1), vloc(nv), estamp(ne, -1), eloc(ne), fstamp(nf, -1);
    std::vector<int32_t> lf, lv, le;
    M.hdr.resize(np);
    M.arena.clear();
    M.arena.reserve((size_t)(ne * 1.4 + nf * 2.2 + nv * 0.6) + 64 * (size_t)np);
    M.nrm.clear();
    M.nrm.reserve((size_t)(nf * 3.0 + nv * 1.2) + 16 * (size_t)np);
    M.nrm_off.assign((size_t)np + 1, 0);
    int64_t vv_acc = 0, vf_acc = 0, ef_acc = 0, ff_acc = 0;
    M.ef_base.assign((size_t)np + 1, 0);
    M.ff_base.assign((size_t)np + 1, 0);
    for (int32_t p = 0; p < np; ++p) {
        lf.clear();
        lv.clear();
        le.clear();
        for (int32_t t = pf_off[p]; t < pf_off[p + 1]; ++t) {
            lf.push_back(pf_val[t]);
            fstamp[pf_val[t]] = p;
        }
        const int32_t nFo = (int32_t)lf.size();
        for (int32_t t = pv_off[p]; t < pv_off[p + 1]; ++t) {
            int32_t v = pv_val[t];
            vstamp[v] = p;
            vloc[v]   = (int32_t)lv.size();
            lv.push_back(v);
        }
        const int32_t nVo = (int32_t)lv.size();
        for (int32_t t = pe_off[p]; t < pe_off[p + 1]; ++t) {
            int32_t e = pe_val[t];
            estamp[e] = p;
            eloc[e]   = (int32_t)le.size();
            le.push_back(e);
        }
        const int32_t nEo = (int32_t)le.size();
        // ribbon faces: faces incident to owned vertices but owned elsewhere
        size_t rf_begin = lf.size();
        for (int32_t i = 0; i < nVo; ++i) {
            int32_t v = lv[i];
            for (int32_t t = vf_off[v]; t < vf_off[v + 1]; ++t) {
                int32_t f = vf_val[t];
                if (fstamp[f] != p) {
                    fstamp[f] = p;
                    lf.push_back(f);
                }
            }
        }
        // and the faces sharing an edge with an owned face, so that every
        // face of an owned edge, and every edge neighbour of an owned face,
        // is local (the edge and face queries read them)
        for (int32_t i = 0; i < nFo; ++i) {
            const int32_t f = lf[i];
            for (int k = 0; k < 3; ++k) {
                const int32_t e = fe[3 * f + k];
                for (int32_t t = ef_off[e]; t < ef_off[e + 1]; ++t) {
                    const int32_t g = ef_val[t];
                    if (fstamp[g] != p) {
                        fstamp[g] = p;
                        lf.push_back(g);
                    }
                }
            }
        }
        std::sort(lf.begin() + rf_begin, lf.end());
        // ribbon vertices and edges: the rest of the local faces' elements
        size_t rv_begin = lv.size(), re_begin = le.size();
        for (size_t i = 0; i < lf.size(); ++i) {
            int32_t f = lf[i];
            for (int k = 0; k < 3; ++k) {
                int32_t v = fv[3 * f + k];
                if (vstamp[v] != p) {
                    vstamp[v] = p;
                    lv.push_back(v);
                }
                int32_t e = fe[3 * f + k];
                if (estamp[e] != p) {
                    estamp[e] = p;
                    le.push_back(e);
                }
            }
        }
        std::sort(lv.begin() + rv_begin, lv.end());
        std::sort(le.begin() + re_begin, le.end());
        for (size_t i = rv_begin; i < lv.size(); ++i) vloc[lv[i]] = (int32_t)i;
        for (size_t i = re_begin; i < le.size(); ++i) eloc[le[i]] = (int32_t)i;

        const int32_t nVl = (int32_t)lv.size(), nEl = (int32_t)le.size(), nFl = (int32_t)lf.size();
        if (nVl > 65535 || nEl > 32767 || nFl > 65535) {
            set_error("patch %d has %d vertices, %d edges, %d faces: exceeds the 16-bit local "
                      "index limits (65535 / 32767 / 65535); use smaller patches",
                      p, nVl, nEl, nFl);
            return RXG_ERR_PATCH_LIMIT;
        }
        PatchHdr& h = M.hdr[p];
        h.nVo = nVo;
        h.nVl = nVl;
        h.nEo = nEo;
        h.nEl = nEl;
        h.nFo = nFo;
        h.nFl = nFl;
        h.v_base  = pv_off[p];
        h.e_base  = pe_off[p];
        h.f_base  = pf_off[p];
        h.vv_base = (int32_t)vv_acc;
        h.vf_base = (int32_t)vf_acc;
        for (int32_t i = 0; i < nVo; ++i) {
            vv_acc += valence[lv[i]];
            vf_acc += vf_off[lv[i] + 1] - vf_off[lv[i]];
        }
        M.ef_base[p] = (int32_t)ef_acc;
        M.ff_base[p] = (int32_t)ff_acc;
        for (int32_t i = 0; i < nEo; ++i) ef_acc += ef_off[le[i] + 1] - ef_off[le[i]];
        for (int32_t i = 0; i < nFo; ++i)
            for (int k = 0; k < 3; ++k) {
                const int32_t e = fe[3 * lf[i] + k];
                ff_acc += ef_off[e + 1] - ef_off[e] - 1;
            }
        if (ef_acc > INT32_MAX || ff_acc > INT32_MAX) {
            set_error("edge/face query sizes exceed 2^31 values");
            return RXG_ERR_PATCH_LIMIT;
        }
        M.ef_base[p + 1] = (int32_t)ef_acc;
        M.ff_base[p + 1] = (int32_t)ff_acc;
        // arena slices
        h.ev_off = (int32_t)M.arena.size();
        for (int32_t i = 0; i < nEl; ++i) {
            int32_t e = le[i];
            uint32_t a = (uint32_t)vloc[M.ev_in[2 * e]], b = (uint32_t)vloc[M.ev_in[2 * e + 1]];
            M.arena.push_back(a | (b << 16));
        }
        M.arena.resize(h.ev_off + pad4(nEl), 0u);
        h.fe_off = (int32_t)M.arena.size();
        {
            int32_t words = pad4((3 * nFl + 1) / 2);
            M.arena.resize(h.fe_off + words, 0u);
            uint16_t* fe16 = reinterpret_cast<uint16_t*>(M.arena.data() + h.fe_off);
            for (int32_t i = 0; i < nFl; ++i) {
                int32_t f = lf[i];
                for (int k = 0; k < 3; ++k) {
                    int32_t  e   = fe[3 * f + k];
                    uint16_t dir = (M.ev_in[2 * e] == fv[3 * f + k]) ? 0 : 1;
                    fe16[3 * i + k] = (uint16_t)((eloc[e] << 1) | dir);
                }
            }
        }
        // vertex-normal incidence block: per owned vertex (input VF order)
        // its incident faces' two other corners in the face's cyclic order
        // (the corner after it, then the one before), as local vertex ids
        // packed a | b << 16, behind 32-bit offsets
        {
            const size_t  b0   = M.nrm.size();
            const int32_t offw = pad4(nVo + 1);
            int64_t       ninc = 0;
            for (int32_t i = 0; i < nVo; ++i) ninc += vf_off[lv[i] + 1] - vf_off[lv[i]];
            const int32_t incw = pad4((int32_t)ninc);
            M.nrm.resize(b0 + offw + incw, 0u);
            uint32_t* off = M.nrm.data() + b0;
            uint32_t* vis = off + offw;
            uint32_t  j   = 0;
            for (int32_t i = 0; i < nVo; ++i) {
                off[i] = j;
                for (int32_t t = vf_off[lv[i]]; t < vf_off[lv[i] + 1]; ++t) {
                    const int32_t* c = fv + 3 * (int64_t)vf_val[t];
                    const int      k = c[0] == lv[i] ? 0 : (c[1] == lv[i] ? 1 : 2);
                    vis[j++] = (uint32_t)vloc[c[(k + 1) % 3]] | ((uint32_t)vloc[c[(k + 2) % 3]] << 16);
                }
            }
            off[nVo] = j;
            if (M.nrm.size() > (size_t)INT32_MAX) {
                set_error("vertex-normal incidence tables exceed 2^31 words");
                return RXG_ERR_PATCH_LIMIT;
            }
            M.nrm_off[p + 1] = (int32_t)M.nrm.size();
        }
        h.rv_off = (int32_t)M.arena.size();
        for (int32_t i = nVo; i < nVl; ++i) M.arena.push_back((uint32_t)M.v_i2l[lv[i]]);
        M.arena.resize(h.rv_off + pad4(nVl - nVo), 0u);
        h.re_off = (int32_t)M.arena.size();
        for (int32_t i = nEo; i < nEl; ++i) M.arena.push_back((uint32_t)M.e_i2l[le[i]]);
        M.arena.resize(h.re_off + pad4(nEl - nEo), 0u);
        h.rf_off = (int32_t)M.arena.size();
        for (int32_t i = nFo; i < nFl; ++i) M.arena.push_back((uint32_t)M.f_i2l[lf[i]]);
        M.arena.resize(h.rf_off + pad4(nFl - nFo), 0u);
        if (M.arena.size() > (size_t)INT32_MAX) {
            set_error("mesh topology arena exceeds 2^31 words");
            return RXG_ERR_PATCH_LIMIT;
        }

        M.max_vl = std::max(M.max_vl, nVl);
        M.max_el = std::max(M.max_el, nEl);
        M.max_fl = std::max(M.max_fl, nFl);
        M.max_vo = std::max(M.max_vo, nVo);
        M.max_eo = std::max(M.max_eo, nEo);
        M.max_fo = std::max(M.max_fo, nFo);
        M.ribbon_v += nVl - nVo;
        M.ribbon_f += nFl - nFo;
    }
    (void)nfp;
    if (vv_acc != 2 * ne || vf_acc != 3 * nf || ef_acc != 3 * nf) {
        set_error("internal: value counts %lld/%lld do not match 2E/3F", (long long)vv_acc,
                  (long long)vf_acc);
        return RXG_ERR_INVALID;
    }
    return RXG_OK;
}

static rxg_status upload(Mesh& M)
{
    RXG_CUDA_TRY(cudaGetDevice(&M.device));
    auto up = [&](void** dst, const void* src, size_t bytes) -> rxg_status {
        if (bytes == 0) bytes = 16;
        RXG_CUDA_TRY(cudaMalloc(dst, bytes));
        M.device_bytes += (int64_t)bytes;
        if (src) RXG_CUDA_TRY(cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice));
        return RXG_OK;
    };
    rxg_status s;
    if ((s = up((void**)&M.d.hdr, M.hdr.data(), M.hdr.size() * sizeof(PatchHdr)))) return s;
    M.d.arena_words = (int64_t)M.arena.size();
    if ((s = up((void**)&M.d.arena, M.arena.data(), M.arena.size() * 4))) return s;
    if ((s = up((void**)&M.d.nrm, M.nrm.data(), M.nrm.size() * 4))) return s;
    if ((s = up((void**)&M.d.nrm_off, M.nrm_off.data(), M.nrm_off.size() * 4))) return s;
    {
        std::vector<int32_t> qb(M.ef_base);
        qb.insert(qb.end(), M.ff_base.begin(), M.ff_base.end());
        if ((s = up((void**)&M.d.qbase, qb.data(), qb.size() * 4))) return s;
    }
    if ((s = up((void**)&M.d.v_l2i, M.v_l2i.data(), M.v_l2i.size() * 4))) return s;
    if ((s = up((void**)&M.d.e_l2i, M.e_l2i.data(), M.e_l2i.size() * 4))) return s;
    if ((s = up((void**)&M.d.f_l2i, M.f_l2i.data(), M.f_l2i.size() * 4))) return s;
    return RXG_OK;
}

static void free_device(Mesh& M)
{
    cudaFree(M.d.hdr);
    cudaFree(M.d.arena);
    cudaFree(M.d.nrm);
    cudaFree(M.d.nrm_off);
    cudaFree(M.d.qbase);
    cudaFree(M.d.v_l2i);
    cudaFree(M.d.e_l2i);
    cudaFree(M.d.f_l2i);
    cudaFree(M.d.fv_lin);
    M.d = DeviceTopo{};
    if (M.copy_stream) cudaStreamDestroy(M.copy_stream);
    M.copy_stream = nullptr;
    for (cudaEvent_t& e : M.copy_ev) {
        if (e) cudaEventDestroy(e);
        e = nullptr;
    }
    for (cudaStream_t& q : M.sweep_streams) {
        if (q) cudaStreamDestroy(q);
        q = nullptr;
    }
    for (cudaEvent_t& e : M.sweep_ev) {
        if (e) cudaEventDestroy(e);
        e = nullptr;
    }
}

}  // namespace rxg

using namespace rxg;

extern "C" {

const char* rxg_status_string(rxg_status s)
{
    switch (s) {
        case RXG_OK: return "RXG_OK";
        case RXG_ERR_INVALID: return "RXG_ERR_INVALID";
        case RXG_ERR_NOMEM: return "RXG_ERR_NOMEM";
        case RXG_ERR_CUDA: return "RXG_ERR_CUDA";
        case RXG_ERR_NONMANIFOLD: return "RXG_ERR_NONMANIFOLD";
        case RXG_ERR_PATCH_LIMIT: return "RXG_ERR_PATCH_LIMIT";
        case RXG_ERR_NOT_CONVERGED: return "RXG_ERR_NOT_CONVERGED";
        case RXG_ERR_DEVICE_TIMEOUT: return "RXG_ERR_DEVICE_TIMEOUT";
        case RXG_ERR_UNSUPPORTED: return "RXG_ERR_UNSUPPORTED";
        case RXG_ERR_NO_DEVICE: return "RXG_ERR_NO_DEVICE";
        default: return "RXG_ERR_UNKNOWN";
    }
}

const char* rxg_last_error(void) { return g_msg; }

rxg_status rxg_mesh_create(const int32_t* fv, int64_t nf, int64_t nv, int32_t patch_faces,
                           rxg_mesh** out)
{
    return rxg_mesh_create_ex(fv, nf, nv, patch_faces, 0, out);
}

}  // extern "C"

rxg_status rxg::create_mesh(const int32_t* fv, int64_t nf, int64_t nv, int32_t patch_faces,
                            int32_t flags, const Partition* part, rxg_mesh** out)
{
    if (!out) {
        set_error("rxg_mesh_create: out is NULL");
        return RXG_ERR_INVALID;
    }
    *out = nullptr;
    if (!fv || nf <= 0 || nv <= 0 || nf > (INT32_MAX / 3) || nv >= INT32_MAX) {
        set_error("rxg_mesh_create: need fv != NULL, 0 < nf < 2^31/3, 0 < nv < 2^31");
        return RXG_ERR_INVALID;
    }
    if (!part && (patch_faces < 16 || patch_faces > 4096)) {
        set_error("rxg_mesh_create: patch_faces must be in [16, 4096] (got %d)", patch_faces);
        return RXG_ERR_INVALID;
    }
    for (int64_t i = 0; i < 3 * nf; ++i)
        if (fv[i] < 0 || fv[i] >= nv) {
            set_error("rxg_mesh_create: face %lld references vertex %d outside [0, %lld)",
                      (long long)(i / 3), fv[i], (long long)nv);
            return RXG_ERR_INVALID;
        }
    for (int64_t f = 0; f < nf; ++f)
        if (fv[3 * f] == fv[3 * f + 1] || fv[3 * f + 1] == fv[3 * f + 2] ||
            fv[3 * f] == fv[3 * f + 2]) {
            set_error("rxg_mesh_create: face %lld repeats a vertex", (long long)f);
            return RXG_ERR_INVALID;
        }
    rxg_mesh* h = new (std::nothrow) rxg_mesh();
    if (!h) {
        set_error("rxg_mesh_create: host allocation failed");
        return RXG_ERR_NOMEM;
    }
    rxg_status s;
    try {
        s = build_host(h->m, fv, nf, nv, patch_faces, (flags & RXG_MESH_SPLIT_COMPONENTS) != 0,
                       part, (flags & RXG_MESH_GPU_PATCHER) != 0);
    } catch (const std::bad_alloc&) {
        set_error("rxg_mesh_create: host allocation failed");
        s = RXG_ERR_NOMEM;
    }
    if (s == RXG_OK) compute_smem_table(h->m);
    if (s == RXG_OK && !(flags & RXG_MESH_HOST_ONLY)) {
        // face -> linear vertex ids, face linear order
        std::vector<int32_t> fvl(3 * nf);
        for (int64_t lf = 0; lf < nf; ++lf) {
            int32_t f = h->m.f_l2i[lf];
            for (int k = 0; k < 3; ++k) fvl[3 * lf + k] = h->m.v_i2l[fv[3 * f + k]];
        }
        s = upload(h->m);
        if (s == RXG_OK) {
            cudaError_t e = cudaMalloc(&h->m.d.fv_lin, fvl.size() * 4);
            if (e == cudaSuccess)
                e = cudaMemcpy(h->m.d.fv_lin, fvl.data(), fvl.size() * 4, cudaMemcpyHostToDevice);
            if (e != cudaSuccess) s = cuda_status(e, "upload fv_lin");
            h->m.device_bytes += (int64_t)fvl.size() * 4;
        }
    }
    if (s != RXG_OK) {
        free_device(h->m);
        delete h;
        return s;
    }
    // the host copy of the arena stays for rxg_mesh_patches (introspection)
    *out = h;
    return RXG_OK;
}

extern "C" {

rxg_status rxg_mesh_create_ex(const int32_t* fv, int64_t nf, int64_t nv, int32_t patch_faces,
                              int32_t flags, rxg_mesh** out)
{
    return create_mesh(fv, nf, nv, patch_faces, flags, nullptr, out);
}

rxg_status rxg_mesh_create_partitioned(const int32_t* fv, int64_t nf, int64_t nv,
                                       const int32_t* face_patch, const int32_t* vertex_patch,
                                       const int32_t* edge_patch, int64_t ne, int32_t flags,
                                       rxg_mesh** out)
{
    if (out) *out = nullptr;
    if (!face_patch || (edge_patch && ne < 0) || (flags & RXG_MESH_SPLIT_COMPONENTS)) {
        set_error("rxg_mesh_create_partitioned: need face_patch, ne >= 0 with edge_patch, and "
                  "no RXG_MESH_SPLIT_COMPONENTS");
        return RXG_ERR_INVALID;
    }
    Partition part;
    part.face   = face_patch;
    part.vertex = vertex_patch;
    part.edge   = edge_patch;
    part.ne     = ne;
    return create_mesh(fv, nf, nv, 0, flags, &part, out);
}

void rxg_mesh_destroy(rxg_mesh* h)
{
    if (!h) return;
    lazy_free(&h->m);
    free_device(h->m);
    delete h;
}

rxg_status rxg_mesh_get_info(const rxg_mesh* h, rxg_mesh_info* info)
{
    if (!h || !info) {
        set_error("rxg_mesh_get_info: NULL argument");
        return RXG_ERR_INVALID;
    }
    const Mesh& M          = h->m;
    info->num_vertices     = M.nv;
    info->num_edges        = M.ne;
    info->num_faces        = M.nf;
    info->num_patches      = M.num_patches;
    info->max_valence      = M.max_valence;
    info->is_closed        = M.closed;
    info->is_edge_manifold = M.edge_manifold;
    info->patch_faces      = M.patch_faces;
    info->max_local_vertices = M.max_vl;
    info->max_local_edges    = M.max_el;
    info->max_local_faces    = M.max_fl;
    info->ribbon_vertices    = M.ribbon_v;
    info->ribbon_faces       = M.ribbon_f;
    info->device_bytes       = M.device_bytes;
    info->num_components     = M.num_components;
    info->is_oriented        = M.oriented;
    info->max_edge_incident_faces = M.max_edge_faces;
    info->max_face_adjacent_faces = M.max_face_faces;
    info->num_face_patches   = M.num_face_patches;
    info->lloyd_runs         = M.lloyd_runs;
    return RXG_OK;
}

rxg_status rxg_mesh_device_context(const rxg_mesh* h, rxg_device_context* ctx)
{
    if (!h || !ctx) {
        set_error("rxg_mesh_device_context: NULL argument");
        return RXG_ERR_INVALID;
    }
    const Mesh& M = h->m;
    if (!M.d.hdr || !M.d.arena) {
        set_error("rxg_mesh_device_context: the mesh has no device copy (built host-only)");
        return RXG_ERR_INVALID;
    }
    static_assert(sizeof(PatchHdr) == 16 * sizeof(int32_t), "patch record is 16 int32");
    ctx->num_vertices       = M.nv;
    ctx->num_edges          = M.ne;
    ctx->num_faces          = M.nf;
    ctx->num_patches        = M.num_patches;
    ctx->max_local_vertices = M.max_vl;
    ctx->max_local_edges    = M.max_el;
    ctx->max_local_faces    = M.max_fl;
    ctx->max_owned_vertices = M.max_vo;
    ctx->max_owned_edges    = M.max_eo;
    ctx->max_owned_faces    = M.max_fo;
    ctx->max_valence        = (int32_t)M.max_valence;
    ctx->max_face_adjacent_faces = M.max_face_faces;
    ctx->patch_hdr          = reinterpret_cast<const int32_t*>(M.d.hdr);
    ctx->arena              = M.d.arena;
    ctx->device             = M.device;
    return RXG_OK;
}

rxg_status rxg_mesh_linear_to_input(const rxg_mesh* h, int32_t elem, int32_t* out)
{
    if (!h || !out || elem < 0 || elem > 2) {
        set_error("rxg_mesh_linear_to_input: bad argument");
        return RXG_ERR_INVALID;
    }
    const std::vector<int32_t>& src =
        elem == RXG_ELEM_VERTEX ? h->m.v_l2i : (elem == RXG_ELEM_EDGE ? h->m.e_l2i : h->m.f_l2i);
    std::memcpy(out, src.data(), src.size() * 4);
    return RXG_OK;
}

rxg_status rxg_mesh_patches(const rxg_mesh* h, int32_t* hdr, uint32_t* arena, int64_t* words)
{
    if (!h || !words) {
        set_error("rxg_mesh_patches: bad argument");
        return RXG_ERR_INVALID;
    }
    *words = (int64_t)h->m.arena.size();
    if (hdr) std::memcpy(hdr, h->m.hdr.data(), h->m.hdr.size() * sizeof(PatchHdr));
    if (arena) std::memcpy(arena, h->m.arena.data(), h->m.arena.size() * 4);
    return RXG_OK;
}

rxg_status rxg_mesh_boundary_vertices(const rxg_mesh* h, int8_t* out, void* stream)
{
    if (!h || !out) {
        set_error("rxg_mesh_boundary_vertices: bad argument");
        return RXG_ERR_INVALID;
    }
    const std::vector<int8_t>& b = h->m.vbnd;
    if (!is_device_ptr(out)) {
        std::memcpy(out, b.data(), b.size());
        return RXG_OK;
    }
    // from the host copy: the flags are static topology, kept with the mesh
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t  e = cudaMemcpyAsync(out, b.data(), b.size(), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return e == cudaSuccess ? RXG_OK : cuda_status(e, "rxg_mesh_boundary_vertices");
}

rxg_status rxg_mesh_input_edges(const rxg_mesh* h, int32_t* ev)
{
    if (!h || !ev) {
        set_error("rxg_mesh_input_edges: bad argument");
        return RXG_ERR_INVALID;
    }
    std::memcpy(ev, h->m.ev_in.data(), h->m.ev_in.size() * 4);
    return RXG_OK;
}

}  // extern "C"
