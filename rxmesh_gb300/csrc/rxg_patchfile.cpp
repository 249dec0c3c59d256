// Reproducible partitions: the partition of a mesh in input ids, and RXMesh's
// saved-patcher files (RXMeshStatic(fv, patcher_file), rxmesh_static.h:61-100;
// Patcher::Patcher(filename) and Patcher::save / serialize,
// include/rxmesh/patcher/patcher.cu:25-32, patcher.h:154-181).
//
// The file is a cereal (v1.3.2, the version RXMesh pins in
// cmake/cereal.cmake) PortableBinaryOutputArchive of the Patcher's fields.
// That archive's published layout, restated here: one byte that is 1 when
// the writer was little-endian (the reader swaps bytes when its own order
// differs), then every field in declaration order of serialize() with no
// names or padding -- uint32 scalars as 4 bytes, a std::vector<uint32_t> as
// a uint64 element count followed by its elements, a float as 4 bytes.
// The fields: patch_size, num_patches, num_vertices, num_edges, num_faces,
// num_seeds, max_num_patches, num_components, num_lloyd_run (uint32);
// face_patch, vertex_patch, edge_patch, patches_val, patches_offset,
// ribbon_ext_val, ribbon_ext_offset (vectors); patching_time_ms (float).
// Offsets are inclusive prefix sums (patch p's entries end at offset[p]).
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <utility>
#include <vector>

#include "rxg_internal.h"

using namespace rxg;

namespace {

constexpr uint32_t kInvalid = 0xFFFFFFFFu;

bool host_little_endian()
{
    const uint32_t one = 1;
    unsigned char  b;
    std::memcpy(&b, &one, 1);
    return b == 1;
}

struct Reader {
    const std::vector<unsigned char>& buf;
    size_t                            pos  = 0;
    bool                              swap = false;

    bool take(void* dst, size_t n)
    {
        if (buf.size() - pos < n) return false;
        std::memcpy(dst, buf.data() + pos, n);
        if (swap) {
            unsigned char* d = static_cast<unsigned char*>(dst);
            for (size_t i = 0; i < n / 2; ++i) std::swap(d[i], d[n - 1 - i]);
        }
        pos += n;
        return true;
    }
    bool u32(uint32_t& v) { return take(&v, 4); }
    bool vec(std::vector<uint32_t>& v)
    {
        uint64_t n;
        if (!take(&n, 8) || n > (buf.size() - pos) / 4) return false;
        v.resize((size_t)n);
        for (auto& x : v)
            if (!u32(x)) return false;
        return true;
    }
};

struct Writer {
    std::vector<unsigned char> buf;
    void put(const void* p, size_t n)
    {
        const unsigned char* b = static_cast<const unsigned char*>(p);
        buf.insert(buf.end(), b, b + n);
    }
    void u32(uint32_t v) { put(&v, 4); }
    void vec(const std::vector<uint32_t>& v)
    {
        const uint64_t n = v.size();
        put(&n, 8);
        if (n) put(v.data(), 4 * v.size());
    }
};

// owner patch of every element in input ids: patch p owns linear ids
// [base, base + count) of each kind
void owners(const Mesh& M, int elem, int32_t* out)
{
    const std::vector<int32_t>& l2i =
        elem == RXG_ELEM_VERTEX ? M.v_l2i : (elem == RXG_ELEM_EDGE ? M.e_l2i : M.f_l2i);
    for (int32_t p = 0; p < M.num_patches; ++p) {
        const PatchHdr& h    = M.hdr[p];
        const int32_t   base = elem == RXG_ELEM_VERTEX ? h.v_base : (elem == RXG_ELEM_EDGE ? h.e_base : h.f_base);
        const int32_t   cnt  = elem == RXG_ELEM_VERTEX ? h.nVo : (elem == RXG_ELEM_EDGE ? h.nEo : h.nFo);
        for (int32_t l = base; l < base + cnt; ++l) out[l2i[l]] = p;
    }
}

}  // namespace

extern "C" {

rxg_status rxg_mesh_partition(const rxg_mesh* h, int32_t* face_patch, int32_t* vertex_patch,
                              int32_t* edge_patch)
{
    if (!h) {
        set_error("rxg_mesh_partition: mesh is NULL");
        return RXG_ERR_INVALID;
    }
    if (face_patch) owners(h->m, RXG_ELEM_FACE, face_patch);
    if (vertex_patch) owners(h->m, RXG_ELEM_VERTEX, vertex_patch);
    if (edge_patch) owners(h->m, RXG_ELEM_EDGE, edge_patch);
    return RXG_OK;
}

rxg_status rxg_mesh_create_from_patch_file(const int32_t* fv, int64_t nf, int64_t nv,
                                           const char* patcher_file, int32_t flags,
                                           rxg_mesh** out)
{
    if (out) *out = nullptr;
    if (!patcher_file || !fv || nf <= 0 || nv <= 0 || (flags & RXG_MESH_SPLIT_COMPONENTS)) {
        set_error("rxg_mesh_create_from_patch_file: bad argument");
        return RXG_ERR_INVALID;
    }
    std::vector<unsigned char> buf;
    {
        FILE* fp = std::fopen(patcher_file, "rb");
        if (!fp) {
            set_error("rxg_mesh_create_from_patch_file: cannot open %s", patcher_file);
            return RXG_ERR_INVALID;
        }
        unsigned char chunk[1 << 16];
        size_t        n;
        while ((n = std::fread(chunk, 1, sizeof(chunk), fp)) > 0) buf.insert(buf.end(), chunk, chunk + n);
        std::fclose(fp);
    }
    Reader r{buf};
    if (buf.empty() || buf[0] > 1) {
        set_error("%s: not a portable binary patcher file", patcher_file);
        return RXG_ERR_INVALID;
    }
    r.pos  = 1;
    r.swap = (buf[0] == 1) != host_little_endian();
    uint32_t              hdr[9];
    std::vector<uint32_t> vecs[7];
    float                 ms = 0.f;
    bool                  ok = true;
    for (uint32_t& x : hdr) ok = ok && r.u32(x);
    for (auto& v : vecs) ok = ok && r.vec(v);
    ok = ok && r.take(&ms, 4) && r.pos == buf.size();
    if (!ok) {
        set_error("%s: truncated or malformed patcher file", patcher_file);
        return RXG_ERR_INVALID;
    }
    const uint32_t np = hdr[1], fnv = hdr[2], fne = hdr[3], fnf = hdr[4];
    const auto&    fpatch = vecs[0];
    const auto&    vpatch = vecs[1];
    const auto&    epatch = vecs[2];
    if ((int64_t)fnv != nv || (int64_t)fnf != nf || fpatch.size() != fnf || vpatch.size() != fnv ||
        epatch.size() != fne) {
        set_error("%s: written for %u vertices / %u faces (%zu / %zu / %zu patch ids), the mesh "
                  "has %lld / %lld", patcher_file, fnv, fnf, vpatch.size(), fpatch.size(),
                  epatch.size(), (long long)nv, (long long)nf);
        return RXG_ERR_INVALID;
    }
    std::vector<int32_t> fp32(fpatch.size()), vp32(vpatch.size()), ep32(epatch.size());
    for (size_t i = 0; i < fpatch.size(); ++i) {
        if (fpatch[i] >= np) {
            set_error("%s: face %zu in patch %u of %u", patcher_file, i, fpatch[i], np);
            return RXG_ERR_INVALID;
        }
        fp32[i] = (int32_t)fpatch[i];
    }
    // owners outside [0, np) (RXMesh writes INVALID32 for a vertex in no
    // face) become -1: ignored for vertices in no face, refused otherwise
    for (size_t i = 0; i < vpatch.size(); ++i) vp32[i] = vpatch[i] < np ? (int32_t)vpatch[i] : -1;
    for (size_t i = 0; i < epatch.size(); ++i) ep32[i] = epatch[i] < np ? (int32_t)epatch[i] : -1;
    Partition part;
    part.face       = fp32.data();
    part.vertex     = vp32.data();
    part.edge       = ep32.data();
    part.ne         = (int64_t)fne;
    part.patch_size = (int32_t)std::min<uint32_t>(hdr[0], 4096u);
    return create_mesh(fv, nf, nv, 0, flags, &part, out);
}

rxg_status rxg_mesh_save_patch_file(const rxg_mesh* h, const char* patcher_file)
{
    if (!h || !patcher_file) {
        set_error("rxg_mesh_save_patch_file: bad argument");
        return RXG_ERR_INVALID;
    }
    const Mesh&   M   = h->m;
    const int32_t np  = M.num_face_patches;
    const int64_t nv = M.nv, ne = M.ne, nf = M.nf;
    std::vector<int32_t> fo(nf), vo(nv), eo(ne);
    owners(M, RXG_ELEM_FACE, fo.data());
    owners(M, RXG_ELEM_VERTEX, vo.data());
    owners(M, RXG_ELEM_EDGE, eo.data());

    std::vector<uint32_t> face_patch(fo.begin(), fo.end()), edge_patch(eo.begin(), eo.end());
    std::vector<uint32_t> vertex_patch(nv);
    for (int64_t v = 0; v < nv; ++v) vertex_patch[v] = vo[v] < np ? (uint32_t)vo[v] : kInvalid;
    // patches_val: each patch's faces in linear order; inclusive offsets
    std::vector<uint32_t> patches_val(nf), patches_offset(np);
    for (int64_t l = 0; l < nf; ++l) patches_val[l] = (uint32_t)M.f_l2i[l];
    for (int32_t p = 0; p < np; ++p) patches_offset[p] = (uint32_t)(M.hdr[p].f_base + M.hdr[p].nFo);
    // the external ribbon of RXMesh's patcher (patcher.cu:640-716): for each
    // face of the patch in patches_val order, each of its vertices, each face
    // at that vertex (in face order) owned by another patch, first occurrence
    std::vector<int32_t> vf_off(nv + 1, 0), vf_val(3 * nf);
    for (int64_t i = 0; i < 3 * nf; ++i) vf_off[M.fv_in[i] + 1]++;
    for (int64_t v = 0; v < nv; ++v) vf_off[v + 1] += vf_off[v];
    {
        std::vector<int32_t> cur(vf_off.begin(), vf_off.end() - 1);
        for (int64_t f = 0; f < nf; ++f)
            for (int k = 0; k < 3; ++k) vf_val[cur[M.fv_in[3 * f + k]]++] = (int32_t)f;
    }
    std::vector<uint32_t> ribbon_val, ribbon_offset(np);
    std::vector<int32_t>  stamp(nf, -1);
    for (int32_t p = 0; p < np; ++p) {
        const int32_t b = M.hdr[p].f_base, e = b + M.hdr[p].nFo;
        for (int32_t l = b; l < e; ++l) {
            const int32_t f = M.f_l2i[l];
            for (int k = 0; k < 3; ++k) {
                const int32_t v = M.fv_in[3 * f + k];
                for (int32_t t = vf_off[v]; t < vf_off[v + 1]; ++t) {
                    const int32_t g = vf_val[t];
                    if (fo[g] != p && stamp[g] != p) {
                        stamp[g] = p;
                        ribbon_val.push_back((uint32_t)g);
                    }
                }
            }
        }
        ribbon_offset[p] = (uint32_t)ribbon_val.size();
    }

    Writer w;
    const unsigned char endian = host_little_endian() ? 1 : 0;
    w.put(&endian, 1);
    const uint32_t hdr[9] = {(uint32_t)M.patch_faces, (uint32_t)np, (uint32_t)nv, (uint32_t)ne,
                             (uint32_t)nf, (uint32_t)np, (uint32_t)np,
                             (uint32_t)M.num_components, 0u};
    for (uint32_t x : hdr) w.u32(x);
    w.vec(face_patch);
    w.vec(vertex_patch);
    w.vec(edge_patch);
    w.vec(patches_val);
    w.vec(patches_offset);
    w.vec(ribbon_val);
    w.vec(ribbon_offset);
    const float ms = 0.f;
    w.put(&ms, 4);

    FILE* fp = std::fopen(patcher_file, "wb");
    if (!fp) {
        set_error("rxg_mesh_save_patch_file: cannot create %s", patcher_file);
        return RXG_ERR_INVALID;
    }
    const bool written = std::fwrite(w.buf.data(), 1, w.buf.size(), fp) == w.buf.size();
    if (std::fclose(fp) != 0 || !written) {
        set_error("rxg_mesh_save_patch_file: write to %s failed", patcher_file);
        return RXG_ERR_INVALID;
    }
    return RXG_OK;
}

}  // extern "C"
