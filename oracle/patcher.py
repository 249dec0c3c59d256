"""numpy restatement of the library's GPU patcher (rxg_patcher.cu), which
follows RXMesh's Lloyd patcher: Patcher::initialize_random_seeds
(include/rxmesh/patcher/patcher.cu:431-535), Patcher::run_lloyd
(patcher.cu:828-960) and its kernels cluster_seed_propagation, interior and
add_more_seeds (patcher_kernel.cuh:57-300), with the library's deterministic
tie rules: a face reached by several regions in one level goes to the lowest
region id, the new seed of a region is its deepest face from the region's
boundary (lowest face id among equals), the split seed of a region over P
faces is its largest-id boundary face (its largest face without boundary),
and the seed generator is splitmix64 from a fixed state.

TEST INFRASTRUCTURE ONLY: the GPU partition must equal lloyd_partition()
face for face.  Pure numpy and scipy, sized for meshes of a few thousand
faces.
"""
import numpy as np

_M64 = (1 << 64) - 1
_FAR = 1 << 40


def face_graph(fv):
    """Face-face adjacency through shared edges (CSR, neighbours in the
    order edge k = (fv[f][k], fv[f][k+1]), then the edge's faces in face
    order) and each face's component as its smallest face id."""
    fv = np.asarray(fv, np.int64)
    nf = len(fv)
    eid, faces_of = {}, []
    fe = np.zeros((nf, 3), np.int64)
    for f in range(nf):
        for k in range(3):
            a, b = int(fv[f, k]), int(fv[f, (k + 1) % 3])
            key = (min(a, b), max(a, b))
            if key not in eid:
                eid[key] = len(faces_of)
                faces_of.append([])
            fe[f, k] = eid[key]
            faces_of[eid[key]].append(f)
    rows = [[g for k in range(3) for g in faces_of[fe[f, k]] if g != f] for f in range(nf)]
    off = np.zeros(nf + 1, np.int64)
    off[1:] = np.cumsum([len(r) for r in rows])
    val = np.array([g for r in rows for g in r], np.int64)
    import scipy.sparse as sp
    import scipy.sparse.csgraph as cg
    _, lab = cg.connected_components(sp.csr_matrix((np.ones(len(val)), val, off), shape=(nf, nf)))
    root = np.full(lab.max() + 1, nf)
    np.minimum.at(root, lab, np.arange(nf))
    return off, val, root[lab]


def _splitmix(state):
    state = (state + 0x9E3779B97F4A7C15) & _M64
    z = state
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _M64
    return state, z ^ (z >> 31)


def initial_seeds(comp, P):
    nf = len(comp)
    total = (nf + P - 1) // P
    state = 0x5EED5EED
    seeds = []
    for r in np.unique(comp):  # components by smallest face id
        m = list(np.nonzero(comp == r)[0])
        n = len(m)
        k = min(n, max(1, int(n * total / nf + 0.5)))
        for i in range(k):
            state, z = _splitmix(state)
            j = i + z % (n - i)
            m[i], m[j] = m[j], m[i]
            seeds.append(int(m[i]))
    return seeds


def lloyd_partition(fv, P, max_runs=200):
    """(face_patch, runs): regions of at most P faces."""
    off, val, comp = face_graph(fv)
    nf = len(comp)
    src = np.repeat(np.arange(nf), np.diff(off))
    seeds = initial_seeds(comp, P)
    for run in range(1, max_runs + 1):
        npatch = len(seeds)
        fp = np.full(nf, -1, np.int64)
        fp[seeds] = np.arange(npatch)
        front = np.array(seeds)
        while len(front):                      # grow, one face ring per level
            sel = np.isin(src, front)
            s, t = src[sel], val[sel]
            free = fp[t] < 0
            s, t = s[free], t[free]
            claim = np.full(nf, _FAR)
            np.minimum.at(claim, t, fp[s])
            front = np.unique(t)
            fp[front] = claim[front]
        sizes = np.bincount(fp, minlength=npatch)
        if sizes.max() <= P:
            return fp.astype(np.int32), run
        bnd = np.zeros(nf, bool)               # faces next to another region
        np.logical_or.at(bnd, src, fp[src] != fp[val])
        depth = np.where(bnd, 0, _FAR)
        front, level = np.nonzero(bnd)[0], 0
        while len(front):                      # inward depth from the boundary
            sel = np.isin(src, front)
            s, t = src[sel], val[sel]
            t = np.unique(t[(fp[t] == fp[s]) & (depth[t] == _FAR)])
            depth[t] = level + 1
            front, level = t, level + 1
        bi = np.nonzero(bnd)[0]
        max_bnd = np.full(npatch, -1)
        np.maximum.at(max_bnd, fp[bi], bi)
        fin = depth < _FAR
        key = depth * (1 << 32) + ((1 << 32) - 1 - np.arange(nf))
        best = np.zeros(npatch, np.int64)
        np.maximum.at(best, fp[fin], key[fin])
        seeds = [(1 << 32) - 1 - (int(best[p]) & 0xFFFFFFFF) if best[p] else seeds[p]
                 for p in range(npatch)]
        if run % 5 == 0:                       # split the regions over P faces
            for p in range(npatch):
                if sizes[p] <= P:
                    continue
                s = int(max_bnd[p]) if max_bnd[p] >= 0 else int(np.nonzero(fp == p)[0].max())
                if s != seeds[p]:
                    seeds.append(s)
    raise RuntimeError("no partition within %d runs" % max_runs)
