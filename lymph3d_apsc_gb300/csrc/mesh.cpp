// mesh.cpp -- host-side mesh set-up (see include/lymph3d_mesh.h).
//
// Integer/graph work done once before the device set-up: cube generation,
// hashed face matching (the reference scans all faces for every face,
// src/MAKE_PARTITION_AND_MPI_FILES.f90:2536-2580), boundary tagging and the
// grouping of tetrahedra into polyhedra.

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <deque>
#include <unordered_map>
#include <vector>

#include "../../include/lymph3d_gpu.h"
#include "../../include/lymph3d_mesh.h"

namespace {

// Vertex triples of the 4 faces, reference numbering
// (MAKE_PARTITION_AND_MPI_FILES.f90:1087-1096), 0-based.
const int FACE_V[4][3] = {{0, 1, 2}, {0, 1, 3}, {1, 2, 3}, {2, 0, 3}};

struct TripleHash {
    size_t operator()(const std::array<int32_t, 3>& k) const {
        uint64_t h = (uint64_t)(uint32_t)k[0] * 0x9E3779B97F4A7C15ull;
        h ^= (uint64_t)(uint32_t)k[1] + 0x7F4A7C159E3779B9ull + (h << 6) + (h >> 2);
        h ^= (uint64_t)(uint32_t)k[2] * 0xC2B2AE3D27D4EB4Full + (h << 6) + (h >> 2);
        return (size_t)h;
    }
};

std::array<int32_t, 3> face_key(const int32_t* tv, int t, int f) {
    std::array<int32_t, 3> k = {tv[t * 4 + FACE_V[f][0]], tv[t * 4 + FACE_V[f][1]], tv[t * 4 + FACE_V[f][2]]};
    std::sort(k.begin(), k.end());
    return k;
}

uint64_t splitmix64(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

double det3x3(const double a[3], const double b[3], const double c[3]) {
    return a[0] * (b[1] * c[2] - b[2] * c[1]) - a[1] * (b[0] * c[2] - b[2] * c[0]) + a[2] * (b[0] * c[1] - b[1] * c[0]);
}

}  // namespace

extern "C" {

int lymph_mesh_cube_sizes(int32_t nx, int32_t ny, int32_t nz, int32_t* n_node, int32_t* n_tet) {
    if (nx < 1 || ny < 1 || nz < 1) return LYMPH_ERR_INVALID;
    int64_t nn = (int64_t)(nx + 1) * (ny + 1) * (nz + 1), nt = (int64_t)6 * nx * ny * nz;
    if (nt > INT32_MAX / 4) return LYMPH_ERR_INVALID;
    if (n_node) *n_node = (int32_t)nn;
    if (n_tet) *n_tet = (int32_t)nt;
    return LYMPH_OK;
}

int lymph_mesh_cube(int32_t nx, int32_t ny, int32_t nz, double* coords, int32_t* tet_vert, int32_t* face_tag) {
    int32_t nn, nt;
    int rc = lymph_mesh_cube_sizes(nx, ny, nz, &nn, &nt);
    if (rc) return rc;
    auto node = [&](int i, int j, int k) { return (int32_t)(i + (nx + 1) * (j + (ny + 1) * k)); };
    for (int k = 0; k <= nz; ++k)
        for (int j = 0; j <= ny; ++j)
            for (int i = 0; i <= nx; ++i) {
                int32_t id = node(i, j, k);
                coords[id * 3 + 0] = (double)i / nx;
                coords[id * 3 + 1] = (double)j / ny;
                coords[id * 3 + 2] = (double)k / nz;
            }
    static const int PERM[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
    int64_t t = 0;
    for (int c = 0; c < nz; ++c)
        for (int b = 0; b < ny; ++b)
            for (int a = 0; a < nx; ++a)
                for (int p = 0; p < 6; ++p) {
                    int cur[3] = {a, b, c};
                    int32_t v[4];
                    v[0] = node(cur[0], cur[1], cur[2]);
                    for (int s = 0; s < 3; ++s) {
                        cur[PERM[p][s]] += 1;
                        v[s + 1] = node(cur[0], cur[1], cur[2]);
                    }
                    double e[3][3];
                    for (int s = 0; s < 3; ++s)
                        for (int d = 0; d < 3; ++d) e[s][d] = coords[v[s + 1] * 3 + d] - coords[v[0] * 3 + d];
                    if (det3x3(e[0], e[1], e[2]) < 0) std::swap(v[1], v[2]);
                    for (int s = 0; s < 4; ++s) tet_vert[t * 4 + s] = v[s];
                    ++t;
                }
    if (face_tag) {
        for (int64_t tt = 0; tt < nt; ++tt)
            for (int f = 0; f < 4; ++f) {
                int tag = 0;
                int32_t w[3] = {tet_vert[tt * 4 + FACE_V[f][0]], tet_vert[tt * 4 + FACE_V[f][1]], tet_vert[tt * 4 + FACE_V[f][2]]};
                auto all = [&](int d, double val) {
                    for (int s = 0; s < 3; ++s)
                        if (coords[w[s] * 3 + d] != val) return false;
                    return true;
                };
                if (all(2, 0.0)) tag = 2;
                else if (all(2, 1.0)) tag = 3;
                else if (all(0, 1.0)) tag = 4;
                else if (all(1, 1.0)) tag = 5;
                else if (all(0, 0.0)) tag = 6;
                else if (all(1, 0.0)) tag = 7;
                face_tag[tt * 4 + f] = tag;
            }
    }
    return LYMPH_OK;
}

int lymph_mesh_match_faces(int32_t n_tet, const int32_t* tv, int32_t* neigh, int32_t* neigh_face) {
    if (n_tet < 0 || (n_tet > 0 && (!tv || !neigh))) return LYMPH_ERR_INVALID;
    std::unordered_map<std::array<int32_t, 3>, int64_t, TripleHash> open;
    open.reserve((size_t)n_tet * 2 + 16);
    for (int64_t i = 0; i < (int64_t)n_tet * 4; ++i) {
        neigh[i] = LYMPH_MESH_UNMATCHED;
        if (neigh_face) neigh_face[i] = -1;
    }
    for (int32_t t = 0; t < n_tet; ++t)
        for (int f = 0; f < 4; ++f) {
            auto k = face_key(tv, t, f);
            auto it = open.find(k);
            if (it == open.end()) {
                open.emplace(k, (int64_t)t * 4 + f);
            } else {
                int64_t other = it->second;
                if (other < 0) return LYMPH_EXIT_NEIGHBOUR_EL_ERROR;  // third face on one triangle
                int32_t t2 = (int32_t)(other / 4), f2 = (int32_t)(other % 4);
                neigh[t * 4 + f] = t2;
                neigh[t2 * 4 + f2] = t;
                if (neigh_face) { neigh_face[t * 4 + f] = f2; neigh_face[t2 * 4 + f2] = f; }
                it->second = -1;
            }
        }
    return LYMPH_OK;
}

int lymph_mesh_tag_boundary(int32_t n_tet, const int32_t* tv, int32_t n_tri, const int32_t* tri_vert,
                            const int32_t* tri_tag, int32_t* face_tag, int32_t* n_unfound) {
    if (n_tet < 0 || n_tri < 0) return LYMPH_ERR_INVALID;
    std::unordered_map<std::array<int32_t, 3>, int32_t, TripleHash> tags;
    tags.reserve((size_t)n_tri * 2 + 16);
    for (int32_t i = 0; i < n_tri; ++i) {
        std::array<int32_t, 3> k = {tri_vert[i * 3], tri_vert[i * 3 + 1], tri_vert[i * 3 + 2]};
        std::sort(k.begin(), k.end());
        tags[k] = tri_tag[i];
    }
    int32_t found = 0;
    for (int32_t t = 0; t < n_tet; ++t)
        for (int f = 0; f < 4; ++f) {
            auto it = tags.find(face_key(tv, t, f));
            face_tag[t * 4 + f] = (it == tags.end()) ? 0 : it->second;
            if (it != tags.end()) ++found;
        }
    if (n_unfound) *n_unfound = n_tri - found > 0 ? n_tri - found : 0;
    return LYMPH_OK;
}

int lymph_mesh_apply_bc(int32_t n_tet, const int32_t* face_tag, int32_t mode, int32_t* neigh, int32_t* fun_tag) {
    if (n_tet < 0 || !face_tag || !neigh) return LYMPH_ERR_INVALID;
    for (int64_t i = 0; i < (int64_t)n_tet * 4; ++i) {
        int tag = face_tag[i];
        if (fun_tag) fun_tag[i] = 0;
        if (neigh[i] >= 0) continue;
        if (tag == 0) return LYMPH_EXIT_SETUP;
        int bc = LYMPH_BC_NEUM;
        if (tag == 2 || tag == 3 || tag == 4 || mode == LYMPH_BCMODE_ALL_DIRICHLET) bc = LYMPH_BC_DIRI;
        neigh[i] = bc;
        if (fun_tag) fun_tag[i] = (tag >= 2 && tag <= 4) ? tag - 1 : ((tag >= 5 && tag <= 7) ? tag - 4 : 1);
    }
    return LYMPH_OK;
}

int lymph_mesh_agglomerate(int32_t n_tet, const int32_t* neigh, uint64_t seed, int32_t min_size, int32_t max_size,
                           int32_t* tet_poly, int32_t* n_poly) {
    if (n_tet < 0 || min_size < 1 || max_size < min_size || !tet_poly || !n_poly) return LYMPH_ERR_INVALID;
    std::vector<int32_t> grp(n_tet, -1);
    std::vector<int32_t> gsize;
    uint64_t s = seed;
    std::deque<int32_t> q;
    for (int32_t t0 = 0; t0 < n_tet; ++t0) {
        if (grp[t0] >= 0) continue;
        int32_t target = min_size + (int32_t)(splitmix64(s) % (uint64_t)(max_size - min_size + 1));
        int32_t g = (int32_t)gsize.size();
        gsize.push_back(0);
        q.clear();
        q.push_back(t0);
        grp[t0] = g;
        while (!q.empty() && gsize[g] < target) {
            int32_t t = q.front();
            q.pop_front();
            if (grp[t] != g) continue;
            gsize[g]++;
            for (int f = 0; f < 4 && (int32_t)(gsize[g] + q.size()) < target; ++f) {
                int32_t n = neigh[t * 4 + f];
                if (n >= 0 && grp[n] < 0) { grp[n] = g; q.push_back(n); }
            }
        }
        // tets queued but not absorbed return to the pool
        for (int32_t t : q)
            if (grp[t] == g) grp[t] = -1;
        // count exactly
    }
    // recount sizes (queue bookkeeping above counts absorbed tets only)
    std::fill(gsize.begin(), gsize.end(), 0);
    for (int32_t t = 0; t < n_tet; ++t) {
        if (grp[t] < 0) return LYMPH_EXIT_SETUP;  // cannot happen: every tet starts or joins a group
        gsize[grp[t]]++;
    }
    // merge groups below min_size into the smallest adjacent group; the merged
    // size stays below max_size + min_size (a straggler has < min_size tets)
    const int32_t merge_cap = max_size + min_size - 1;
    int ng = (int)gsize.size();
    std::vector<int32_t> parent(ng);
    for (int g = 0; g < ng; ++g) parent[g] = g;
    auto find = [&](int32_t g) { while (parent[g] != g) g = parent[g] = parent[parent[g]]; return g; };
    std::vector<std::vector<int32_t>> members(ng);
    for (int32_t t = 0; t < n_tet; ++t) members[grp[t]].push_back(t);
    for (int g = 0; g < ng; ++g) {
        int rg = find(g);
        if (rg != g || gsize[g] >= min_size) continue;
        int best = -1;
        for (int32_t t : members[g])
            for (int f = 0; f < 4; ++f) {
                int32_t n = neigh[t * 4 + f];
                if (n < 0) continue;
                int h = find(grp[n]);
                if (h == g) continue;
                if (gsize[h] + gsize[g] > merge_cap) continue;
                if (best < 0 || gsize[h] < gsize[best]) best = h;
            }
        if (best >= 0) {
            parent[g] = best;
            gsize[best] += gsize[g];
            for (int32_t t : members[g]) members[best].push_back(t);
            members[g].clear();
            gsize[g] = 0;
        }
    }
    // number polyhedra by first tetrahedron
    std::vector<int32_t> id(ng, -1);
    int32_t np = 0;
    for (int32_t t = 0; t < n_tet; ++t) {
        int r = find(grp[t]);
        if (id[r] < 0) id[r] = np++;
        tet_poly[t] = id[r];
    }
    *n_poly = np;
    return LYMPH_OK;
}

int lymph_mesh_agglomerate_hex(int32_t n_tet, int32_t* tet_poly, int32_t* n_poly) {
    if (n_tet < 0 || n_tet % 6 != 0 || !tet_poly || !n_poly) return LYMPH_ERR_INVALID;
    for (int32_t t = 0; t < n_tet; ++t) tet_poly[t] = t / 6;
    *n_poly = n_tet / 6;
    return LYMPH_OK;
}

int lymph_mesh_find_tet(int32_t n_tet, const int32_t* tv, const double* X, const double* pt, int32_t* tet) {
    if (n_tet <= 0 || !tv || !X || !pt || !tet) return LYMPH_ERR_INVALID;
    int32_t best = -1, nearest = 0;
    double best_min = -1e300, dmin = 1e300;
    for (int32_t t = 0; t < n_tet; ++t) {
        const double* a = &X[tv[t * 4] * 3];
        double e[3][3], r[3];
        for (int s = 0; s < 3; ++s)
            for (int d = 0; d < 3; ++d) e[s][d] = X[tv[t * 4 + s + 1] * 3 + d] - a[d];
        for (int d = 0; d < 3; ++d) r[d] = pt[d] - a[d];
        double det = det3x3(e[0], e[1], e[2]);
        // barycentric coordinates by Cramer's rule on [e0 e1 e2] l = r
        double l1 = det3x3(r, e[1], e[2]) / det, l2 = det3x3(e[0], r, e[2]) / det, l3 = det3x3(e[0], e[1], r) / det;
        double l0 = 1.0 - l1 - l2 - l3;
        double mn = std::min(std::min(l0, l1), std::min(l2, l3));
        if (mn > best_min) { best_min = mn; best = t; }
        double c[3] = {0, 0, 0};
        for (int s = 0; s < 4; ++s)
            for (int d = 0; d < 3; ++d) c[d] += 0.25 * X[tv[t * 4 + s] * 3 + d];
        double dd = (c[0] - pt[0]) * (c[0] - pt[0]) + (c[1] - pt[1]) * (c[1] - pt[1]) + (c[2] - pt[2]) * (c[2] - pt[2]);
        if (dd < dmin) { dmin = dd; nearest = t; }
    }
    *tet = (best_min >= -1e-12) ? best : nearest;
    return LYMPH_OK;
}

}  // extern "C"
