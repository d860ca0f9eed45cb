// host_tables.cpp — init-time precompute of the PD-IPC cloth step.
//
// Follows, per cloth model, PdIpcClothModel::init (Simulator/PD-IPC/PdIpcClothModel.h:142-343),
// the boundary topology of PdIpcModel::postProcessBoundaryInfo (PdIpcModel.h:84-172),
// the grid collision patches of PdIpcClothModel::setCollisionPatches (:45-140),
// the system assembly of PdIpcSimulator::setupHessMat (PdIpcSimulator.cpp:270-414)
// and the patch lists of gpuCollisionInit (cpp:1151-1300).  Everything is
// computed in FP64 with a fixed summation order and rounded to the working
// precision at upload; the patch partition alone is computed in FP32 as the
// reference does (qeal = float), so it is the same in every precision mode.
#include "host_tables.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <limits>
#include <utility>

namespace pdipc {

namespace {

inline uint64_t edge_key(int a, int b) {
    if (a > b) std::swap(a, b);
    return ((uint64_t)(uint32_t)a << 32) | (uint32_t)b;
}

int find_edge(const std::vector<uint64_t>& keys, int a, int b) {
    uint64_t k = edge_key(a, b);
    auto it = std::lower_bound(keys.begin(), keys.end(), k);
    return (it != keys.end() && *it == k) ? (int)(it - keys.begin()) : -1;
}

// Grid patch index of every face, or -1 if its centroid falls outside every
// cell.  The reference scans the len x len cells in row-major order and takes
// the first closed cell holding the centroid; the same cell is found here from
// the floor estimate by checking its neighbours in that order.
void grid_patches(const double* X, int nv, const int* F, int nf, int patch_dim,
                  std::vector<std::vector<int>>& patches) {
    const float inf = std::numeric_limits<float>::infinity();
    float lo[3] = {inf, inf, inf}, hi[3] = {-inf, -inf, -inf};
    for (int i = 0; i < nv; ++i)
        for (int k = 0; k < 3; ++k) {
            float p = (float)X[3 * i + k];
            lo[k] = std::min(lo[k], p);
            hi[k] = std::max(hi[k], p);
        }
    float sq = std::sqrt((float)nv);
    int len = (int)(sq < (float)patch_dim ? sq : (float)patch_dim);
    if (len < 1) len = 1;
    float ext[3] = {hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]};
    // normal axis: the strictly thinnest one; on a tie (where the reference
    // leaves the pair uninitialised) the last axis of minimum extent.
    int nrm = -1;
    for (int k = 0; k < 3; ++k)
        if (ext[k] < ext[(k + 1) % 3] && ext[k] < ext[(k + 2) % 3]) nrm = k;
    if (nrm < 0) {
        float m = std::min(ext[0], std::min(ext[1], ext[2]));
        for (int k = 0; k < 3; ++k)
            if (ext[k] == m) nrm = k;
    }
    const int u = (nrm == 0) ? 1 : 0;
    const int v = (nrm == 2) ? 1 : 2;
    const float su = ext[u] / (float)len, sv = ext[v] / (float)len;
    auto in_cell = [](float c, float b0, float s) {
        float b1 = b0 + s;
        return c >= b0 && c <= b1;
    };
    std::vector<std::vector<int>> cells((size_t)len * len);
    for (int f = 0; f < nf; ++f) {
        float c[3] = {0.f, 0.f, 0.f};
        for (int k = 0; k < 3; ++k)
            for (int a = 0; a < 3; ++a) c[a] += (float)X[3 * F[3 * f + k] + a];
        for (int a = 0; a < 3; ++a) c[a] /= 3.f;
        auto first_index = [&](float cv, float lo0, float s) -> int {
            int guess = (s > 0.f) ? (int)std::floor((cv - lo0) / s) : 0;
            int start = std::max(0, std::min(len - 1, guess) - 1);
            for (int r = start; r < len && r <= guess + 1; ++r)
                if (in_cell(cv, lo0 + (float)r * s, s)) return r;
            return -1;
        };
        int r = first_index(c[u], lo[u], su);
        if (r < 0) continue;
        int cc = first_index(c[v], lo[v], sv);
        if (cc < 0) continue;
        cells[(size_t)r * len + cc].push_back(f);
    }
    patches.clear();
    for (auto& cl : cells)
        if (!cl.empty()) patches.push_back(std::move(cl));
}

// Volumetric models: a patch_dim^3 grid over the box of the boundary points,
// each boundary face in the first closed cell (x-major, then y, then z) that
// holds its centroid (PdIpcVolumetricModel::setCollisionPatches,
// PdIpcVolumetricModel.h:114-182; FP32 as the reference).  The first cell of
// a product of per-axis interval tests is the per-axis first index.
void grid3_patches(const double* X, int nv, const int* F, int nf, int patch_dim,
                   std::vector<std::vector<int>>& patches) {
    const float inf = std::numeric_limits<float>::infinity();
    float lo[3] = {inf, inf, inf}, hi[3] = {-inf, -inf, -inf};
    std::vector<char> on(nv, 0);
    for (int q = 0; q < 3 * nf; ++q) on[F[q]] = 1;
    for (int i = 0; i < nv; ++i)
        if (on[i])
            for (int k = 0; k < 3; ++k) {
                float p = (float)X[3 * i + k];
                lo[k] = std::min(lo[k], p);
                hi[k] = std::max(hi[k], p);
            }
    const int len = std::max(1, patch_dim);
    float step[3];
    for (int k = 0; k < 3; ++k) step[k] = (hi[k] - lo[k]) / (float)len;
    auto first_index = [&](float cv, float lo0, float s) -> int {
        int guess = (s > 0.f) ? (int)std::floor((cv - lo0) / s) : 0;
        int start = std::max(0, std::min(len - 1, guess) - 1);
        for (int r = start; r < len && r <= guess + 1; ++r) {
            const float b0 = lo0 + (float)r * s, b1 = b0 + s;
            if (cv >= b0 && cv <= b1) return r;
        }
        return -1;
    };
    std::vector<std::vector<int>> cells((size_t)len * len * len);
    for (int f = 0; f < nf; ++f) {
        float c[3] = {0.f, 0.f, 0.f};
        for (int k = 0; k < 3; ++k)
            for (int a = 0; a < 3; ++a) c[a] += (float)X[3 * F[3 * f + k] + a];
        for (int a = 0; a < 3; ++a) c[a] /= 3.f;
        int id[3];
        bool ok = true;
        for (int a = 0; a < 3 && ok; ++a) ok = (id[a] = first_index(c[a], lo[a], step[a])) >= 0;
        if (ok) cells[((size_t)id[0] * len + id[1]) * len + id[2]].push_back(f);
    }
    patches.clear();
    for (auto& cl : cells)
        if (!cl.empty()) patches.push_back(std::move(cl));
}

std::string build_topology(const double* X, int nv, const int* F, int nf, int patch_dim, bool volumetric,
                           MeshTopology& t);

}  // namespace

std::string build_mesh_topology(const double* X, int nv, const int* F, int nf, int patch_dim, MeshTopology& t) {
    return build_topology(X, nv, F, nf, patch_dim, false, t);
}

std::string tet_boundary_faces(const double* X, int nv, const int* T, int nt, std::vector<int>& faces) {
    static const int kFace[4][3] = {{3, 1, 0}, {3, 2, 1}, {3, 0, 2}, {2, 1, 0}};  // PdIpcVolumetricModel.h:32-36
    struct Rec {
        std::array<int, 3> key;
        int f[3];
        int tet;
    };
    std::vector<Rec> recs;
    recs.reserve(4 * (size_t)nt);
    for (int e = 0; e < nt; ++e) {
        for (int q = 0; q < 4; ++q)
            if (T[4 * e + q] < 0 || T[4 * e + q] >= nv) return "tet index out of range";
        for (int k = 0; k < 4; ++k) {
            Rec r;
            for (int j = 0; j < 3; ++j) r.f[j] = T[4 * e + kFace[k][j]];
            r.key = {r.f[0], r.f[1], r.f[2]};
            std::sort(r.key.begin(), r.key.end());
            r.tet = e;
            recs.push_back(r);
        }
    }
    std::stable_sort(recs.begin(), recs.end(), [](const Rec& a, const Rec& b) { return a.key < b.key; });
    faces.clear();
    for (size_t a = 0; a < recs.size();) {
        size_t b = a;
        while (b < recs.size() && recs[b].key == recs[a].key) ++b;
        if (b - a == 1) {
            const Rec& r = recs[a];
            auto P = [&](int i, int k) { return X[3 * i + k]; };
            double cent[3] = {0, 0, 0}, fc[3] = {0, 0, 0};
            for (int k = 0; k < 3; ++k) {
                for (int q = 0; q < 4; ++q) cent[k] += P(T[4 * r.tet + q], k) / 4.0;
                for (int q = 0; q < 3; ++q) fc[k] += P(r.f[q], k) / 3.0;
            }
            double u[3], v[3];
            for (int k = 0; k < 3; ++k) {
                u[k] = P(r.f[1], k) - P(r.f[0], k);
                v[k] = P(r.f[2], k) - P(r.f[0], k);
            }
            const double n[3] = {u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2], u[0] * v[1] - u[1] * v[0]};
            const double dot = n[0] * (cent[0] - fc[0]) + n[1] * (cent[1] - fc[1]) + n[2] * (cent[2] - fc[2]);
            if (dot > 0) faces.insert(faces.end(), {r.f[0], r.f[2], r.f[1]});
            else faces.insert(faces.end(), {r.f[0], r.f[1], r.f[2]});
        }
        a = b;
    }
    if (faces.empty()) return "tetrahedral mesh has no boundary face";
    return "";
}

namespace {

std::string build_topology(const double* X, int nv, const int* F, int nf, int patch_dim, bool volumetric,
                           MeshTopology& t) {
    if (nv <= 0 || nf <= 0) return "empty mesh";
    for (int i = 0; i < 3 * nf; ++i)
        if (F[i] < 0 || F[i] >= nv) return "face index out of range";
    // edges: sorted unique (min,max) pairs (Model/TriangleMesh/BaseSurfaceMesh.cpp:219-234)
    std::vector<uint64_t> keys;
    keys.reserve(3 * (size_t)nf);
    for (int f = 0; f < nf; ++f)
        for (int k = 0; k < 3; ++k) keys.push_back(edge_key(F[3 * f + k], F[3 * f + (k + 1) % 3]));
    std::sort(keys.begin(), keys.end());
    keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
    const int ne = (int)keys.size();
    t.edges.resize(2 * (size_t)ne);
    t.point_edges.assign(nv, {});
    for (int e = 0; e < ne; ++e) {
        int a = (int)(keys[e] >> 32), b = (int)(keys[e] & 0xffffffffu);
        t.edges[2 * e] = a;
        t.edges[2 * e + 1] = b;
        t.point_edges[a].push_back(e);
        t.point_edges[b].push_back(e);
    }
    // edge -> faces, point -> faces, ascending face id
    t.edge_faces.assign(ne, {});
    std::vector<std::vector<int>> point_faces(nv);
    std::vector<int> face_edge(3 * (size_t)nf);  // edges (01, 12, 20) of each face
    for (int f = 0; f < nf; ++f) {
        for (int k = 0; k < 3; ++k) {
            int e = find_edge(keys, F[3 * f + k], F[3 * f + (k + 1) % 3]);
            face_edge[3 * f + k] = e;
            t.edge_faces[e].push_back(f);
            point_faces[F[3 * f + k]].push_back(f);
        }
    }
    // ownership: smallest current owned list wins, first on ties (PdIpcModel.h:136-171)
    t.face_edges_own.assign(nf, {});
    for (int e = 0; e < ne; ++e) {
        const auto& fl = t.edge_faces[e];
        int best = fl[0];
        for (size_t q = 1; q < fl.size(); ++q)
            if (t.face_edges_own[fl[q]].size() < t.face_edges_own[best].size()) best = fl[q];
        t.face_edges_own[best].push_back(e);
    }
    t.face_points_own.assign(nf, {});
    for (int p = 0; p < nv; ++p) {
        const auto& fl = point_faces[p];
        if (fl.empty()) {
            if (volumetric) continue;  // interior node of a tetrahedral mesh: not on the surface
            return "mesh has an isolated vertex";
        }
        int best = fl[0];
        for (size_t q = 1; q < fl.size(); ++q)
            if (t.face_points_own[fl[q]].size() < t.face_points_own[best].size()) best = fl[q];
        t.face_points_own[best].push_back(p);
    }
    if (volumetric) grid3_patches(X, nv, F, nf, patch_dim, t.patches);
    else grid_patches(X, nv, F, nf, patch_dim, t.patches);
    return "";
}

}  // namespace

std::string build_host_tables(const std::vector<ModelInput>& models, double gravity, HostTables& H) {
    H = HostTables();
    std::vector<int> order;
    for (int i = 0; i < (int)models.size(); ++i)
        if (!models[i].is_static) order.push_back(i);
    const int nclothModels = (int)order.size();
    for (int i = 0; i < (int)models.size(); ++i)
        if (models[i].is_static) order.push_back(i);
    if (nclothModels == 0) return "no cloth model added";

    std::vector<MeshTopology> topo(models.size());
    std::vector<std::vector<int>> mF(models.size());  // collision faces: given, or a tet mesh's boundary
    std::vector<int> vbase(models.size()), fbase(models.size()), ebase(models.size());
    int nv = 0, nf = 0, ne = 0, nsim = 0;
    for (int q = 0; q < (int)order.size(); ++q) {
        const ModelInput& m = models[order[q]];
        std::string err;
        if (m.is_volumetric) err = tet_boundary_faces(m.X.data(), m.nv, m.T.data(), m.nt, mF[order[q]]);
        else mF[order[q]] = m.F;
        if (!err.empty()) return err;
        const int mnf = (int)mF[order[q]].size() / 3;
        err = build_topology(m.X.data(), m.nv, mF[order[q]].data(), mnf, m.patch_dim, m.is_volumetric,
                             topo[order[q]]);
        if (!err.empty()) return err;
        vbase[order[q]] = nv;
        fbase[order[q]] = nf;
        ebase[order[q]] = ne;
        nv += m.nv;
        nf += mnf;
        ne += (int)topo[order[q]].edges.size() / 2;
        if (!m.is_static) nsim += m.nv;
    }
    H.nsim = nsim;
    H.ntot = nv;
    H.X.resize(3 * (size_t)nv);
    for (int mi : order)
        std::copy(models[mi].X.begin(), models[mi].X.end(), H.X.begin() + 3 * (size_t)vbase[mi]);
    H.vertexModel.resize(nv);
    for (int q = 0; q < (int)order.size(); ++q)
        std::fill(H.vertexModel.begin() + vbase[order[q]], H.vertexModel.begin() + vbase[order[q]] + models[order[q]].nv,
                  q);

    // ---- cloth precompute: PdIpcClothModel::init (ClothModel.h:177-328) ----
    H.mass.assign(nsim, 0.0);
    H.Delastic.assign(nsim, 0.0);
    H.curvNorm.assign(nsim, 0.0);
    H.strain.assign(nsim, 0.0);
    H.pinSlot.assign(nsim, -1);
    H.lPtr.assign(nsim + 1, 0);
    std::vector<double> bendArea(nsim, 0.0);
    for (int q = 0; q < nclothModels; ++q) {
        const int mi = order[q];
        const ModelInput& m = models[mi];
        const MeshTopology& t = topo[mi];
        const int o = vbase[mi];
        auto P = [&](int i, int k) { return m.X[3 * i + k]; };
        if (m.is_volumetric) {
            // node mass = density * sum of the incident tets' volumes, no 1/4
            // (BaseTetMeshHandle::computeVolume, BaseTetMeshHandle.cpp:107-124;
            // PdIpcVolumetricModel.h:224-233); no springs or bending: stencil = self
            for (int e = 0; e < m.nt; ++e) {
                const int* Tv = &m.T[4 * e];
                double D[9];
                for (int r = 0; r < 3; ++r)
                    for (int k = 0; k < 3; ++k) D[3 * r + k] = P(Tv[r + 1], k) - P(Tv[0], k);
                const double det = D[0] * (D[4] * D[8] - D[5] * D[7]) - D[1] * (D[3] * D[8] - D[5] * D[6]) +
                                   D[2] * (D[3] * D[7] - D[4] * D[6]);
                const double vol = std::fabs(det / 6.0);
                for (int k = 0; k < 4; ++k) H.mass[o + Tv[k]] += vol * m.density;
            }
            for (int i = 0; i < m.nv; ++i) {
                if (!(H.mass[o + i] > 0.0)) return "tetrahedral mesh has a node in no tet";
                H.lPtr[o + i + 1] = 1;
            }
            continue;
        }
        std::vector<double> area(m.nv, 0.0);
        for (int f = 0; f < m.nf; ++f) {  // TriangleArea (Commom/GeometryComputation.cpp:3-6)
            const int* Fv = &m.F[3 * f];
            double a[3], b[3];
            for (int k = 0; k < 3; ++k) {
                a[k] = P(Fv[1], k) - P(Fv[0], k);
                b[k] = P(Fv[2], k) - P(Fv[0], k);
            }
            double c[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
            double ar = 0.5 * std::fabs(std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]));
            for (int k = 0; k < 3; ++k) area[Fv[k]] += ar / 3.0;
        }
        // per-triangle stretch stiffness: a vertex's spring weight is the mean
        // over its triangles (the reference's weight is per vertex,
        // PdIpcGpuFunc.cu:673, set from one k per model, PdIpcClothModel.h:282,300)
        std::vector<double> kv;
        if (!m.tri_stretch.empty()) {
            kv.assign(m.nv, 0.0);
            std::vector<int> nt(m.nv, 0);
            for (int f = 0; f < m.nf; ++f)
                for (int k = 0; k < 3; ++k) {
                    kv[m.F[3 * f + k]] += m.tri_stretch[f];
                    ++nt[m.F[3 * f + k]];
                }
            for (int i = 0; i < m.nv; ++i) kv[i] = nt[i] ? kv[i] / nt[i] : m.k_stretch;
        }
        for (int i = 0; i < m.nv; ++i) {
            const int g = o + i;
            H.mass[g] = area[i] * m.density;
            bendArea[g] = area[i] * m.k_bend;
            H.strain[g] = kv.empty() ? m.k_stretch : kv[i];
            const int deg = (int)t.point_edges[i].size();
            H.lPtr[g + 1] = deg + 1;  // counts for now
        }
        // Triangle strain limits: the tet constraint of
        // solveVolumetricStrainConstraintKernel (PdIpcGpuFunc.cu:439-599) for a
        // triangle, F = Ds Dm^-1 (3 x 2), with Dm the rest edges in the rest
        // triangle's orthonormal frame (e1 along the first edge, e2 in the plane)
        // and weight k x rest area.  An element with fourth vertex -1.
        if (m.k_tri_strain > 0.0 || !m.tri_strain.empty()) {
            auto P = [&](int i, int k) { return m.X[3 * i + k]; };
            for (int f = 0; f < m.nf; ++f) {
                const double kf = m.tri_strain.empty() ? m.k_tri_strain : m.tri_strain[f];
                if (!(kf > 0.0)) continue;
                const int* Fv = &m.F[3 * f];
                double a[3], b[3];
                for (int k = 0; k < 3; ++k) {
                    a[k] = P(Fv[1], k) - P(Fv[0], k);
                    b[k] = P(Fv[2], k) - P(Fv[0], k);
                }
                const double n[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
                const double la = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
                const double ln = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
                if (!(la > 0.0) || !(ln > 0.0)) return "degenerate cloth triangle under a strain limit";
                double e1[3], e2[3];
                for (int k = 0; k < 3; ++k) e1[k] = a[k] / la;
                // e2 = (n x e1) / |n|: in the plane, perpendicular to e1
                e2[0] = (n[1] * e1[2] - n[2] * e1[1]) / ln;
                e2[1] = (n[2] * e1[0] - n[0] * e1[2]) / ln;
                e2[2] = (n[0] * e1[1] - n[1] * e1[0]) / ln;
                auto dot = [](const double* u, const double* v) { return u[0] * v[0] + u[1] * v[1] + u[2] * v[2]; };
                // Dm columns: the rest edges in (e1, e2)
                const double d00 = dot(a, e1), d01 = dot(b, e1), d10 = dot(a, e2), d11 = dot(b, e2);
                const double det = d00 * d11 - d01 * d10;
                const double idm[9] = {d11 / det, -d01 / det, -d10 / det, d00 / det, 0, 0, 0, 0, 0};
                for (double v : idm) H.tetIdm.push_back(v);
                for (int k = 0; k < 3; ++k) H.tets.push_back(o + Fv[k]);
                H.tets.push_back(-1);
                H.tetW.push_back(kf * 0.5 * ln);
            }
        }
    }
    // prefix the stencil sizes, then fill the stencils
    for (int g = 0; g < nsim; ++g) H.lPtr[g + 1] += H.lPtr[g];
    const size_t nl = (size_t)H.lPtr[nsim];
    H.lNbr.assign(nl, 0);
    H.lRest.assign(nl, 0.0);
    H.lLbo.assign(nl, 0.0);
    H.lBend.assign(nl, 0.0);
    H.lBendT.assign(nl, 0.0);
    for (int q = 0; q < nclothModels; ++q) {
        const int mi = order[q];
        const ModelInput& m = models[mi];
        const MeshTopology& t = topo[mi];
        const int o = vbase[mi];
        auto P = [&](int i, int k) { return m.X[3 * i + k]; };
        if (m.is_volumetric) {
            for (int i = 0; i < m.nv; ++i) H.lNbr[H.lPtr[o + i]] = o + i;  // lLbo, lBend stay 0
            for (int p : m.pins) {
                if (p < 0 || p >= m.nv) return "pin index out of range";
                if (H.pinSlot[o + p] == -1) {
                    H.pinSlot[o + p] = (int)H.pinK.size();
                    H.pinK.push_back(m.k_pin);
                }
            }
            // strain constraints (setupHessMat, PdIpcSimulator.cpp:302-354): rest = (rows
            // p1-p0, p2-p0, p3-p0)^-1, weight k_strain * |det| / 6
            for (int e = 0; e < m.nt; ++e) {
                const int* Tv = &m.T[4 * e];
                double D[9];  // row r = p_{r+1} - p_0
                for (int r = 0; r < 3; ++r)
                    for (int k = 0; k < 3; ++k) D[3 * r + k] = P(Tv[r + 1], k) - P(Tv[0], k);
                const double c00 = D[4] * D[8] - D[5] * D[7], c01 = D[5] * D[6] - D[3] * D[8],
                             c02 = D[3] * D[7] - D[4] * D[6];
                const double det = D[0] * c00 + D[1] * c01 + D[2] * c02;
                if (!(std::fabs(det) > 0.0)) return "degenerate tetrahedron";
                // inverse of the row matrix D: inv[r][c] = cofactor[c][r] / det
                const double inv[9] = {c00 / det, (D[2] * D[7] - D[1] * D[8]) / det, (D[1] * D[5] - D[2] * D[4]) / det,
                                       c01 / det, (D[0] * D[8] - D[2] * D[6]) / det, (D[2] * D[3] - D[0] * D[5]) / det,
                                       c02 / det, (D[1] * D[6] - D[0] * D[7]) / det, (D[0] * D[4] - D[1] * D[3]) / det};
                // Dm^-1 row-major = inv transposed (rest's column-major data in the reference)
                for (int r = 0; r < 3; ++r)
                    for (int c = 0; c < 3; ++c) H.tetIdm.push_back(inv[3 * c + r]);
                for (int k = 0; k < 4; ++k) H.tets.push_back(o + Tv[k]);
                H.tetW.push_back(m.k_strain * std::fabs(det / 6.0));
            }
            continue;
        }
        // area and cotangent weights: -1/2 sum of cot of the angles opposite each edge
        std::vector<double> area(m.nv, 0.0);
        for (int f = 0; f < m.nf; ++f) {
            const int* Fv = &m.F[3 * f];
            double a[3], b[3];
            for (int k = 0; k < 3; ++k) {
                a[k] = P(Fv[1], k) - P(Fv[0], k);
                b[k] = P(Fv[2], k) - P(Fv[0], k);
            }
            double c[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
            double ar = 0.5 * std::fabs(std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]));
            for (int k = 0; k < 3; ++k) area[Fv[k]] += ar / 3.0;
        }
        const int mne = (int)t.edges.size() / 2;
        std::vector<double> cotw(mne, 0.0);
        for (int e = 0; e < mne; ++e) {
            const int a = t.edges[2 * e], b = t.edges[2 * e + 1];
            for (int f : t.edge_faces[e]) {
                int opp = -1;
                for (int k = 0; k < 3 && opp == -1; ++k) {
                    int vk = m.F[3 * f + k];
                    if (vk != a && vk != b) opp = vk;
                }
                double x10[3], x20[3];
                for (int k = 0; k < 3; ++k) {
                    x10[k] = P(a, k) - P(opp, k);
                    x20[k] = P(b, k) - P(opp, k);
                }
                double l10 = std::sqrt(x10[0] * x10[0] + x10[1] * x10[1] + x10[2] * x10[2]);
                double l20 = std::sqrt(x20[0] * x20[0] + x20[1] * x20[1] + x20[2] * x20[2]);
                double th = std::acos((x10[0] * x20[0] + x10[1] * x20[1] + x10[2] * x20[2]) / (l10 * l20));
                cotw[e] += -0.5 * (1.0 / std::tan(th));
            }
        }
        for (int i = 0; i < m.nv; ++i) {
            const int g = o + i;
            const int base = H.lPtr[g];
            const int deg = (int)t.point_edges[i].size();
            H.lNbr[base] = g;
            double sum = 0.0;
            for (int k = 0; k < deg; ++k) {
                const int e = t.point_edges[i][k];
                const int ve = (t.edges[2 * e] == i) ? t.edges[2 * e + 1] : t.edges[2 * e];
                H.lNbr[base + 1 + k] = ve + o;
                double d[3] = {P(i, 0) - P(ve, 0), P(i, 1) - P(ve, 1), P(i, 2) - P(ve, 2)};
                H.lRest[base + 1 + k] = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                const double ew = cotw[e] / area[i];
                sum += ew;
                H.lLbo[base + 1 + k] = ew;
            }
            H.lLbo[base] = -sum;
            double cv[3] = {0.0, 0.0, 0.0};
            for (int k = 0; k <= deg; ++k) {
                const int vk = H.lNbr[base + k] - o;
                for (int a = 0; a < 3; ++a) cv[a] += H.lLbo[base + k] * P(vk, a);
                H.lBend[base + k] = H.lLbo[base + k] * m.k_bend * area[i];
            }
            H.curvNorm[g] = std::sqrt(cv[0] * cv[0] + cv[1] * cv[1] + cv[2] * cv[2]);
        }
        for (int p : m.pins) {
            if (p < 0 || p >= m.nv) return "pin index out of range";
            if (H.pinSlot[o + p] == -1) {
                H.pinSlot[o + p] = (int)H.pinK.size();
                H.pinK.push_back(m.k_pin);
            }
        }
    }
    // transposed bending coefficient: what the stencil of neighbour k puts on i
    for (int i = 0; i < nsim; ++i)
        for (int s = H.lPtr[i]; s < H.lPtr[i + 1]; ++s) {
            const int k = H.lNbr[s];
            int pos = -1;
            for (int r = H.lPtr[k]; r < H.lPtr[k + 1]; ++r)
                if (H.lNbr[r] == i) {
                    pos = r;
                    break;
                }
            if (pos < 0) return "asymmetric neighbour lists";
            H.lBendT[s] = H.lBend[pos];
        }

    // ---- system matrix: pins + springs + LBO bending (setupHessMat cpp:270-414) ----
    std::vector<std::vector<std::pair<int, double>>> rows(nsim);
    for (int i = 0; i < nsim; ++i)
        if (H.pinSlot[i] >= 0) H.Delastic[i] += H.pinK[H.pinSlot[i]];
    for (int i = 0; i < nsim; ++i) {
        const double k = H.strain[i];
        for (int s = H.lPtr[i] + 1; s < H.lPtr[i + 1]; ++s) {
            H.Delastic[i] += k;
            rows[i].push_back({H.lNbr[s], -k});
        }
    }
    for (int i = 0; i < nsim; ++i) {
        const int b0 = H.lPtr[i], n = H.lPtr[i + 1] - b0;
        for (int r = 0; r < n; ++r)
            for (int c = 0; c < n; ++c) {
                const int a = H.lNbr[b0 + r], b = H.lNbr[b0 + c];
                const double v = bendArea[i] * H.lLbo[b0 + r] * H.lLbo[b0 + c];
                if (a == b) H.Delastic[a] += v;
                else rows[a].push_back({b, v});
            }
    }
    // tet strain terms: w G^T G with G = [-sum_k Dm^-T(:,k) | Dm^-T] (3 x 4);
    // a triangle element (fourth vertex -1): G^T = S Dm^-1 (3 x 2), S the rows
    // (-1, -1), (1, 0), (0, 1), the third row of G zero
    H.ntet = (int)H.tetW.size();
    for (int e = 0; e < H.ntet; ++e) {
        const double* idm = &H.tetIdm[9 * (size_t)e];
        const bool tri = H.tets[4 * (size_t)e + 3] < 0;
        double G[3][4];
        if (tri) {
            for (int j = 0; j < 2; ++j) {
                G[j][1] = idm[j];
                G[j][2] = idm[2 + j];
                G[j][0] = -(G[j][1] + G[j][2]);
                G[j][3] = 0.0;
            }
            for (int c = 0; c < 4; ++c) G[2][c] = 0.0;
        } else {
            for (int i = 0; i < 3; ++i) {
                G[i][1] = idm[i];
                G[i][2] = idm[3 + i];
                G[i][3] = idm[6 + i];
                G[i][0] = -(G[i][1] + G[i][2] + G[i][3]);
            }
        }
        const int nvert = tri ? 3 : 4;
        for (int r = 0; r < nvert; ++r)
            for (int c = 0; c < nvert; ++c) {
                double v = 0.0;
                for (int k = 0; k < 3; ++k) v += G[k][r] * G[k][c];
                v *= H.tetW[e];
                const int a = H.tets[4 * (size_t)e + r], b = H.tets[4 * (size_t)e + c];
                if (a == b) H.Delastic[a] += v;
                else rows[a].push_back({b, v});
            }
    }
    // vertex -> (tet, slot) incidence, ascending tet
    H.vtPtr.assign(nsim + 1, 0);
    for (int e = 0; e < H.ntet; ++e)
        for (int k = 0; k < 4; ++k)
            if (H.tets[4 * (size_t)e + k] >= 0) ++H.vtPtr[H.tets[4 * (size_t)e + k] + 1];
    for (int i = 0; i < nsim; ++i) H.vtPtr[i + 1] += H.vtPtr[i];
    H.vtIdx.assign(H.vtPtr[nsim], 0);
    {
        std::vector<int> fill(H.vtPtr.begin(), H.vtPtr.end() - 1);
        for (int e = 0; e < H.ntet; ++e)
            for (int k = 0; k < 4; ++k)
                if (H.tets[4 * (size_t)e + k] >= 0) H.vtIdx[fill[H.tets[4 * (size_t)e + k]]++] = (e << 2) | k;
    }
    H.nPtr.assign(nsim + 1, 0);
    for (int i = 0; i < nsim; ++i) {
        auto& R = rows[i];
        std::stable_sort(R.begin(), R.end(),
                         [](const std::pair<int, double>& x, const std::pair<int, double>& y) { return x.first < y.first; });
        size_t a = 0;
        while (a < R.size()) {
            size_t b = a;
            double s = 0.0;
            while (b < R.size() && R[b].first == R[a].first) s += R[b++].second;
            if (!(std::fabs(s) < 1e-12)) {  // IG drop (gpuSolverInit cpp:656-658)
                H.nCol.push_back(R[a].first);
                H.nVal.push_back(-s);
            }
            a = b;
        }
        H.nPtr[i + 1] = (int)H.nCol.size();
        std::vector<std::pair<int, double>>().swap(R);
    }

    // ---- collision topology (gpuCollisionInit cpp:1151-1300) ----
    H.faces.reserve(3 * (size_t)nf);
    H.edges.reserve(2 * (size_t)ne);
    H.pfPtr.assign(1, 0);
    H.ppPtr.assign(1, 0);
    H.pePtr.assign(1, 0);
    H.pxPtr.assign(1, 0);
    for (int mi : order) {
        const ModelInput& m = models[mi];
        const MeshTopology& t = topo[mi];
        const std::vector<int>& F = mF[mi];
        const int o = vbase[mi], fo = fbase[mi], eo = ebase[mi];
        for (size_t q = 0; q < F.size(); ++q) H.faces.push_back(F[q] + o);
        for (size_t q = 0; q < t.edges.size(); ++q) H.edges.push_back(t.edges[q] + o);
        std::vector<int> es, ps, xs;
        for (const auto& patch : t.patches) {
            es.clear();
            ps.clear();
            xs.clear();
            for (int f : patch) {
                H.pfIdx.push_back(f + fo);
                for (int e : t.face_edges_own[f]) es.push_back(e + eo);
                for (int p : t.face_points_own[f]) ps.push_back(p + o);
                for (int k = 0; k < 3; ++k) xs.push_back(F[3 * f + k] + o);
            }
            for (auto* vv : {&es, &ps, &xs}) {
                std::sort(vv->begin(), vv->end());
                vv->erase(std::unique(vv->begin(), vv->end()), vv->end());
            }
            H.peIdx.insert(H.peIdx.end(), es.begin(), es.end());
            H.ppIdx.insert(H.ppIdx.end(), ps.begin(), ps.end());
            H.pxIdx.insert(H.pxIdx.end(), xs.begin(), xs.end());
            H.pfPtr.push_back((int)H.pfIdx.size());
            H.pePtr.push_back((int)H.peIdx.size());
            H.ppPtr.push_back((int)H.ppIdx.size());
            H.pxPtr.push_back((int)H.pxIdx.size());
            H.pStatic.push_back(m.is_static ? 1 : 0);
        }
    }
    H.npatch = (int)H.pStatic.size();
    H.collMassSim = H.mass;
    (void)gravity;
    return "";
}

}  // namespace pdipc
