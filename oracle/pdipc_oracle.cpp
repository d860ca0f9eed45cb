// pdipc_oracle.cpp — CPU restatement of the reference PD-IPC cloth time step.
//
// TEST INFRASTRUCTURE ONLY.  This file is the correctness oracle for the GB300
// library and the timed CPU baseline; nothing in the shipped library links,
// loads or calls it.  It restates, in plain C++17 (no Eigen, no CUDA), what the
// reference does on its GPU path — the reference has no CPU implementation of
// PD-IPC (RunPlatform is stored but never consulted, Simulator/BaseSimulator.h:13-18).
//
// Parity status: unpinned by reference outputs.  The reference ships no tests,
// no golden trajectories and cannot be compiled here (MSVC project, Eigen/Qt/TBB
// absent).  The only known answers are the example scene's topology caches
// (example/ClothArmadillo/cloth1/{boundary.dat,patchInfo.dat}); tests pin the
// edge enumeration and patch partition of this oracle against them.
//
// Precision: templated on the state scalar T and the CCD/contact scalar TC.
// <float,float> reproduces the reference arithmetic (qeal = float,
// DataCore.h:8,19); <double,double> is the FP64 oracle; <float,double> mirrors
// the library's mixed mode.  Compiled with -ffp-contract=off so results do not
// depend on whether the host CPU fuses multiply-adds.
//
// Summation order: the reference accumulates the right-hand side and the
// collision diagonal with float atomics (PdIpcGpuFunc.cu:713-725, 2826-2888),
// so its order is unspecified.  Here every sum is a gather in ascending
// source order: rhs_i = ((rhs0_i + own_i + sum_{k in N(i)} bend_k(i) aq_k)
// + contact_i) + pin_i, and contact contributions in candidate-list order.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <numeric>
#include <set>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "pdipc.h"

namespace orc {

using i64 = long long;

// ---------------------------------------------------------------------------
// Mesh topology (Model/TriangleMesh/BaseSurfaceMesh.cpp:219-275 and
// Simulator/PD-IPC/PdIpcModel.h:84-172).
// ---------------------------------------------------------------------------
struct Topology {
    int nv = 0, nf = 0;
    std::vector<std::array<int, 3>> faces;
    std::vector<std::array<int, 2>> edges;           // sorted unique (min,max)
    std::vector<std::vector<int>> point_edges;       // edge ids, ascending
    std::vector<std::vector<int>> edge_faces;        // face ids, ascending
    std::vector<std::vector<int>> face_owned_edges;  // boundaryFacesSharedEdges
    std::vector<std::vector<int>> face_owned_points; // boundaryFacesSharedPoints
    std::vector<std::vector<int>> patches;           // face ids per patch
};

static std::array<int, 2> sorted_pair(int a, int b) {
    return a < b ? std::array<int, 2>{a, b} : std::array<int, 2>{b, a};
}

// Edge list: every face contributes (f[k], f[k+1]) sorted; sort
// lexicographically; unique (BaseSurfaceMesh.cpp:221-234).  Edge ids therefore
// follow (min,max) order, and each vertex's edge list is ascending in the
// neighbouring vertex id.
static void build_edges(Topology& t) {
    std::vector<std::array<int, 2>> el;
    el.reserve(3 * (size_t)t.nf);
    for (auto& f : t.faces)
        for (int k = 0; k < 3; ++k) el.push_back(sorted_pair(f[k], f[(k + 1) % 3]));
    std::sort(el.begin(), el.end());
    el.erase(std::unique(el.begin(), el.end()), el.end());
    t.edges = el;
    t.point_edges.assign(t.nv, {});
    for (int e = 0; e < (int)el.size(); ++e) {
        t.point_edges[el[e][0]].push_back(e);
        t.point_edges[el[e][1]].push_back(e);
    }
    t.edge_faces.assign(el.size(), {});
    for (int f = 0; f < t.nf; ++f)
        for (int k = 0; k < 3; ++k) {
            auto key = sorted_pair(t.faces[f][k], t.faces[f][(k + 1) % 3]);
            int e = (int)(std::lower_bound(el.begin(), el.end(), key) - el.begin());
            t.edge_faces[e].push_back(f);
        }
}

// Ownership: every edge and every point is handed to exactly one incident face,
// the first one (in incidence order) whose owned list is currently smallest
// (PdIpcModel.h:136-171).  Patch-pair expansion then never repeats a primitive.
static bool build_ownership(Topology& t, bool volumetric = false) {
    std::vector<std::vector<int>> point_faces(t.nv);
    for (int f = 0; f < t.nf; ++f)
        for (int k = 0; k < 3; ++k) point_faces[t.faces[f][k]].push_back(f);
    // edges shared faces, in the order faces push their (01,12,20) edges
    std::vector<std::vector<int>> esf(t.edges.size());
    for (int f = 0; f < t.nf; ++f) {
        const auto& F = t.faces[f];
        int ks[3][2] = {{0, 1}, {1, 2}, {2, 0}};
        for (auto& kk : ks) {
            auto key = sorted_pair(F[kk[0]], F[kk[1]]);
            int e = (int)(std::lower_bound(t.edges.begin(), t.edges.end(), key) - t.edges.begin());
            esf[e].push_back(f);
        }
    }
    t.face_owned_edges.assign(t.nf, {});
    for (int e = 0; e < (int)t.edges.size(); ++e) {
        int best = esf[e][0];
        size_t bs = t.face_owned_edges[best].size();
        for (size_t k = 1; k < esf[e].size(); ++k) {
            int f = esf[e][k];
            if (t.face_owned_edges[f].size() < bs) { best = f; bs = t.face_owned_edges[f].size(); }
        }
        t.face_owned_edges[best].push_back(e);
    }
    t.face_owned_points.assign(t.nf, {});
    for (int p = 0; p < t.nv; ++p) {
        if (point_faces[p].empty()) {
            if (volumetric) continue;  // interior node of a tet mesh
            return false;              // isolated vertex: the reference reads past the list
        }
        int best = point_faces[p][0];
        size_t bs = t.face_owned_points[best].size();
        for (size_t k = 1; k < point_faces[p].size(); ++k) {
            int f = point_faces[p][k];
            if (t.face_owned_points[f].size() < bs) { best = f; bs = t.face_owned_points[f].size(); }
        }
        t.face_owned_points[best].push_back(p);
    }
    return true;
}

// Grid collision patches (PdIpcClothModel.h:45-140), in float as the reference
// (qeal = float).  Cells form a len x len grid over the bounding box in the two
// axes other than the thinnest one; a face goes to the first cell (row-major)
// whose closed box holds its centroid; empty cells are dropped.  When no axis
// is strictly thinnest the reference leaves the axis pair uninitialised; here
// the last axis achieving the minimum extent is taken as the normal.
static void build_patches(Topology& t, const std::vector<double>& X, int patch_dim) {
    const float FMAX = std::numeric_limits<float>::infinity();
    float mn[3] = {FMAX, FMAX, FMAX}, mx[3] = {-FMAX, -FMAX, -FMAX};
    for (int i = 0; i < t.nv; ++i)
        for (int k = 0; k < 3; ++k) {
            float p = (float)X[3 * i + k];
            mn[k] = std::min(mn[k], p);
            mx[k] = std::max(mx[k], p);
        }
    int len = (int)(std::sqrt((float)t.nv) < (float)patch_dim ? std::sqrt((float)t.nv) : (float)patch_dim);
    if (len < 1) len = 1;
    float size[3];
    for (int k = 0; k < 3; ++k) size[k] = mx[k] - mn[k];
    int nrm = -1;
    if (size[0] < size[1] && size[0] < size[2]) nrm = 0;
    if (size[1] < size[0] && size[1] < size[2]) nrm = 1;
    if (size[2] < size[0] && size[2] < size[1]) nrm = 2;
    if (nrm < 0) {
        float m = std::min(size[0], std::min(size[1], size[2]));
        for (int k = 0; k < 3; ++k)
            if (size[k] == m) nrm = k;
    }
    int u = nrm == 0 ? 1 : 0;
    int v = nrm == 2 ? 1 : 2;
    const float su = size[u] / (float)len, sv = size[v] / (float)len;
    std::vector<std::vector<int>> pocket((size_t)len * len);
    for (int f = 0; f < t.nf; ++f) {
        float c[3] = {0.f, 0.f, 0.f};
        for (int k = 0; k < 3; ++k)
            for (int a = 0; a < 3; ++a) c[a] += (float)X[3 * t.faces[f][k] + a];
        for (int a = 0; a < 3; ++a) c[a] /= 3.f;
        for (int r = 0; r < len; ++r) {
            float bu0 = mn[u] + (float)r * su, bu1 = bu0 + su;
            if (!(c[u] >= bu0 && c[u] <= bu1)) continue;
            bool done = false;
            for (int cc = 0; cc < len; ++cc) {
                float bv0 = mn[v] + (float)cc * sv, bv1 = bv0 + sv;
                if (c[v] >= bv0 && c[v] <= bv1) {
                    pocket[(size_t)r * len + cc].push_back(f);
                    done = true;
                    break;
                }
            }
            if (done) break;
        }
    }
    t.patches.clear();
    for (auto& p : pocket)
        if (!p.empty()) t.patches.push_back(p);
}

// Boundary surface of a tet mesh (PdIpcVolumetricModel::registerBoundaryInfo,
// PdIpcVolumetricModel.h:27-112): faces (3,1,0), (3,2,1), (3,0,2), (2,1,0) of
// every tet; a face met once is boundary, turned away from its tet's centroid.
// The reference walks an unordered_map; here the faces come in ascending order
// of their sorted vertex triple.
static std::vector<std::array<int, 3>> tet_surface(const std::vector<double>& X, const std::vector<int>& T, int nt) {
    static const int fi[4][3] = {{3, 1, 0}, {3, 2, 1}, {3, 0, 2}, {2, 1, 0}};
    std::map<std::array<int, 3>, std::vector<std::array<int, 4>>> m;
    for (int e = 0; e < nt; ++e)
        for (auto& q : fi) {
            std::array<int, 3> f = {T[4 * e + q[0]], T[4 * e + q[1]], T[4 * e + q[2]]};
            std::array<int, 3> key = f;
            std::sort(key.begin(), key.end());
            m[key].push_back({f[0], f[1], f[2], e});
        }
    std::vector<std::array<int, 3>> out;
    for (auto& kv : m) {
        if (kv.second.size() != 1) continue;
        const auto& d = kv.second[0];
        double cent[3] = {0, 0, 0}, fc[3] = {0, 0, 0}, a[3], b[3];
        for (int k = 0; k < 3; ++k) {
            for (int q = 0; q < 4; ++q) cent[k] += X[3 * T[4 * d[3] + q] + k] / 4.0;
            for (int q = 0; q < 3; ++q) fc[k] += X[3 * d[q] + k] / 3.0;
            a[k] = X[3 * d[1] + k] - X[3 * d[0] + k];
            b[k] = X[3 * d[2] + k] - X[3 * d[0] + k];
        }
        double n[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
        double dot = 0;
        for (int k = 0; k < 3; ++k) dot += n[k] * (cent[k] - fc[k]);
        if (dot > 0) out.push_back({d[0], d[2], d[1]});
        else out.push_back({d[0], d[1], d[2]});
    }
    return out;
}

// Volumetric collision patches (PdIpcVolumetricModel.h:114-182): a
// patch_dim^3 grid over the box of the boundary points, in float; a face goes
// to the first cell in (x, y, z) order whose closed box holds its centroid.
// The cell test is a product of per-axis tests, so the first cell is the first
// index along each axis.
static void build_patches3(Topology& t, const std::vector<double>& X, int patch_dim) {
    const float FMAX = std::numeric_limits<float>::infinity();
    float mn[3] = {FMAX, FMAX, FMAX}, mx[3] = {-FMAX, -FMAX, -FMAX};
    for (auto& f : t.faces)
        for (int q = 0; q < 3; ++q)
            for (int k = 0; k < 3; ++k) {
                float p = (float)X[3 * f[q] + k];
                mn[k] = std::min(mn[k], p);
                mx[k] = std::max(mx[k], p);
            }
    const int len = std::max(1, patch_dim);
    float size[3];
    for (int k = 0; k < 3; ++k) size[k] = (mx[k] - mn[k]) / (float)len;
    std::vector<std::vector<int>> pocket((size_t)len * len * len);
    for (int f = 0; f < t.nf; ++f) {
        float c[3] = {0.f, 0.f, 0.f};
        for (int k = 0; k < 3; ++k)
            for (int a = 0; a < 3; ++a) c[a] += (float)X[3 * t.faces[f][k] + a];
        for (int a = 0; a < 3; ++a) c[a] /= 3.f;
        int id[3] = {-1, -1, -1};
        for (int a = 0; a < 3; ++a)
            for (int r = 0; r < len; ++r) {
                float b0 = mn[a] + (float)r * size[a], b1 = b0 + size[a];
                if (c[a] >= b0 && c[a] <= b1) { id[a] = r; break; }
            }
        if (id[0] < 0 || id[1] < 0 || id[2] < 0) continue;
        pocket[((size_t)id[0] * len + id[1]) * len + id[2]].push_back(f);
    }
    t.patches.clear();
    for (auto& p : pocket)
        if (!p.empty()) t.patches.push_back(p);
}

struct ModelIn {
    std::vector<double> X;
    std::vector<int> F;
    std::vector<int> T;  // 4 per tet (volumetric)
    int nv = 0, nf = 0, nt = 0;
    bool is_static = false;
    bool is_volumetric = false;
    double density = 0, k_stretch = 0, k_bend = 0, k_pin = 0, k_strain = 0;
    // cloth: per-triangle stretch (a vertex takes the mean over its triangles)
    // and per-triangle strain limits (the tet constraint on a triangle)
    std::vector<double> tri_stretch, tri_strain;
    double k_tri_strain = 0;
    std::vector<int> pins;
    int patch_dim = 10;
};

// Singular value decomposition F = U diag(s) V^T of a row-major 3x3 matrix with
// U, V proper rotations, |s0| >= |s1| >= |s2| and the sign of det F carried by
// s2 (the convention of the reference's GPU SVD, whose result it post-processes
// in solveVolumetricStrainConstraintKernel, PdIpcGpuFunc.cu:487-525).  One-sided
// Jacobi (Hestenes): rotate column pairs of A = F (and of V) until orthogonal.
template <typename R>
static void svd3_onesided(const R* F, R* U, R* s, R* V) {
    R A[3][3], W[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) A[i][j] = F[3 * i + j];
    const R eps = std::numeric_limits<R>::epsilon();
    for (int sweep = 0; sweep < 40; ++sweep) {
        bool rotated = false;
        const int pq[3][2] = {{0, 1}, {0, 2}, {1, 2}};
        for (auto& pr : pq) {
            const int p = pr[0], q = pr[1];
            R al = 0, be = 0, ga = 0;
            for (int i = 0; i < 3; ++i) {
                al += A[i][p] * A[i][p];
                be += A[i][q] * A[i][q];
                ga += A[i][p] * A[i][q];
            }
            if (!(std::fabs(ga) > eps * std::sqrt(al * be))) continue;
            rotated = true;
            const R zeta = (be - al) / (R(2) * ga);
            const R t = (zeta >= 0 ? R(1) : R(-1)) / (std::fabs(zeta) + std::sqrt(R(1) + zeta * zeta));
            const R c = R(1) / std::sqrt(R(1) + t * t), sn = c * t;
            for (int i = 0; i < 3; ++i) {
                const R ap = A[i][p], aq = A[i][q];
                A[i][p] = c * ap - sn * aq;
                A[i][q] = sn * ap + c * aq;
                const R wp = W[i][p], wq = W[i][q];
                W[i][p] = c * wp - sn * wq;
                W[i][q] = sn * wp + c * wq;
            }
        }
        if (!rotated) break;
    }
    R nrm[3];
    for (int j = 0; j < 3; ++j) nrm[j] = std::sqrt(A[0][j] * A[0][j] + A[1][j] * A[1][j] + A[2][j] * A[2][j]);
    int ord[3] = {0, 1, 2};
    std::sort(ord, ord + 3, [&](int a, int b) { return nrm[a] > nrm[b]; });
    R Us[3][3], Vs[3][3];
    for (int j = 0; j < 3; ++j) {
        s[j] = nrm[ord[j]];
        for (int i = 0; i < 3; ++i) {
            Us[i][j] = s[j] > R(0) ? A[i][ord[j]] / s[j] : R(0);
            Vs[i][j] = W[i][ord[j]];
        }
    }
    auto det3 = [](R M[3][3]) {
        return M[0][0] * (M[1][1] * M[2][2] - M[1][2] * M[2][1]) - M[0][1] * (M[1][0] * M[2][2] - M[1][2] * M[2][0]) +
               M[0][2] * (M[1][0] * M[2][1] - M[1][1] * M[2][0]);
    };
    // complete U where singular values vanish
    if (!(s[1] > R(0))) {  // rank <= 1: any unit vector orthogonal to u0, then the cross product
        R a[3] = {Us[0][0], Us[1][0], Us[2][0]};
        if (!(s[0] > R(0))) { a[0] = 1; a[1] = 0; a[2] = 0; for (int i = 0; i < 3; ++i) Us[i][0] = a[i]; }
        R e[3] = {0, 0, 0};
        e[std::fabs(a[0]) < R(0.6) ? 0 : 1] = 1;
        R d = a[0] * e[0] + a[1] * e[1] + a[2] * e[2], b[3], bn = 0;
        for (int i = 0; i < 3; ++i) { b[i] = e[i] - d * a[i]; bn += b[i] * b[i]; }
        for (int i = 0; i < 3; ++i) Us[i][1] = b[i] / std::sqrt(bn);
    }
    if (!(s[2] > R(0))) {
        Us[0][2] = Us[1][0] * Us[2][1] - Us[2][0] * Us[1][1];
        Us[1][2] = Us[2][0] * Us[0][1] - Us[0][0] * Us[2][1];
        Us[2][2] = Us[0][0] * Us[1][1] - Us[1][0] * Us[0][1];
    }
    if (det3(Vs) < 0)  // keep F = U S V^T: flip the last column of both
        for (int i = 0; i < 3; ++i) { Vs[i][2] = -Vs[i][2]; Us[i][2] = -Us[i][2]; }
    if (det3(Us) < 0) {  // the sign of det F goes to the smallest singular value
        for (int i = 0; i < 3; ++i) Us[i][2] = -Us[i][2];
        s[2] = -s[2];
    }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) { U[3 * i + j] = Us[i][j]; V[3 * i + j] = Vs[i][j]; }
}

// solveVolumetricStrainConstraintKernel (PdIpcGpuFunc.cu:439-599): F = Ds Dm^-1,
// SVD, a negative determinant flipped onto the smallest singular value, the
// singular values clamped to [0.999, 1.001] (clamp, cu:307-316), R = U S' V^T,
// and w R G scattered to the tet's four vertices (here returned per vertex).
template <typename R>
static void tet_project(const R* x0, const R* x1, const R* x2, const R* x3, const R* idm, R w, R out[4][3]) {
    R Ds[9];
    for (int k = 0; k < 3; ++k) {
        Ds[3 * k + 0] = x1[k] - x0[k];
        Ds[3 * k + 1] = x2[k] - x0[k];
        Ds[3 * k + 2] = x3[k] - x0[k];
    }
    R F[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) F[3 * i + j] = Ds[3 * i] * idm[j] + Ds[3 * i + 1] * idm[3 + j] + Ds[3 * i + 2] * idm[6 + j];
    R U[9], sv[3], V[9];
    svd3_onesided(F, U, sv, V);
    if (sv[0] * sv[1] * sv[2] < 0) sv[2] = -sv[2];
    std::sort(sv, sv + 3, [](R a, R b) { return a > b; });
    R sc[3];
    for (int k = 0; k < 3; ++k) {
        R r = sv[k] < R(1.001) ? sv[k] : R(1.001);
        sc[k] = r < R(0.999) ? R(0.999) : r;
    }
    R Rm[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) Rm[3 * i + j] = U[3 * i] * sc[0] * V[3 * j] + U[3 * i + 1] * sc[1] * V[3 * j + 1] +
                                                  U[3 * i + 2] * sc[2] * V[3 * j + 2];
    R G[3][4];
    for (int i = 0; i < 3; ++i) {
        G[i][1] = idm[i];
        G[i][2] = idm[3 + i];
        G[i][3] = idm[6 + i];
        G[i][0] = -(G[i][1] + G[i][2] + G[i][3]);
    }
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 3; ++r) out[c][r] = w * (Rm[3 * r] * G[0][c] + Rm[3 * r + 1] * G[1][c] + Rm[3 * r + 2] * G[2][c]);
}

// The same strain limit on a cloth triangle (no reference counterpart: the
// reference applies it to tets): F = Ds Dm^-1 (3 x 2, Dm the rest edges in the
// rest triangle's orthonormal frame, idm row-major 2 x 2) with the deformed
// unit normal appended as a third column, so F has singular values
// (s0, s1, 1) and a positive determinant (the AutoFlipSVD convention needs no
// flip, AutoFlipSVD.h:253-309); clamped to [0.999, 1.001]; the first two
// columns P of U S' V^T are the projection; out[c] = w P G[c], G = S Dm^-1
// with S the edge-selection rows (-1, -1), (1, 0), (0, 1).
template <typename R>
static void tri_project(const R* x0, const R* x1, const R* x2, const R* idm, R w, R out[4][3]) {
    R F[9];
    for (int k = 0; k < 3; ++k) {
        const R a = x1[k] - x0[k], b = x2[k] - x0[k];
        F[3 * k + 0] = a * idm[0] + b * idm[2];
        F[3 * k + 1] = a * idm[1] + b * idm[3];
    }
    R n[3] = {F[3] * F[7] - F[6] * F[4], F[6] * F[1] - F[0] * F[7], F[0] * F[4] - F[3] * F[1]};
    const R nn = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    for (int k = 0; k < 3; ++k) F[3 * k + 2] = nn > R(0) ? n[k] / nn : R(0);
    R U[9], sv[3], V[9];
    svd3_onesided(F, U, sv, V);
    R sc[3];
    for (int k = 0; k < 3; ++k) {
        const R a = sv[k] < R(0) ? -sv[k] : sv[k];
        R r = a < R(1.001) ? a : R(1.001);
        sc[k] = r < R(0.999) ? R(0.999) : r;
        if (sv[k] < R(0)) sc[k] = -sc[k];
    }
    R P[3][2];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 2; ++j)
            P[i][j] = U[3 * i] * sc[0] * V[3 * j] + U[3 * i + 1] * sc[1] * V[3 * j + 1] + U[3 * i + 2] * sc[2] * V[3 * j + 2];
    const R G[3][2] = {{-(idm[0] + idm[2]), -(idm[1] + idm[3])}, {idm[0], idm[1]}, {idm[2], idm[3]}};
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) out[c][r] = w * (P[r][0] * G[c][0] + P[r][1] * G[c][1]);
    out[3][0] = out[3][1] = out[3][2] = R(0);
}

// Adjoint of R(F) = U C V^T (F = U diag(s) V^T, row-major; c the clamped
// singular values, dc = dc/ds): Fb = U Pb V^T from Rb, with Rb' = U^T Rb V,
// Pb_kk = dc_k Rb'_kk and, for k < m, Pb_km = a Rb'_km + b Rb'_mk,
// Pb_mk = b Rb'_km + a Rb'_mk, a = (c_m s_m - c_k s_k) / (s_m^2 - s_k^2),
// b = (c_m s_k - c_k s_m) / (s_m^2 - s_k^2) (the SVD's differentials U^T dU,
// V^T dV); unclamped pairs a = 1, b = 0; equal values clamped to one bound
// a = -b = c / (s_k + s_m).  The library's k_adj_elem computes the same.
template <typename R>
static void clamp_svd_adjoint(const R* U, const R* s, const R* V, const R* c, const R* dc, const R* Rb, R* Fb) {
    R Rp[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            R a = 0;
            for (int k = 0; k < 3; ++k)
                for (int l = 0; l < 3; ++l) a += U[3 * k + i] * Rb[3 * k + l] * V[3 * l + j];
            Rp[3 * i + j] = a;
        }
    R Pb[9];
    for (int k = 0; k < 3; ++k) Pb[4 * k] = dc[k] * Rp[4 * k];
    for (int k = 0; k < 3; ++k)
        for (int m = k + 1; m < 3; ++m) {
            R al, be;
            if (c[k] == s[k] && c[m] == s[m]) {
                al = 1;
                be = 0;
            } else {
                const R den = s[m] * s[m] - s[k] * s[k];
                const R q = s[k] * s[k] + s[m] * s[m];
                if (den * den < R(1e-28) * q * q) {
                    const R ss = s[k] + s[m];
                    al = ss != R(0) ? c[k] / ss : R(0);
                    be = -al;
                } else {
                    al = (c[m] * s[m] - c[k] * s[k]) / den;
                    be = (c[m] * s[k] - c[k] * s[m]) / den;
                }
            }
            Pb[3 * k + m] = al * Rp[3 * k + m] + be * Rp[3 * m + k];
            Pb[3 * m + k] = be * Rp[3 * k + m] + al * Rp[3 * m + k];
        }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            R a = 0;
            for (int k = 0; k < 3; ++k)
                for (int l = 0; l < 3; ++l) a += U[3 * i + k] * Pb[3 * k + l] * V[3 * j + l];
            Fb[3 * i + j] = a;
        }
}

// Adjoint of one strain-limit element (tet_project / tri_project above) at
// the positions the forward projected: out[c] went to vertex c's right-hand
// side, so with rb the right-hand sides' adjoint (per vertex c) the vertices'
// position adjoints land in eb[c] (4 x 3).
template <typename R>
static void elem_adjoint(const R* const* x, bool tri, const R* idm, R w, const R* const* rb, R eb[4][3]) {
    R F[9], U[9], sv[3], V[9], c[3], dc[3], Rb[9] = {}, Fb[9];
    auto clampv = [](R a, R& d) {
        d = (a > R(0.999) && a < R(1.001)) ? R(1) : R(0);
        return a < R(1.001) ? (a < R(0.999) ? R(0.999) : a) : R(1.001);
    };
    for (int c2 = 0; c2 < 4; ++c2)
        for (int k = 0; k < 3; ++k) eb[c2][k] = 0;
    if (tri) {
        for (int k = 0; k < 3; ++k) {
            const R a = x[1][k] - x[0][k], b = x[2][k] - x[0][k];
            F[3 * k + 0] = a * idm[0] + b * idm[2];
            F[3 * k + 1] = a * idm[1] + b * idm[3];
        }
        const R n[3] = {F[3] * F[7] - F[6] * F[4], F[6] * F[1] - F[0] * F[7], F[0] * F[4] - F[3] * F[1]};
        const R nl = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        for (int k = 0; k < 3; ++k) F[3 * k + 2] = nl > R(0) ? n[k] / nl : R(0);
        svd3_onesided(F, U, sv, V);
        for (int k = 0; k < 3; ++k) {
            c[k] = clampv(sv[k] < R(0) ? -sv[k] : sv[k], dc[k]);
            if (sv[k] < R(0)) c[k] = -c[k];
        }
        const R G[3][2] = {{-(idm[0] + idm[2]), -(idm[1] + idm[3])}, {idm[0], idm[1]}, {idm[2], idm[3]}};
        for (int r = 0; r < 3; ++r)
            for (int j = 0; j < 2; ++j) {
                R a = 0;
                for (int v = 0; v < 3; ++v) a += rb[v][r] * G[v][j];
                Rb[3 * r + j] = w * a;
            }
        clamp_svd_adjoint(U, sv, V, c, dc, Rb, Fb);
        if (nl > R(0)) {  // the unit-normal column, n = a x b
            R nb[3] = {Fb[2], Fb[5], Fb[8]};
            const R h[3] = {n[0] / nl, n[1] / nl, n[2] / nl};
            const R pr = h[0] * nb[0] + h[1] * nb[1] + h[2] * nb[2];
            for (int k = 0; k < 3; ++k) nb[k] = (nb[k] - h[k] * pr) / nl;
            const R a[3] = {F[0], F[3], F[6]}, b[3] = {F[1], F[4], F[7]};
            const R ab[3] = {b[1] * nb[2] - b[2] * nb[1], b[2] * nb[0] - b[0] * nb[2], b[0] * nb[1] - b[1] * nb[0]};
            const R bb[3] = {nb[1] * a[2] - nb[2] * a[1], nb[2] * a[0] - nb[0] * a[2], nb[0] * a[1] - nb[1] * a[0]};
            for (int k = 0; k < 3; ++k) {
                Fb[3 * k] += ab[k];
                Fb[3 * k + 1] += bb[k];
            }
        }
        for (int k = 0; k < 3; ++k) {
            const R d0 = Fb[3 * k] * idm[0] + Fb[3 * k + 1] * idm[1];
            const R d1 = Fb[3 * k] * idm[2] + Fb[3 * k + 1] * idm[3];
            eb[1][k] = d0;
            eb[2][k] = d1;
            eb[0][k] = -(d0 + d1);
        }
        return;
    }
    for (int k = 0; k < 3; ++k) {
        const R d[3] = {x[1][k] - x[0][k], x[2][k] - x[0][k], x[3][k] - x[0][k]};
        for (int j = 0; j < 3; ++j) F[3 * k + j] = d[0] * idm[j] + d[1] * idm[3 + j] + d[2] * idm[6 + j];
    }
    svd3_onesided(F, U, sv, V);
    for (int k = 0; k < 3; ++k) {  // c_k = clamp(|s_k|): a negative determinant's s_2 flipped
        c[k] = clampv(sv[k] < R(0) ? -sv[k] : sv[k], dc[k]);
        if (sv[k] < R(0)) dc[k] = -dc[k];
    }
    R G[3][4];
    for (int i = 0; i < 3; ++i) {
        G[i][1] = idm[i];
        G[i][2] = idm[3 + i];
        G[i][3] = idm[6 + i];
        G[i][0] = -(G[i][1] + G[i][2] + G[i][3]);
    }
    for (int r = 0; r < 3; ++r)
        for (int j = 0; j < 3; ++j) {
            R a = 0;
            for (int v = 0; v < 4; ++v) a += rb[v][r] * G[j][v];
            Rb[3 * r + j] = w * a;
        }
    clamp_svd_adjoint(U, sv, V, c, dc, Rb, Fb);
    for (int k = 0; k < 3; ++k)
        for (int v = 0; v < 3; ++v) {
            const R d = Fb[3 * k] * idm[3 * v] + Fb[3 * k + 1] * idm[3 * v + 1] + Fb[3 * k + 2] * idm[3 * v + 2];
            eb[1 + v][k] = d;
            eb[0][k] -= d;
        }
}

// FP64 coplanarity-cubic CCD of one candidate (pdipc_params.ccd_mode 1; no
// reference kernel: the reference compiles Commom/PolynomialSolver.h:10-60 and
// never calls it).  Four points moving linearly are coplanar where
// f(t) = u1 . (u2 x u3) = 0, u_k(t) = (x_k - x_0) + t (d_k - d_0), a cubic; its
// roots in [0, 1] come from bisecting the monotone pieces between the roots of
// f'; the first root where the primitives touch (point inside the triangle,
// edges crossing; relative tolerance 1e-6 toward contact) is the time of
// impact, else 1.  PT: x_0 the point; EE: edges (x_0, x_1), (x_2, x_3).
static double cubic_eval(const double c[4], double t) { return ((c[3] * t + c[2]) * t + c[1]) * t + c[0]; }
static double dot3d(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static void cross3d(const double* a, const double* b, double* r) {
    r[0] = a[1] * b[2] - a[2] * b[1];
    r[1] = a[2] * b[0] - a[0] * b[2];
    r[2] = a[0] * b[1] - a[1] * b[0];
}
template <bool kPT>
static bool touching_at(const double (*x)[3], const double (*d)[3], double t, double tol) {
    double p[4][3];
    for (int j = 0; j < 4; ++j)
        for (int k = 0; k < 3; ++k) p[j][k] = x[j][k] + t * d[j][k];
    auto sub = [](const double* a, const double* b, double* r) {
        for (int k = 0; k < 3; ++k) r[k] = a[k] - b[k];
    };
    if (kPT) {
        double e1[3], e2[3], n[3], a[3], b[3], c[3], q[3];
        sub(p[2], p[1], e1);
        sub(p[3], p[1], e2);
        cross3d(e1, e2, n);
        const double nn = dot3d(n, n);
        if (!(nn > 0.0)) return false;
        sub(p[1], p[0], a);
        sub(p[2], p[0], b);
        sub(p[3], p[0], c);
        cross3d(b, c, q);
        const double wa = dot3d(q, n) / nn;
        cross3d(c, a, q);
        const double wb = dot3d(q, n) / nn;
        cross3d(a, b, q);
        const double wc = dot3d(q, n) / nn;
        return wa >= -tol && wb >= -tol && wc >= -tol;
    }
    double ea[3], eb[3], w[3];
    sub(p[1], p[0], ea);
    sub(p[3], p[2], eb);
    sub(p[0], p[2], w);
    const double aa = dot3d(ea, ea), bb = dot3d(eb, eb), ab = dot3d(ea, eb);
    const double den = aa * bb - ab * ab;
    if (!(den > 1e-24 * aa * bb)) return false;
    const double wa = dot3d(w, ea), wb = dot3d(w, eb);
    const double s = (ab * wb - bb * wa) / den, u = (aa * wb - ab * wa) / den;
    return s >= -tol && s <= 1.0 + tol && u >= -tol && u <= 1.0 + tol;
}
template <bool kPT>
static double ccd_cubic(const double (*x)[3], const double (*d)[3]) {
    double u0[3][3], u1[3][3];
    for (int k = 0; k < 3; ++k)
        for (int a = 0; a < 3; ++a) {
            u0[k][a] = x[k + 1][a] - x[0][a];
            u1[k][a] = d[k + 1][a] - d[0][a];
        }
    double c[4], bc[3], t1[3], t2[3], t3[3];
    cross3d(u0[1], u0[2], bc);
    c[0] = dot3d(u0[0], bc);
    cross3d(u1[1], u0[2], t1);
    cross3d(u0[1], u1[2], t2);
    c[1] = dot3d(u1[0], bc) + dot3d(u0[0], t1) + dot3d(u0[0], t2);
    cross3d(u1[1], u1[2], t3);
    c[2] = dot3d(u1[0], t1) + dot3d(u1[0], t2) + dot3d(u0[0], t3);
    c[3] = dot3d(u1[0], t3);
    double scale = 0.0;
    for (int k = 0; k < 3; ++k)
        scale = std::max(scale, std::max(std::sqrt(dot3d(u0[k], u0[k])), std::sqrt(dot3d(u1[k], u1[k]))));
    const double s3 = scale * scale * scale;
    if (!(s3 > 0.0) || !(std::fabs(c[0]) + std::fabs(c[1]) + std::fabs(c[2]) + std::fabs(c[3]) > 1e-14 * s3))
        return 1.0;
    double br[4] = {0.0, 1.0, 1.0, 1.0};
    int nb = 1;
    {
        const double A = 3.0 * c[3], B = 2.0 * c[2], C = c[1];
        double r0 = 2.0, r1 = 2.0;
        if (std::fabs(A) > 1e-300) {
            const double disc = B * B - 4.0 * A * C;
            if (disc >= 0.0) {
                const double q = -0.5 * (B + std::copysign(std::sqrt(disc), B));
                r0 = q / A;
                r1 = q != 0.0 ? C / q : r0;
            }
        } else if (std::fabs(B) > 1e-300) {
            r0 = -C / B;
        }
        if (r0 > r1) std::swap(r0, r1);
        if (r0 > 0.0 && r0 < 1.0) br[nb++] = r0;
        if (r1 > 0.0 && r1 < 1.0 && r1 != r0) br[nb++] = r1;
        br[nb] = 1.0;
    }
    const double tol = 1e-6;
    for (int s = 0; s < nb; ++s) {
        double lo = br[s], hi = br[s + 1];
        double flo = cubic_eval(c, lo);
        const double fhi = cubic_eval(c, hi);
        double root;
        if (flo == 0.0) {
            root = lo;
        } else if ((flo < 0.0) != (fhi < 0.0) || fhi == 0.0) {
            for (int it = 0; it < 64 && hi - lo > 0.0; ++it) {
                const double mid = 0.5 * (lo + hi);
                if (mid <= lo || mid >= hi) break;
                const double fm = cubic_eval(c, mid);
                if ((fm < 0.0) == (flo < 0.0) && fm != 0.0) {
                    lo = mid;
                    flo = fm;
                } else {
                    hi = mid;
                }
            }
            root = lo;
        } else {
            continue;
        }
        if (touching_at<kPT>(x, d, root, tol) || touching_at<kPT>(x, d, hi, tol)) return root;
    }
    return 1.0;
}

// Morton code of a quantised, centred patch centre.  The reference calls the
// un-vendored Resorting::MortonCode64(int,int,int) (AipcBvhs.cpp:181); this is
// the 63-bit interleave used by the library: each coordinate offset by 2^20,
// clamped to 21 bits, bit b of x/y/z at positions 3b/3b+1/3b+2.
static uint64_t spread21(uint64_t v) {
    v &= 0x1fffffull;
    v = (v | (v << 32)) & 0x1f00000000ffffull;
    v = (v | (v << 16)) & 0x1f0000ff0000ffull;
    v = (v | (v << 8)) & 0x100f00f00f00f00full;
    v = (v | (v << 4)) & 0x10c30c30c30c30c3ull;
    v = (v | (v << 2)) & 0x1249249249249249ull;
    return v;
}
static uint64_t morton63(int x, int y, int z) {
    auto q = [](int a) -> uint64_t {
        long long s = (long long)a + (1ll << 20);
        if (s < 0) s = 0;
        if (s > (1ll << 21) - 1) s = (1ll << 21) - 1;
        return (uint64_t)s;
    };
    return spread21(q(x)) | (spread21(q(y)) << 1) | (spread21(q(z)) << 2);
}

template <typename T>
static T omega_first(T rho2) {  // PdIpcGpuFunc.cu:1321 — 2.0/(2-rho) in double, stored as qeal
    T d = T(2) - rho2;
    return (T)(2.0 / (double)d);
}
template <typename T>
static T omega_next(T rho2, T omega) {  // PdIpcGpuFunc.cu:1341
    T d = T(4) - rho2 * omega;
    return (T)(4.0 / (double)d);
}

// ---------------------------------------------------------------------------
// The simulator.
// ---------------------------------------------------------------------------
template <typename T, typename TC>
struct Sim {
    pdipc_params prm;
    int global_form = 0;  // 0: reference R2 operator with path tables; 1: two J sweeps
    std::vector<ModelIn> models;
    bool initialized = false;

    int nsim = 0, ntot = 0;
    // state (AoS xyz, the reference layout)
    std::vector<T> X, X0, Xold, dir, V, Xrest_all, rhs0, rhs, Dinert, Delastic, D, collDiag, collRhs;
    std::vector<T> grav, invMass;
    std::vector<int> pinFlag;
    std::vector<T> pinStiff;
    std::vector<TC> collMass;
    // local step tables (flattened per vertex: [self, neighbours ascending])
    std::vector<int> lOff, lNum, lNbr;
    std::vector<T> lStrain, lRest, lLbo, lBend, lBendT, curvNorm;
    // system off-diagonals N_ij = -A_ij (CSR, ascending columns)
    std::vector<int> nPtr, nCol;
    std::vector<T> nVal;
    // tet strain constraints: global ids, row-major Dm^-1, weight; vertex -> 4*tet+slot
    int ntet = 0;
    std::vector<std::array<int, 4>> tets;
    std::vector<T> tetIdm, tetW, tetOut;
    std::vector<int> vtPtr, vtIdx;
    // reference R2 form
    std::vector<int> r2Ptr, r2Col, r2Const, r2First, pathPtr, pathK;
    std::vector<T> pathA, r2Val, r1Op, firstTerm;
    // collision topology (global ids)
    std::vector<std::array<int, 3>> faces;
    std::vector<std::array<int, 2>> edges;
    std::vector<std::vector<int>> pFaces, pPoints, pEdges, pAll;
    std::vector<char> pStatic;
    int npatch = 0;
    // patch tree (heap-indexed median split, AipcBvhs)
    std::vector<int> nodeElem;                   // -2 null, -1 internal, >=0 patch id
    std::vector<std::array<T, 6>> nodeBox;
    std::vector<int> patchNode;
    std::vector<uint64_t> morton;
    std::vector<int> order;
    // candidates
    std::vector<std::array<int, 2>> pairs;
    std::vector<std::array<int, 4>> pt, ee;
    // stats
    pdipc_stats st{};
    std::vector<T> xsweepA, xsweepB, xsweepY;
    // adjoint: positions at the start of every local-global iteration of a
    // taped step, and whether an outer iteration clamped the step or had contacts
    std::vector<std::vector<T>>* lgTape = nullptr;
    bool contactSeen = false;
    // forward-mode tangent carried through a step (two-sweep form): of the
    // positions, of the inertial rhs, and the strain weights' direction
    struct Tangent {
        std::vector<T> dP, dr0, dk;
    };
    Tangent* tan = nullptr;
    int threads = 1;

    explicit Sim(const pdipc_params& p, int form, int nthreads) : prm(p), global_form(form) {
        threads = nthreads > 0 ? nthreads : 1;
    }

    T tp(double v) const { return (T)v; }

    // ---------------- initialisation ----------------
    int initialize() {
        nsim = 0;
        ntot = 0;
        for (auto& m : models) if (!m.is_static) nsim += m.nv;
        ntot = nsim;
        for (auto& m : models) if (m.is_static) ntot += m.nv;
        if (nsim == 0) return PDIPC_ERR_STATE;
        X.assign(3 * (size_t)ntot, T(0));
        std::vector<Topology> topo;
        // order: sim models first then static, each in add order
        std::vector<int> morder;
        for (int i = 0; i < (int)models.size(); ++i) if (!models[i].is_static) morder.push_back(i);
        for (int i = 0; i < (int)models.size(); ++i) if (models[i].is_static) morder.push_back(i);
        std::vector<int> voff(models.size()), foff(models.size()), eoff(models.size());
        int vo = 0, fo = 0, eo = 0;
        topo.resize(models.size());
        for (int mi : morder) {
            auto& m = models[mi];
            Topology& t = topo[mi];
            t.nv = m.nv;
            if (m.is_volumetric) {
                t.faces = tet_surface(m.X, m.T, m.nt);
                t.nf = (int)t.faces.size();
            } else {
                t.nf = m.nf;
                t.faces.resize(m.nf);
                for (int f = 0; f < m.nf; ++f) t.faces[f] = {m.F[3 * f], m.F[3 * f + 1], m.F[3 * f + 2]};
            }
            if (t.nf == 0) return PDIPC_ERR_ARG;
            build_edges(t);
            if (!build_ownership(t, m.is_volumetric)) return PDIPC_ERR_ARG;
            if (m.is_volumetric) build_patches3(t, m.X, m.patch_dim);
            else build_patches(t, m.X, m.patch_dim);
            voff[mi] = vo; foff[mi] = fo; eoff[mi] = eo;
            for (int i = 0; i < m.nv; ++i)
                for (int k = 0; k < 3; ++k) X[3 * (size_t)(vo + i) + k] = (T)m.X[3 * i + k];
            vo += m.nv; fo += t.nf; eo += (int)t.edges.size();
        }
        // --- per-vertex cloth tables (PdIpcClothModel.h:177-328) ---
        invMass.assign(nsim, T(0));
        std::vector<double> massD(nsim, 0.0);
        grav.assign(3 * (size_t)nsim, T(0));
        pinFlag.assign(nsim, -1);
        pinStiff.clear();
        lOff.assign(nsim, 0); lNum.assign(nsim, 0);
        lNbr.clear(); lStrain.clear(); lRest.clear(); lLbo.clear(); lBend.clear(); curvNorm.assign(nsim, T(0));
        std::vector<double> bendArea(nsim, 0.0);       // A_i * b
        std::vector<std::vector<double>> lboD(nsim);
        std::vector<double> strainD(nsim, 0.0);
        tets.clear(); tetIdm.clear(); tetW.clear();
        std::vector<double> tetIdmD, tetWD;
        for (int mi : morder) {
            auto& m = models[mi];
            if (m.is_static) continue;
            Topology& t = topo[mi];
            int o = voff[mi];
            if (m.is_volumetric) {
                // node mass = density * sum of incident tet volumes (BaseTetMeshHandle.cpp:107-124)
                auto P = [&](int i, int k) { return m.X[3 * i + k]; };
                for (int e = 0; e < m.nt; ++e) {
                    const int* q = &m.T[4 * e];
                    double E[3][3];  // rows p_{r+1} - p_0 (setupHessMat cpp:313-318)
                    for (int r = 0; r < 3; ++r)
                        for (int k = 0; k < 3; ++k) E[r][k] = P(q[r + 1], k) - P(q[0], k);
                    double det = E[0][0] * (E[1][1] * E[2][2] - E[1][2] * E[2][1]) -
                                 E[0][1] * (E[1][0] * E[2][2] - E[1][2] * E[2][0]) +
                                 E[0][2] * (E[1][0] * E[2][1] - E[1][1] * E[2][0]);
                    if (det == 0.0) return PDIPC_ERR_ARG;
                    double vol = std::fabs(det / 6.0);
                    for (int k = 0; k < 4; ++k) massD[o + q[k]] += vol * m.density;
                    // rest = E^-1 (Gauss-Jordan); Dm^-1 row-major = rest^T
                    double a[3][6];
                    for (int r = 0; r < 3; ++r)
                        for (int c = 0; c < 6; ++c) a[r][c] = c < 3 ? E[r][c] : (c - 3 == r ? 1.0 : 0.0);
                    for (int c = 0; c < 3; ++c) {
                        int piv = c;
                        for (int r = c + 1; r < 3; ++r) if (std::fabs(a[r][c]) > std::fabs(a[piv][c])) piv = r;
                        for (int k = 0; k < 6; ++k) std::swap(a[c][k], a[piv][k]);
                        double d = a[c][c];
                        for (int k = 0; k < 6; ++k) a[c][k] /= d;
                        for (int r = 0; r < 3; ++r)
                            if (r != c) {
                                double f = a[r][c];
                                for (int k = 0; k < 6; ++k) a[r][k] -= f * a[c][k];
                            }
                    }
                    for (int r = 0; r < 3; ++r)
                        for (int c = 0; c < 3; ++c) tetIdmD.push_back(a[c][3 + r]);
                    tets.push_back({o + q[0], o + q[1], o + q[2], o + q[3]});
                    tetWD.push_back(m.k_strain * vol);
                }
                for (int i = 0; i < m.nv; ++i) {
                    int g = o + i;
                    if (!(massD[g] > 0.0)) return PDIPC_ERR_ARG;
                    invMass[g] = (T)(1.0 / massD[g]);
                    lOff[g] = (int)lNbr.size();
                    lNum[g] = 1;  // no springs or bending: stencil = self
                    lNbr.push_back(g);
                    lStrain.push_back(T(0));
                    lRest.push_back(T(0));
                    lLbo.push_back(T(0));
                    lBend.push_back(T(0));
                    lboD[g] = {0.0};
                }
                for (int p : m.pins) {
                    if (p < 0 || p >= m.nv) return PDIPC_ERR_ARG;
                    if (pinFlag[o + p] == -1) {
                        pinFlag[o + p] = (int)pinStiff.size();
                        pinStiff.push_back((T)m.k_pin);
                    }
                }
                continue;
            }
            std::vector<double> area(m.nv, 0.0);
            auto P = [&](int i, int k) { return m.X[3 * i + k]; };
            for (int f = 0; f < m.nf; ++f) {
                const auto& F = t.faces[f];
                double a[3], b[3];
                for (int k = 0; k < 3; ++k) { a[k] = P(F[1], k) - P(F[0], k); b[k] = P(F[2], k) - P(F[0], k); }
                double c[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
                double ar = 0.5 * std::fabs(std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]));
                for (int k = 0; k < 3; ++k) area[F[k]] += ar / 3.0;
            }
            std::vector<double> restLen(t.edges.size()), cotw(t.edges.size(), 0.0);
            for (size_t e = 0; e < t.edges.size(); ++e) {
                int a = t.edges[e][0], b = t.edges[e][1];
                double d[3] = {P(a, 0) - P(b, 0), P(a, 1) - P(b, 1), P(a, 2) - P(b, 2)};
                restLen[e] = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                for (int f : t.edge_faces[e]) {
                    int opp = -1;
                    for (int k = 0; k < 3; ++k) {
                        int vk = t.faces[f][k];
                        if (vk != a && vk != b) opp = vk;
                        if (opp != -1) break;
                    }
                    double x10[3], x20[3];
                    for (int k = 0; k < 3; ++k) { x10[k] = P(a, k) - P(opp, k); x20[k] = P(b, k) - P(opp, k); }
                    double l10 = std::sqrt(x10[0] * x10[0] + x10[1] * x10[1] + x10[2] * x10[2]);
                    double l20 = std::sqrt(x20[0] * x20[0] + x20[1] * x20[1] + x20[2] * x20[2]);
                    double th = std::acos((x10[0] * x20[0] + x10[1] * x20[1] + x10[2] * x20[2]) / (l10 * l20));
                    cotw[e] += -0.5 * (1.0 / std::tan(th));
                }
            }
            // per-vertex stretch weight: k_stretch, or the mean of the vertex's
            // triangles' stiffnesses (the reference's weight is per vertex,
            // PdIpcGpuFunc.cu:673)
            std::vector<double> kv(m.nv, m.k_stretch);
            if (!m.tri_stretch.empty()) {
                std::vector<int> nt(m.nv, 0);
                std::fill(kv.begin(), kv.end(), 0.0);
                for (int f = 0; f < m.nf; ++f)
                    for (int k = 0; k < 3; ++k) {
                        kv[t.faces[f][k]] += m.tri_stretch[f];
                        ++nt[t.faces[f][k]];
                    }
                for (int i = 0; i < m.nv; ++i) kv[i] = nt[i] ? kv[i] / nt[i] : m.k_stretch;
            }
            for (int i = 0; i < m.nv; ++i) {
                int g = o + i;
                massD[g] = area[i] * m.density;
                invMass[g] = (T)(1.0 / massD[g]);
                bendArea[g] = area[i] * m.k_bend;
                strainD[g] = kv[i];
            }
            // triangle strain limits: element (v0, v1, v2, -1), Dm^-1 (2 x 2) of the
            // rest edges in the rest triangle's orthonormal frame, weight k x area
            if (m.k_tri_strain > 0.0 || !m.tri_strain.empty()) {
                for (int f = 0; f < m.nf; ++f) {
                    const double kf = m.tri_strain.empty() ? m.k_tri_strain : m.tri_strain[f];
                    if (!(kf > 0.0)) continue;
                    const auto& F = t.faces[f];
                    double a[3], b[3];
                    for (int k = 0; k < 3; ++k) { a[k] = P(F[1], k) - P(F[0], k); b[k] = P(F[2], k) - P(F[0], k); }
                    const double n[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
                    const double la = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
                    const double ln = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
                    if (!(la > 0.0) || !(ln > 0.0)) return PDIPC_ERR_ARG;
                    double e1[3], e2[3];
                    for (int k = 0; k < 3; ++k) e1[k] = a[k] / la;
                    e2[0] = (n[1] * e1[2] - n[2] * e1[1]) / ln;
                    e2[1] = (n[2] * e1[0] - n[0] * e1[2]) / ln;
                    e2[2] = (n[0] * e1[1] - n[1] * e1[0]) / ln;
                    const double d00 = a[0] * e1[0] + a[1] * e1[1] + a[2] * e1[2];
                    const double d01 = b[0] * e1[0] + b[1] * e1[1] + b[2] * e1[2];
                    const double d10 = a[0] * e2[0] + a[1] * e2[1] + a[2] * e2[2];
                    const double d11 = b[0] * e2[0] + b[1] * e2[1] + b[2] * e2[2];
                    const double det = d00 * d11 - d01 * d10;
                    const double idm[9] = {d11 / det, -d01 / det, -d10 / det, d00 / det, 0, 0, 0, 0, 0};
                    for (double v : idm) tetIdmD.push_back(v);
                    tets.push_back({o + F[0], o + F[1], o + F[2], -1});
                    tetWD.push_back(kf * 0.5 * ln);
                }
            }
            for (int i = 0; i < m.nv; ++i) {
                int g = o + i;
                int deg = (int)t.point_edges[i].size();
                lOff[g] = (int)lNbr.size();
                lNum[g] = deg + 1;
                std::vector<double> lbo(deg + 1, 0.0);
                std::vector<int> nb(deg + 1);
                std::vector<double> rl(deg + 1, 0.0);
                nb[0] = g;
                double sum = 0.0;
                std::vector<std::array<double, 3>> qq(deg + 1);
                qq[0] = {P(i, 0), P(i, 1), P(i, 2)};
                for (int k = 0; k < deg; ++k) {
                    int e = t.point_edges[i][k];
                    int ve = (t.edges[e][0] == i) ? t.edges[e][1] : t.edges[e][0];
                    nb[k + 1] = ve + o;
                    double d[3] = {P(i, 0) - P(ve, 0), P(i, 1) - P(ve, 1), P(i, 2) - P(ve, 2)};
                    rl[k + 1] = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                    double ew = cotw[e] / area[i];
                    sum += ew;
                    lbo[k + 1] = ew;
                    qq[k + 1] = {P(ve, 0), P(ve, 1), P(ve, 2)};
                }
                lbo[0] = -sum;
                double cv[3] = {0, 0, 0};
                for (int k = 0; k < deg + 1; ++k)
                    for (int a = 0; a < 3; ++a) cv[a] += lbo[k] * qq[k][a];
                curvNorm[g] = (T)std::sqrt(cv[0] * cv[0] + cv[1] * cv[1] + cv[2] * cv[2]);
                for (int k = 0; k < deg + 1; ++k) {
                    lNbr.push_back(nb[k]);
                    lStrain.push_back((T)kv[i]);
                    lRest.push_back((T)rl[k]);
                    lLbo.push_back((T)lbo[k]);
                    lBend.push_back((T)(lbo[k] * m.k_bend * area[i]));
                }
                lboD[g] = lbo;
            }
            for (int p : m.pins) {
                if (p < 0 || p >= m.nv) return PDIPC_ERR_ARG;
                if (pinFlag[o + p] == -1) {
                    pinFlag[o + p] = (int)pinStiff.size();
                    pinStiff.push_back((T)m.k_pin);
                }
            }
        }
        // transposed bending coefficient: bendT(i, s) = bend_{k}(slot of i in k's list), k = N(i)[s]
        lBendT.assign(lNbr.size(), T(0));
        for (int i = 0; i < nsim; ++i) {
            for (int s = 0; s < lNum[i]; ++s) {
                int k = lNbr[lOff[i] + s];
                int pos = -1;
                for (int r = 0; r < lNum[k]; ++r)
                    if (lNbr[lOff[k] + r] == i) { pos = r; break; }
                if (pos < 0) return PDIPC_ERR_ARG;
                lBendT[lOff[i] + s] = lBend[lOff[k] + pos];
            }
        }
        for (int i = 0; i < nsim; ++i)
            grav[3 * (size_t)i + 1] = (T)prm.gravity * (T)massD[i];
        // --- system matrix (setupHessMat, PdIpcSimulator.cpp:270-414) ---
        std::vector<std::map<int, double>> rows(nsim);
        std::vector<double> diagE(nsim, 0.0);
        for (int i = 0; i < nsim; ++i)
            if (pinFlag[i] >= 0) diagE[i] += (double)pinStiff[pinFlag[i]];
        for (int i = 0; i < nsim; ++i) {
            double k = strainD[i];
            for (int s = 1; s < lNum[i]; ++s) {
                int j = lNbr[lOff[i] + s];
                diagE[i] += k;
                rows[i][j] -= k;
            }
        }
        for (int i = 0; i < nsim; ++i) {
            int n = lNum[i];
            for (int r = 0; r < n; ++r)
                for (int c = 0; c < n; ++c) {
                    int a = lNbr[lOff[i] + r], b = lNbr[lOff[i] + c];
                    double v = bendArea[i] * lboD[i][r] * lboD[i][c];
                    if (a == b) diagE[a] += v;
                    else rows[a][b] += v;
                }
        }
        // tet strain terms w G^T G (setupHessMat cpp:302-354)
        ntet = (int)tets.size();
        for (int e = 0; e < ntet; ++e) {
            const double* idm = &tetIdmD[9 * (size_t)e];
            const bool tri = tets[e][3] < 0;  // triangle element: G^T = S Dm^-1 (3 x 2)
            double G[3][4] = {};
            if (tri) {
                for (int j = 0; j < 2; ++j) {
                    G[j][1] = idm[j]; G[j][2] = idm[2 + j];
                    G[j][0] = -(G[j][1] + G[j][2]);
                }
            } else {
                for (int i = 0; i < 3; ++i) {
                    G[i][1] = idm[i]; G[i][2] = idm[3 + i]; G[i][3] = idm[6 + i];
                    G[i][0] = -(G[i][1] + G[i][2] + G[i][3]);
                }
            }
            const int nvert = tri ? 3 : 4;
            for (int r = 0; r < nvert; ++r)
                for (int c = 0; c < nvert; ++c) {
                    double v = 0.0;
                    for (int k = 0; k < 3; ++k) v += G[k][r] * G[k][c];
                    v *= tetWD[e];
                    int a = tets[e][r], b = tets[e][c];
                    if (a == b) diagE[a] += v;
                    else rows[a][b] += v;
                }
        }
        tetIdm.assign(tetIdmD.begin(), tetIdmD.end());
        tetW.assign(tetWD.begin(), tetWD.end());
        vtPtr.assign(nsim + 1, 0);
        for (auto& q : tets) for (int k = 0; k < 4; ++k) if (q[k] >= 0) ++vtPtr[q[k] + 1];
        for (int i = 0; i < nsim; ++i) vtPtr[i + 1] += vtPtr[i];
        vtIdx.assign(vtPtr[nsim], 0);
        {
            std::vector<int> fill(vtPtr.begin(), vtPtr.end() - 1);
            for (int e = 0; e < ntet; ++e)
                for (int k = 0; k < 4; ++k)
                    if (tets[e][k] >= 0) vtIdx[fill[tets[e][k]]++] = 4 * e + k;
        }
        tetOut.assign(12 * (size_t)ntet, T(0));
        Delastic.assign(nsim, T(0));
        for (int i = 0; i < nsim; ++i) Delastic[i] = (T)diagE[i];
        nPtr.assign(nsim + 1, 0);
        nCol.clear(); nVal.clear();
        for (int i = 0; i < nsim; ++i) {
            for (auto& kv : rows[i]) {
                if (std::fabs(kv.second) < 1e-12) continue;  // IG drop, cpp:640-669
                nCol.push_back(kv.first);
                nVal.push_back((T)(-kv.second));
            }
            nPtr[i + 1] = (int)nCol.size();
        }
        if (global_form == 0) build_r2_tables();
        // --- state ---
        X0.assign(3 * (size_t)nsim, T(0));
        V.assign(3 * (size_t)nsim, T(0));
        Xold = X;
        Xrest_all = X;
        dir.assign(3 * (size_t)ntot, T(0));
        rhs0.assign(3 * (size_t)nsim, T(0));
        rhs.assign(3 * (size_t)nsim, T(0));
        Dinert.assign(nsim, T(0));
        D.assign(nsim, T(0));
        collDiag.assign(ntot, T(0));
        collRhs.assign(3 * (size_t)ntot, T(0));
        collMass.assign(ntot, (TC)prm.static_mass);
        for (int i = 0; i < nsim; ++i) collMass[i] = (TC)(T)massD[i];
        // --- collision topology (gpuCollisionInit cpp:1151-1504) ---
        faces.clear(); edges.clear();
        pFaces.clear(); pPoints.clear(); pEdges.clear(); pAll.clear(); pStatic.clear();
        for (int mi : morder) {
            Topology& t = topo[mi];
            int o = voff[mi], fo2 = foff[mi], eo2 = eoff[mi];
            for (auto& f : t.faces) faces.push_back({f[0] + o, f[1] + o, f[2] + o});
            for (auto& e : t.edges) edges.push_back({e[0] + o, e[1] + o});
            for (auto& p : t.patches) {
                std::set<int> es, ps, xs;
                std::vector<int> fl;
                for (int f : p) {
                    fl.push_back(f + fo2);
                    for (int e : t.face_owned_edges[f]) es.insert(e + eo2);
                    for (int q : t.face_owned_points[f]) ps.insert(q + o);
                    for (int k = 0; k < 3; ++k) xs.insert(t.faces[f][k] + o);
                }
                pFaces.push_back(fl);
                pEdges.emplace_back(es.begin(), es.end());
                pPoints.emplace_back(ps.begin(), ps.end());
                pAll.emplace_back(xs.begin(), xs.end());
                pStatic.push_back(models[mi].is_static ? 1 : 0);
            }
        }
        npatch = (int)pFaces.size();
        build_tree();
        st = pdipc_stats{};
        st.n_sim = nsim;
        st.n_total = ntot;
        st.n_patches = npatch;
        initialized = true;
        return PDIPC_OK;
    }

    // R1/R2 tables of the reference (gpuSolverInit cpp:640-882): R2 = R1*R1
    // sparsity, entries |v|<1e-12 dropped, per entry the list of path terms
    // N_ik*N_jk (|.|<1e-12 dropped), const-order flag (j==i) and first-order
    // link (j in R1 row i).
    void build_r2_tables() {
        std::vector<std::map<int, int>> rowpos(nsim);
        for (int i = 0; i < nsim; ++i)
            for (int e = nPtr[i]; e < nPtr[i + 1]; ++e) rowpos[i][nCol[e]] = e;
        r2Ptr.assign(nsim + 1, 0);
        r2Col.clear(); r2Const.clear(); r2First.clear(); pathPtr.clear(); pathK.clear(); pathA.clear();
        pathPtr.push_back(0);
        for (int i = 0; i < nsim; ++i) {
            std::map<int, double> acc;
            for (int e = nPtr[i]; e < nPtr[i + 1]; ++e) {
                int k = nCol[e];
                double nik = (double)nVal[e];
                for (int f = nPtr[k]; f < nPtr[k + 1]; ++f) acc[nCol[f]] += nik * (double)nVal[f];
            }
            for (auto& kv : acc) {
                if (std::fabs(kv.second) < 1e-12) continue;
                int j = kv.first;
                // paths k ascending: k in R1 row i and in R1 row j
                std::vector<std::pair<int, double>> paths;
                for (int e = nPtr[i]; e < nPtr[i + 1]; ++e) {
                    int k = nCol[e];
                    auto it = rowpos[j].find(k);
                    if (it == rowpos[j].end()) continue;
                    double a = (double)nVal[e] * (double)nVal[it->second];
                    if (std::fabs(a) < 1e-12) continue;
                    paths.push_back({k, a});
                }
                if (paths.empty()) continue;
                r2Col.push_back(j);
                r2Const.push_back(j == i ? 1 : 0);
                auto itf = rowpos[i].find(j);
                r2First.push_back(itf == rowpos[i].end() ? -1 : itf->second);
                for (auto& pk : paths) { pathK.push_back(pk.first); pathA.push_back((T)pk.second); }
                pathPtr.push_back((int)pathK.size());
            }
            r2Ptr[i + 1] = (int)r2Col.size();
        }
        r2Val.assign(r2Col.size(), T(0));
        r1Op.assign(nCol.size(), T(0));
        firstTerm.assign(3 * (size_t)nsim, T(0));
    }

    // Patch tree of AipcBvhs::init (AipcBvhs.cpp:134-213): centres of the
    // initial (unswept, inflated) patch boxes, centred, scaled if wider than
    // 100, times 1000, truncated, Morton-coded, stably sorted; heap-indexed
    // median split with children 2n, 2n+1.
    void build_tree() {
        T infl = (T)(prm.inflation_radius < 0 ? 0.5 * prm.dhat : prm.inflation_radius);
        std::vector<std::array<T, 6>> box(npatch);
        for (int p = 0; p < npatch; ++p) {
            std::array<T, 6> b;
            for (int k = 0; k < 3; ++k) { b[k] = std::numeric_limits<T>::infinity(); b[k + 3] = -b[k]; }
            for (int v : pAll[p])
                for (int k = 0; k < 3; ++k) {
                    b[k] = std::min(b[k], (T)(X[3 * (size_t)v + k] - infl));
                    b[k + 3] = std::max(b[k + 3], (T)(X[3 * (size_t)v + k] + infl));
                }
            box[p] = b;
        }
        morton.assign(npatch, 0);
        order.resize(npatch);
        if (npatch == 0) { nodeElem.clear(); nodeBox.clear(); patchNode.clear(); return; }
        std::vector<std::array<T, 3>> c(npatch);
        T vmin[3], vmax[3];
        for (int k = 0; k < 3; ++k) { vmin[k] = std::numeric_limits<T>::infinity(); vmax[k] = -vmin[k]; }
        for (int p = 0; p < npatch; ++p)
            for (int k = 0; k < 3; ++k) {
                c[p][k] = (box[p][k] + box[p][k + 3]) / T(2);
                vmin[k] = std::min(vmin[k], c[p][k]);
                vmax[k] = std::max(vmax[k], c[p][k]);
            }
        T ctr[3];
        for (int k = 0; k < 3; ++k) ctr[k] = (vmin[k] + vmax[k]) / T(2);
        T scale = T(0);
        for (int k = 0; k < 3; ++k) scale = std::max(scale, (T)std::fabs(vmax[k] - ctr[k]));
        for (int p = 0; p < npatch; ++p) {
            int q[3];
            for (int k = 0; k < 3; ++k) {
                T v = c[p][k] - ctr[k];
                if (scale > T(100)) v = v / scale;
                q[k] = (int)(v * T(1000));
            }
            morton[p] = morton63(q[0], q[1], q[2]);
        }
        std::iota(order.begin(), order.end(), 0);
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return morton[a] < morton[b]; });
        int maxn = max_node(1, 0, npatch);
        nodeElem.assign(maxn + 1, -2);
        nodeBox.assign(maxn + 1, std::array<T, 6>{});
        patchNode.assign(npatch, -1);
        init_rec(1, 0, npatch);
    }
    int max_node(int n, int b, int e) {
        if (b + 1 == e) return n;
        int m = b + (e - b) / 2;
        return std::max(max_node(2 * n, b, m), max_node(2 * n + 1, m, e));
    }
    void init_rec(int n, int b, int e) {
        if (b + 1 == e) {
            nodeElem[n] = order[b];
            patchNode[order[b]] = n;
            return;
        }
        int m = b + (e - b) / 2;
        init_rec(2 * n, b, m);
        init_rec(2 * n + 1, m, e);
        nodeElem[n] = -1;
    }

    // ---------------- broad phase (gpuCcdCulling cpp:1799-1869) ----------------
    void patch_boxes(const std::vector<T>& xo, const std::vector<T>& dx, std::vector<std::array<T, 6>>& pb) {
        T infl = (T)(prm.inflation_radius < 0 ? 0.5 * prm.dhat : prm.inflation_radius);
        pb.resize(npatch);
#pragma omp parallel for schedule(static) num_threads(threads)
        for (int p = 0; p < npatch; ++p) {
            std::array<T, 6> b;
            for (int k = 0; k < 3; ++k) { b[k] = std::numeric_limits<T>::max(); b[k + 3] = -std::numeric_limits<T>::max(); }
            for (int f : pFaces[p]) {
                // getFaceBbox with displacement (PdIpcGpuFunc.cu:1350-1375)
                for (int k = 0; k < 3; ++k) {
                    T a0 = xo[3 * (size_t)faces[f][0] + k], a1 = xo[3 * (size_t)faces[f][1] + k], a2 = xo[3 * (size_t)faces[f][2] + k];
                    T b0 = a0 + dx[3 * (size_t)faces[f][0] + k], b1 = a1 + dx[3 * (size_t)faces[f][1] + k], b2 = a2 + dx[3 * (size_t)faces[f][2] + k];
                    T mn = std::min(std::min(std::min(a0, a1), a2), std::min(std::min(b0, b1), b2)) - infl;
                    T mx = std::max(std::max(std::max(a0, a1), a2), std::max(std::max(b0, b1), b2)) + infl;
                    b[k] = std::min(b[k], mn);
                    b[k + 3] = std::max(b[k + 3], mx);
                }
            }
            pb[p] = b;
        }
    }
    static bool overlap(const std::array<T, 6>& a, const std::array<T, 6>& b) {
        if (a[3] < b[0] || b[3] < a[0]) return false;
        if (a[4] < b[1] || b[4] < a[1]) return false;
        if (a[5] < b[2] || b[5] < a[2]) return false;
        return true;
    }
    void refit(const std::vector<std::array<T, 6>>& pb) {
        for (int n = (int)nodeElem.size() - 1; n >= 1; --n) {
            if (nodeElem[n] >= 0) nodeBox[n] = pb[nodeElem[n]];
            else if (nodeElem[n] == -1) {
                for (int k = 0; k < 3; ++k) {
                    nodeBox[n][k] = std::min(nodeBox[2 * n][k], nodeBox[2 * n + 1][k]);
                    nodeBox[n][k + 3] = std::max(nodeBox[2 * n][k + 3], nodeBox[2 * n + 1][k + 3]);
                }
            }
        }
    }
    // traverseIterative (PdIpcGpuFunc.cu:1628-1697): reports (q, p) with q < p.
    void traverse(int q, std::vector<std::array<int, 2>>& out) {
        const auto& qb = nodeBox[patchNode[q]];
        int stack[128];
        int sp = 0;
        stack[sp++] = 0;
        int node = 1;
        int nn = (int)nodeElem.size();
        if (nn <= 1) return;
        if (nodeElem[1] >= 0) return;  // single patch
        do {
            int cl = 2 * node, cr = cl + 1;
            bool ol = cl < nn && nodeElem[cl] != -2 && overlap(qb, nodeBox[cl]);
            bool orr = cr < nn && nodeElem[cr] != -2 && overlap(qb, nodeBox[cr]);
            if (ol && nodeElem[cl] >= 0 && q < nodeElem[cl]) out.push_back({q, nodeElem[cl]});
            if (orr && nodeElem[cr] >= 0 && q < nodeElem[cr]) out.push_back({q, nodeElem[cr]});
            bool tl = ol && nodeElem[cl] == -1, tr = orr && nodeElem[cr] == -1;
            if (!tl && !tr) node = stack[--sp];
            else {
                node = tl ? cl : cr;
                if (tl && tr) stack[sp++] = cr;
            }
        } while (node != 0);
    }
    void broadphase(const std::vector<T>& xo, const std::vector<T>& dx) {
        std::vector<std::array<T, 6>> pb;
        patch_boxes(xo, dx, pb);
        refit(pb);
        std::vector<std::vector<std::array<int, 2>>> per(npatch);
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads)
        for (int q = 0; q < npatch; ++q) traverse(q, per[q]);
        pairs.clear();
        for (int q = 0; q < npatch; ++q) {
            std::sort(per[q].begin(), per[q].end());
            for (auto& pr : per[q])
                if (!(pStatic[pr[0]] && pStatic[pr[1]])) pairs.push_back(pr);
        }
        // expansion (getCcdPotentialICPairsListKernel, PdIpcGpuFunc.cu:1838-1948)
        pt.clear();
        ee.clear();
        for (auto& pr : pairs) {
            int A = pr[0], B = pr[1];
            for (int v : pPoints[A])
                for (int f : pFaces[B]) pt.push_back({v, faces[f][0], faces[f][1], faces[f][2]});
            for (int v : pPoints[B])
                for (int f : pFaces[A]) pt.push_back({v, faces[f][0], faces[f][1], faces[f][2]});
            for (int a : pEdges[A])
                for (int b : pEdges[B]) ee.push_back({edges[a][0], edges[a][1], edges[b][0], edges[b][1]});
        }
        st.patch_pairs = (i64)pairs.size();
        st.pt_candidates = (i64)pt.size();
        st.ee_candidates = (i64)ee.size();
    }

    // ---------------- geometry (PdIpcGpuFunc.cu:2152-2292) ----------------
    static TC dot3(const TC* a, const TC* b) { TC s = 0; for (int k = 0; k < 3; ++k) s += a[k] * b[k]; return s; }
    static void sub3(const TC* a, const TC* b, TC* r) { for (int k = 0; k < 3; ++k) r[k] = a[k] - b[k]; }
    static void cross3(const TC* a, const TC* b, TC* r) {
        r[0] = a[1] * b[2] - b[1] * a[2];
        r[1] = a[2] * b[0] - b[2] * a[0];
        r[2] = a[0] * b[1] - b[0] * a[1];
    }
    static TC vtx_edge_sq(const TC* v, const TC* ea, const TC* eb, TC* r, TC* d) {
        TC va[3], ba[3];
        sub3(v, ea, va); sub3(eb, ea, ba);
        TC vb = dot3(va, ba), bb = dot3(ba, ba);
        if (vb < 0) *r = 0; else if (vb > bb) *r = 1; else *r = vb / bb;
        for (int k = 0; k < 3; ++k) d[k] = v[k] - (ea[k] * ((TC)1.0 - *r) + eb[k] * *r);
        return dot3(d, d);
    }
    static TC edge_edge_sq(const TC* xi, const TC* xj, const TC* xa, const TC* xb, TC* r, TC* s, TC* d) {
        TC xba[3], xji[3], xai[3], tmp[3];
        sub3(xb, xa, xba); sub3(xj, xi, xji); sub3(xa, xi, xai);
        cross3(xji, xba, d);
        TC nn = dot3(d, d);
        cross3(xai, xji, tmp);
        TC w_aiji = dot3(d, tmp);
        cross3(xai, xba, tmp);
        TC w_aiba = dot3(d, tmp);
        if (nn > (TC)1e-24f && w_aiji >= 0 && w_aiji <= nn && w_aiba >= 0 && w_aiba <= nn) {
            *r = w_aiba / nn;
            *s = w_aiji / nn;
        } else {
            TC best = (TC)999999999, dd, v, nd[3];
            if (w_aiba < 0 && ((dd = vtx_edge_sq(xi, xa, xb, &v, nd)) < best)) { best = dd; *r = 0; *s = v; }
            if (w_aiba > nn && ((dd = vtx_edge_sq(xj, xa, xb, &v, nd)) < best)) { best = dd; *r = 1; *s = v; }
            if (w_aiji < 0 && ((dd = vtx_edge_sq(xa, xi, xj, &v, nd)) < best)) { best = dd; *r = v; *s = 0; }
            if (w_aiji > nn && ((dd = vtx_edge_sq(xb, xi, xj, &v, nd)) < best)) { best = dd; *r = v; *s = 1; }
        }
        for (int k = 0; k < 3; ++k)
            d[k] = xi[k] * (1 - *r) + xj[k] * *r - xa[k] * ((TC)1.0 - *s) - xb[k] * *s;
        return dot3(d, d);
    }
    static TC vtx_tri(const TC* xi, const TC* xa, const TC* xb, const TC* xc, TC* ba, TC* bb, TC* bc, TC* d) {
        TC xba[3], xca[3], xia[3], tmp[3];
        sub3(xb, xa, xba); sub3(xc, xa, xca); sub3(xi, xa, xia);
        cross3(xba, xca, d);
        TC nn = dot3(d, d);
        cross3(xia, xca, tmp);
        TC w_iaca = dot3(d, tmp);
        cross3(xba, xia, tmp);
        TC w_baia = dot3(d, tmp);
        if (nn > (TC)1e-24f && w_iaca >= 0 && w_baia >= 0 && nn - w_iaca - w_baia >= 0) {
            *bb = w_iaca / nn;
            *bc = w_baia / nn;
            *ba = 1 - *bb - *bc;
        } else {
            TC best = (TC)999999999, r, dd, N[3];
            if (nn - w_iaca - w_baia < 0 && ((dd = vtx_edge_sq(xi, xb, xc, &r, N)) < best)) { best = dd; *bb = 1 - r; *bc = r; *ba = 0; }
            if (w_iaca < 0 && ((dd = vtx_edge_sq(xi, xa, xc, &r, N)) < best)) { best = dd; *bb = 0; *bc = r; *ba = 1 - *bb - *bc; }
            if (w_baia < 0 && ((dd = vtx_edge_sq(xi, xa, xb, &r, N)) < best)) { best = dd; *bb = r; *bc = 0; *ba = 1 - *bb - *bc; }
        }
        for (int k = 0; k < 3; ++k) d[k] = xi[k] - xa[k] * *ba - xb[k] * *bb - xc[k] * *bc;
        return dot3(d, d);
    }
    static TC mn3(TC a, TC b, TC c) { return std::min(std::min(a, b), c); }
    static TC mx3(TC a, TC b, TC c) { return std::max(std::max(a, b), c); }
    template <typename R>
    static bool pt_ccd_broad(const R* p, const R* t0, const R* t1, const R* t2, const R* dp, const R* d0,
                             const R* d1, const R* d2, R dist) {
        auto lo3 = [](R a, R b, R c) { return std::min(std::min(a, b), c); };
        auto hi3 = [](R a, R b, R c) { return std::max(std::max(a, b), c); };
        for (int k = 0; k < 3; ++k) {
            R tmin = lo3(t0[k], t1[k], t2[k]);
            tmin = lo3(tmin, t0[k] + d0[k], t1[k] + d1[k]);
            tmin = std::min(tmin, t2[k] + d2[k]);
            R tmax = hi3(t0[k], t1[k], t2[k]);
            tmax = hi3(tmax, t0[k] + d0[k], t1[k] + d1[k]);
            tmax = std::max(tmax, t2[k] + d2[k]);
            R pmin = std::min(p[k], p[k] + dp[k]), pmax = std::max(p[k], p[k] + dp[k]);
            if ((pmin - tmax) > dist || (tmin - pmax) > dist) return false;
        }
        return true;
    }
    template <typename R>
    static bool ee_ccd_broad(const R* a0, const R* a1, const R* b0, const R* b1, const R* da0, const R* da1,
                             const R* db0, const R* db1, R dist) {
        for (int k = 0; k < 3; ++k) {
            R mina = std::min(a0[k], a0[k] + da0[k]); mina = std::min(mina, a1[k]); mina = std::min(mina, a1[k] + da1[k]);
            R maxa = std::max(a0[k], a0[k] + da0[k]); maxa = std::max(maxa, a1[k]); maxa = std::max(maxa, a1[k] + da1[k]);
            R minb = std::min(b0[k], b0[k] + db0[k]); minb = std::min(minb, b1[k]); minb = std::min(minb, b1[k] + db1[k]);
            R maxb = std::max(b0[k], b0[k] + db0[k]); maxb = std::max(maxb, b1[k]); maxb = std::max(maxb, b1[k] + db1[k]);
            if ((mina - maxb) > dist || (minb - maxa) > dist) return false;
        }
        return true;
    }
    static TC sqn(const TC* a) { return dot3(a, a); }
    // additive CCD, point-triangle (ccdVertexTriangleToi, PdIpcGpuFunc.cu:2460-2529)
    TC ccd_pt(TC* x0, TC* d0, TC* x1, TC* d1, TC* x2, TC* d2, TC* x3, TC* d3) const {
        TC mov[3];
        for (int k = 0; k < 3; ++k) mov[k] = (d0[k] + d1[k] + d2[k] + d3[k]) / (TC)4.0;
        for (int k = 0; k < 3; ++k) { d0[k] -= mov[k]; d1[k] -= mov[k]; d2[k] -= mov[k]; d3[k] -= mov[k]; }
        TC m2 = std::max(sqn(d1), sqn(d2));
        m2 = std::max(m2, sqn(d3));
        TC maxd = std::sqrt(sqn(d0)) + std::sqrt(m2);
        if (maxd == (TC)0.0) return 1;
        TC a, b, c, dd[3];
        TC d2c = vtx_tri(x0, x1, x2, x3, &a, &b, &c, dd);
        TC dc = std::sqrt(d2c);
        TC gap = (TC)prm.ccd_eta * dc;
        TC toc = 0;
        for (int i = 0; i < prm.ccd_max_iter; ++i) {
            TC lb = (TC)0.9 * d2c / (dc * maxd);
            for (int k = 0; k < 3; ++k) { x0[k] += lb * d0[k]; x1[k] += lb * d1[k]; x2[k] += lb * d2[k]; x3[k] += lb * d3[k]; }
            d2c = vtx_tri(x0, x1, x2, x3, &a, &b, &c, dd);
            dc = std::sqrt(d2c);
            if (toc != (TC)0 && dc < gap) break;
            toc += lb;
            if (toc > (TC)1.0) { toc = 1; break; }
        }
        return toc;
    }
    static TC pp_min(const TC* x0, const TC* x1, const TC* x2, const TC* x3) {
        auto d2 = [](const TC* a, const TC* b) {
            return (a[0] - b[0]) * (a[0] - b[0]) + (a[1] - b[1]) * (a[1] - b[1]) + (a[2] - b[2]) * (a[2] - b[2]);
        };
        TC r = d2(x0, x2);
        r = std::min(d2(x0, x3), r);
        r = std::min(d2(x1, x2), r);
        r = std::min(d2(x1, x3), r);
        return r;
    }
    // additive CCD, edge-edge (ccdEdgeEdgeToi, PdIpcGpuFunc.cu:2531-2607)
    TC ccd_ee(TC* x0, TC* d0, TC* x1, TC* d1, TC* x2, TC* d2, TC* x3, TC* d3) const {
        TC mov[3];
        for (int k = 0; k < 3; ++k) mov[k] = (d0[k] + d1[k] + d2[k] + d3[k]) / (TC)4.0;
        for (int k = 0; k < 3; ++k) { d0[k] -= mov[k]; d1[k] -= mov[k]; d2[k] -= mov[k]; d3[k] -= mov[k]; }
        TC m0 = std::max(sqn(d0), sqn(d1)), m1 = std::max(sqn(d2), sqn(d3));
        TC maxd = std::sqrt(m0) + std::sqrt(m1);
        if (maxd == 0) return 1;
        TC r, s, dd[3];
        TC d2c = edge_edge_sq(x0, x1, x2, x3, &r, &s, dd);
        TC f = d2c;
        if (f <= 0) { d2c = pp_min(x0, x1, x2, x3); f = d2c; }
        TC dc = std::sqrt(d2c);
        TC gap = (TC)prm.ccd_eta * f / dc;
        TC toc = 0;
        for (int i = 0; i < prm.ccd_max_iter; ++i) {
            TC lb = (TC)0.9 * f / (dc * maxd);
            for (int k = 0; k < 3; ++k) { x0[k] += lb * d0[k]; x1[k] += lb * d1[k]; x2[k] += lb * d2[k]; x3[k] += lb * d3[k]; }
            d2c = edge_edge_sq(x0, x1, x2, x3, &r, &s, dd);
            f = d2c;
            if (f <= 0) { d2c = pp_min(x0, x1, x2, x3); f = d2c; }
            dc = std::sqrt(d2c);
            if (toc != (TC)0 && (f / dc) < gap) break;
            toc += lb;
            if (toc > (TC)1.0) { toc = 1; break; }
        }
        return toc;
    }
    void load4(const std::vector<T>& x, const std::array<int, 4>& ids, TC out[4][3]) const {
        for (int j = 0; j < 4; ++j)
            for (int k = 0; k < 3; ++k) out[j][k] = (TC)x[3 * (size_t)ids[j] + k];
    }
    // getImpactOfTimeKernel (PdIpcGpuFunc.cu:2610-2704); per-candidate toi (1 when skipped)
    TC toi_pt_one(const std::array<int, 4>& c, const std::vector<T>& xa, const std::vector<T>& xb) const {
        if (c[0] == c[1] || c[0] == c[2] || c[0] == c[3]) return 1;
        TC p[4][3], q[4][3], d[4][3];
        load4(xa, c, p);
        load4(xb, c, q);
        for (int j = 0; j < 4; ++j) for (int k = 0; k < 3; ++k) d[j][k] = q[j][k] - p[j][k];
        if (prm.ccd_mode == 2) return (TC)cubic_toi<true>(c, xa, xb);
        TC t = 1;
        if (pt_ccd_broad(p[0], p[1], p[2], p[3], d[0], d[1], d[2], d[3], (TC)prm.ccd_slack))
            t = ccd_pt(p[0], d[0], p[1], d[1], p[2], d[2], p[3], d[3]);
        if (prm.ccd_mode == 1) t = std::min(t, (TC)cubic_toi<true>(c, xa, xb));
        return t;
    }
    TC toi_ee_one(const std::array<int, 4>& c, const std::vector<T>& xa, const std::vector<T>& xb) const {
        if (c[0] == c[2] || c[0] == c[3] || c[1] == c[2] || c[1] == c[3]) return 1;
        TC p[4][3], q[4][3], d[4][3];
        load4(xa, c, p);
        load4(xb, c, q);
        for (int j = 0; j < 4; ++j) for (int k = 0; k < 3; ++k) d[j][k] = q[j][k] - p[j][k];
        if (prm.ccd_mode == 2) return (TC)cubic_toi<false>(c, xa, xb);
        TC t = 1;
        if (ee_ccd_broad(p[0], p[1], p[2], p[3], d[0], d[1], d[2], d[3], (TC)prm.ccd_slack))
            t = ccd_ee(p[0], d[0], p[1], d[1], p[2], d[2], p[3], d[3]);
        if (prm.ccd_mode == 1) t = std::min(t, (TC)cubic_toi<false>(c, xa, xb));
        return t;
    }
    // ccd_mode 1: the FP64 coplanarity-cubic time of impact of one candidate
    // (the swept-box test in FP64, then orc::ccd_cubic on coordinates relative
    // to the first point); 1 when it finds no contact.
    template <bool kPT>
    double cubic_toi(const std::array<int, 4>& c, const std::vector<T>& xa, const std::vector<T>& xb) const {
        double p[4][3], d[4][3];
        for (int j = 0; j < 4; ++j)
            for (int k = 0; k < 3; ++k) {
                p[j][k] = (double)(TC)xa[3 * (size_t)c[j] + k];
                d[j][k] = (double)(TC)xb[3 * (size_t)c[j] + k] - p[j][k];
            }
        const double sl = prm.ccd_slack;
        const bool near = kPT ? pt_ccd_broad(p[0], p[1], p[2], p[3], d[0], d[1], d[2], d[3], sl)
                              : ee_ccd_broad(p[0], p[1], p[2], p[3], d[0], d[1], d[2], d[3], sl);
        if (!near) return 1.0;
        for (int j = 3; j >= 0; --j)
            for (int k = 0; k < 3; ++k) p[j][k] -= p[0][k];
        return ccd_cubic<kPT>(p, d);
    }
    // global toi: min over candidates (NaN results never win, as in the
    // reference's `toi < toiList` test), then times 0.98 if below 1.
    TC global_toi(const std::vector<T>& xa, const std::vector<T>& xb, std::vector<double>* tp_, std::vector<double>* te_) {
        TC best = 1;
        i64 npt = (i64)pt.size(), nee = (i64)ee.size();
        if (tp_) tp_->assign(npt, 1.0);
        if (te_) te_->assign(nee, 1.0);
#pragma omp parallel num_threads(threads)
        {
            TC lb = 1;
#pragma omp for schedule(static) nowait
            for (i64 i = 0; i < npt; ++i) {
                TC t = toi_pt_one(pt[i], xa, xb);
                if (tp_) (*tp_)[i] = (double)t;
                if (t < lb) lb = t;
            }
#pragma omp for schedule(static) nowait
            for (i64 i = 0; i < nee; ++i) {
                TC t = toi_ee_one(ee[i], xa, xb);
                if (te_) (*te_)[i] = (double)t;
                if (t < lb) lb = t;
            }
#pragma omp critical
            if (lb < best) best = lb;
        }
        if (best < (TC)1.0) best = (TC)((double)best * prm.toi_scale);
        return best;
    }

    // setCollisionConstraintsKernel (PdIpcGpuFunc.cu:2756-2892)
    struct Contrib { int ids[4]; TC w; TC tgt[4][3]; bool on; };
    TC barrier(TC d2, TC dh2, TC kap) const {
        TC e = 0;
        if (d2 < dh2) {
            TC t2 = d2 - dh2;
            e = -kap * t2 * t2 * std::log(d2 / dh2) / (dh2 * dh2);
        }
        return e;
    }
    void contact_one(int type, const std::array<int, 4>& c, const std::vector<T>& x, Contrib& out) const {
        out.on = false;
        TC dh = (TC)(T)prm.dhat;
        TC dh2 = (TC)((T)prm.dhat * (T)prm.dhat);
        TC kap = (TC)(T)prm.kappa;
        TC dt = (TC)(T)prm.time_step;
        TC p[4][3];
        load4(x, c, p);
        TC d[3], dist2, mp, mq;
        if (type == 0) {
            if (c[0] == c[1] || c[0] == c[2] || c[0] == c[3]) return;
            for (int k = 0; k < 3; ++k) {  // point_triangle_cd_broadphase
                TC tmin = mn3(p[1][k], p[2][k], p[3][k]), tmax = mx3(p[1][k], p[2][k], p[3][k]);
                if ((p[0][k] - tmax) > dh || (tmin - p[0][k]) > dh) return;
            }
            TC a, b, cc;
            dist2 = vtx_tri(p[0], p[1], p[2], p[3], &a, &b, &cc, d);
            if (dist2 >= dh2) return;
            mp = collMass[c[0]];
            mq = a * collMass[c[1]] + b * collMass[c[2]] + cc * collMass[c[3]];
        } else {
            if (c[0] == c[2] || c[0] == c[3] || c[1] == c[2] || c[1] == c[3]) return;
            for (int k = 0; k < 3; ++k) {  // edge_edge_cd_broadphase
                TC mina = std::min(p[0][k], p[1][k]), maxa = std::max(p[0][k], p[1][k]);
                TC minb = std::min(p[2][k], p[3][k]), maxb = std::max(p[2][k], p[3][k]);
                if ((mina - maxb) > dh || (minb - maxa) > dh) return;
            }
            TC r, s;
            dist2 = edge_edge_sq(p[0], p[1], p[2], p[3], &r, &s, d);
            if (dist2 >= dh2) return;
            mp = (1 - r) * collMass[c[0]] + r * collMass[c[1]];
            mq = (1 - s) * collMass[c[2]] + s * collMass[c[3]];
        }
        TC dist = std::sqrt(dist2);
        TC w = barrier(dist2, dh2, kap) + std::min(mp, mq) / (dt * dt);
        TC rp = mq / (mp + mq), rq = mp / (mp + mq);
        TC len = std::sqrt(dot3(d, d));
        for (int k = 0; k < 3; ++k) d[k] /= len;
        dist = dh - dist;
        TC dp = dist * rp, dq = dist * rq;
        out.on = true;
        out.w = w;
        for (int j = 0; j < 4; ++j) out.ids[j] = c[j];
        for (int k = 0; k < 3; ++k) {
            if (type == 0) {
                out.tgt[0][k] = w * (p[0][k] + dp * d[k]);
                out.tgt[1][k] = w * (p[1][k] - dq * d[k]);
                out.tgt[2][k] = w * (p[2][k] - dq * d[k]);
                out.tgt[3][k] = w * (p[3][k] - dq * d[k]);
            } else {
                out.tgt[0][k] = w * (p[0][k] + dp * d[k]);
                out.tgt[1][k] = w * (p[1][k] + dp * d[k]);
                out.tgt[2][k] = w * (p[2][k] - dq * d[k]);
                out.tgt[3][k] = w * (p[3][k] - dq * d[k]);
            }
        }
    }
    i64 contacts(const std::vector<T>& x) {
        std::fill(collDiag.begin(), collDiag.end(), T(0));
        std::fill(collRhs.begin(), collRhs.end(), T(0));
        i64 npt = (i64)pt.size(), nee = (i64)ee.size();
        std::vector<Contrib> cb(npt + nee);
#pragma omp parallel for schedule(static) num_threads(threads)
        for (i64 i = 0; i < npt + nee; ++i) {
            if (i < npt) contact_one(0, pt[i], x, cb[i]);
            else contact_one(1, ee[i - npt], x, cb[i]);
        }
        i64 active = 0;
        for (i64 i = 0; i < npt + nee; ++i) {
            if (!cb[i].on) continue;
            ++active;
            for (int j = 0; j < 4; ++j) {
                int v = cb[i].ids[j];
                collDiag[v] += (T)cb[i].w;
                for (int k = 0; k < 3; ++k) collRhs[3 * (size_t)v + k] += (T)cb[i].tgt[j][k];
            }
        }
        return active;
    }

    // ---------------- PD kernels ----------------
    // predictiveKernel (PdIpcGpuFunc.cu:88-147)
    void predict(T dt) {
#pragma omp parallel for schedule(static) num_threads(threads)
        for (int i = 0; i < nsim; ++i) {
            if (pinFlag[i] != -1) { V[3 * i] = V[3 * i + 1] = V[3 * i + 2] = T(0); continue; }
            T m = invMass[i] * dt;
            T y[3];
            for (int k = 0; k < 3; ++k) {
                T v = V[3 * i + k] + m * grav[3 * i + k];
                v = v * dt;
                y[k] = v + X[3 * i + k];
            }
            T mm = (T)(1.0 / (double)(dt * m));
            Dinert[i] = (T)(1.0 / (double)(invMass[i] * dt * dt));
            for (int k = 0; k < 3; ++k) {
                rhs0[3 * i + k] = mm * y[k];
                X[3 * i + k] = y[k];
            }
        }
    }
    // solveClothPointsStrainAndBendingConstraintKernel (PdIpcGpuFunc.cu:627-728)
    // in gather form, plus the contact rhs and solvePointsConstraintKernel (cu:764-790).
    void local_rhs(std::vector<T>& aq) {
        aq.assign(3 * (size_t)nsim, T(0));
#pragma omp parallel for schedule(static) num_threads(threads)
        for (int i = 0; i < nsim; ++i) {
            int o = lOff[i], n = lNum[i];
            T a[3];
            for (int k = 0; k < 3; ++k) a[k] = X[3 * i + k] * lLbo[o];
            for (int s = 1; s < n; ++s) {
                int j = lNbr[o + s];
                for (int k = 0; k < 3; ++k) a[k] += X[3 * (size_t)j + k] * lLbo[o + s];
            }
            T nrm = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
            if (nrm >= T(1e-10)) {
                T c = curvNorm[i] / nrm;
                for (int k = 0; k < 3; ++k) a[k] *= c;
            }
            for (int k = 0; k < 3; ++k) aq[3 * (size_t)i + k] = a[k];
        }
#pragma omp parallel for schedule(static) num_threads(threads)
        for (int e = 0; e < ntet; ++e) {
            T out[4][3] = {};
            const auto& q = tets[e];
            if (q[3] < 0)
                tri_project<T>(&X[3 * (size_t)q[0]], &X[3 * (size_t)q[1]], &X[3 * (size_t)q[2]], &tetIdm[9 * (size_t)e],
                               tetW[e], out);
            else
                tet_project<T>(&X[3 * (size_t)q[0]], &X[3 * (size_t)q[1]], &X[3 * (size_t)q[2]],
                               &X[3 * (size_t)q[3]], &tetIdm[9 * (size_t)e], tetW[e], out);
            for (int c = 0; c < 4; ++c)
                for (int k = 0; k < 3; ++k) tetOut[12 * (size_t)e + 3 * c + k] = out[c][k];
        }
#pragma omp parallel for schedule(static) num_threads(threads)
        for (int i = 0; i < nsim; ++i) {
            int o = lOff[i], n = lNum[i];
            T x[3] = {X[3 * i], X[3 * i + 1], X[3 * i + 2]};
            T tx[3] = {0, 0, 0};
            T strain = lStrain[o];
            for (int s = 1; s < n; ++s) {
                int j = lNbr[o + s];
                T d[3];
                for (int k = 0; k < 3; ++k) d[k] = x[k] - X[3 * (size_t)j + k];
                T cl = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                T rc = strain * (lRest[o + s] / cl);
                for (int k = 0; k < 3; ++k) tx[k] += rc * d[k];
            }
            for (int k = 0; k < 3; ++k) tx[k] += lBend[o] * aq[3 * (size_t)i + k];
            T r[3];
            for (int k = 0; k < 3; ++k) r[k] = rhs0[3 * i + k] + tx[k];
            for (int s = 1; s < n; ++s) {
                int j = lNbr[o + s];
                for (int k = 0; k < 3; ++k) r[k] += lBendT[o + s] * aq[3 * (size_t)j + k];
            }
            for (int q = vtPtr[i]; q < vtPtr[i + 1]; ++q)  // tet projections, ascending tet
                for (int k = 0; k < 3; ++k) r[k] += tetOut[3 * (size_t)vtIdx[q] + k];
            for (int k = 0; k < 3; ++k) r[k] += collRhs[3 * (size_t)i + k];
            if (pinFlag[i] >= 0) {
                T ks = pinStiff[pinFlag[i]];
                for (int k = 0; k < 3; ++k) r[k] += ks * Xrest_all[3 * (size_t)i + k];
            }
            for (int k = 0; k < 3; ++k) rhs[3 * i + k] = r[k];
        }
    }
    // J sweep: y_i = (1-w) x_i + w ((sum_j N_ij x_j + b_i) / D_i)
    void jsweep(const std::vector<T>& x, std::vector<T>& y, T w, const std::vector<T>& invD) {
#pragma omp parallel for schedule(static) num_threads(threads)
        for (int i = 0; i < nsim; ++i) {
            T s[3] = {0, 0, 0};
            for (int e = nPtr[i]; e < nPtr[i + 1]; ++e) {
                int j = nCol[e];
                for (int k = 0; k < 3; ++k) s[k] += nVal[e] * x[3 * (size_t)j + k];
            }
            for (int k = 0; k < 3; ++k)
                y[3 * (size_t)i + k] = (T(1) - w) * x[3 * (size_t)i + k] + w * ((s[k] + rhs[3 * (size_t)i + k]) * invD[i]);
        }
    }
    void global_jj() {
        T w = (T)prm.jacobi_relax;
        std::vector<T> invD(nsim);
        for (int i = 0; i < nsim; ++i) invD[i] = T(1) / D[i];
        size_t n3 = 3 * (size_t)nsim;
        std::vector<T>& Y = xsweepY;
        std::vector<T>& B = xsweepA;
        Y.resize(n3); B.resize(n3);
        std::vector<T> xcur(X.begin(), X.begin() + n3);
        // x1 = S(S(x0))
        jsweep(xcur, Y, w, invD);
        std::vector<T> prev = xcur;
        jsweep(Y, B, w, invD);
        xcur = B;
        T rho = (T)prm.cheby_rho;
        rho = rho * rho;
        T om = omega_first(rho);
        for (int it = 1; it < prm.cheby_iterations; ++it) {
            jsweep(xcur, Y, w, invD);
            jsweep(Y, B, w, invD);
#pragma omp parallel for schedule(static) num_threads(threads)
            for (size_t q = 0; q < n3; ++q) B[q] = om * (B[q] - prev[q]) + prev[q];
            prev.swap(xcur);
            xcur = B;
            om = omega_next(rho, om);
        }
        std::copy(xcur.begin(), xcur.end(), X.begin());
    }
    // Reference form: updateSuperJacobiOperatorsHost (cu:976-1038) then
    // chebyshevJacobiR2SolverHost (cu:1245-1346).
    void update_r2_ops() {
        T w = (T)prm.jacobi_relax;
#pragma omp parallel for schedule(static) num_threads(threads)
        for (int i = 0; i < nsim; ++i)
            for (int e = nPtr[i]; e < nPtr[i + 1]; ++e) r1Op[e] = nVal[e] / D[i];
#pragma omp parallel for schedule(static) num_threads(threads)
        for (int i = 0; i < nsim; ++i) {
            for (int q = r2Ptr[i]; q < r2Ptr[i + 1]; ++q) {
                T v = 0;
                for (int p = pathPtr[q]; p < pathPtr[q + 1]; ++p) v += pathA[p] / (D[i] * D[pathK[p]]);
                v *= w * w;
                v += (T(1) - w) * (T(1) - w) * (T)r2Const[q];
                if (r2First[q] > -1) v += T(2) * (T(1) - w) * w * r1Op[r2First[q]];
                r2Val[q] = v;
            }
        }
    }
    void global_r2() {
        T w = (T)prm.jacobi_relax;
        size_t n3 = 3 * (size_t)nsim;
#pragma omp parallel for schedule(static) num_threads(threads)
        for (int i = 0; i < nsim; ++i) {
            for (int k = 0; k < 3; ++k) {
                T v = 0;
                for (int e = nPtr[i]; e < nPtr[i + 1]; ++e) {
                    int j = nCol[e];
                    v += r1Op[e] * (rhs[3 * (size_t)j + k] / D[j]);
                }
                firstTerm[3 * (size_t)i + k] = w * w * v + (T(2) - w) * w * rhs[3 * (size_t)i + k] / D[i];
            }
        }
        std::vector<T>& A = xsweepA;
        std::vector<T>& Bn = xsweepB;
        A.resize(n3); Bn.resize(n3);
        std::vector<T> prev(X.begin(), X.begin() + n3), cur(n3);
        auto r2mul = [&](const std::vector<T>& x, std::vector<T>& y) {
#pragma omp parallel for schedule(static) num_threads(threads)
            for (int i = 0; i < nsim; ++i)
                for (int k = 0; k < 3; ++k) {
                    T v = 0;
                    for (int q = r2Ptr[i]; q < r2Ptr[i + 1]; ++q) v += r2Val[q] * x[3 * (size_t)r2Col[q] + k];
                    y[3 * (size_t)i + k] = v + firstTerm[3 * (size_t)i + k];
                }
        };
        r2mul(prev, cur);
        T rho = (T)prm.cheby_rho;
        rho = rho * rho;
        T om = omega_first(rho);
        for (int it = 1; it < prm.cheby_iterations; ++it) {
            r2mul(cur, Bn);
#pragma omp parallel for schedule(static) num_threads(threads)
            for (size_t q = 0; q < n3; ++q) Bn[q] = om * (Bn[q] - prev[q]) + prev[q];
            prev.swap(cur);
            cur.swap(Bn);
            om = omega_next(rho, om);
        }
        std::copy(cur.begin(), cur.end(), X.begin());
    }

    void pd_solve() {
        // sysDiag = elastic + inertial (+ collision): cpp:1556-1560
#pragma omp parallel for schedule(static) num_threads(threads)
        for (int i = 0; i < nsim; ++i) D[i] = (Delastic[i] + Dinert[i]) + collDiag[i];
        if (tan) {
            pd_solve_tangent();
            return;
        }
        if (global_form == 0) update_r2_ops();
        std::vector<T> aq;
        for (int lg = 0; lg < prm.lg_iterations; ++lg) {
            if (lgTape) lgTape->emplace_back(X.begin(), X.begin() + 3 * (size_t)nsim);
            local_rhs(aq);
            if (global_form == 0) global_r2();
            else global_jj();
        }
    }

    // advance (PdIpcSimulator.cpp:1683-1796)
    int step_once() {
        T dt = (T)prm.time_step;
        size_t n3 = 3 * (size_t)nsim;
        std::copy(X.begin(), X.begin() + n3, X0.begin());
        std::copy(X.begin(), X.begin() + n3, Xold.begin());
        std::fill(collDiag.begin(), collDiag.end(), T(0));
        std::fill(collRhs.begin(), collRhs.end(), T(0));
        predict(dt);
        int outer = 0;
        int max_outer = prm.fixed_outer > 0 ? prm.fixed_outer : prm.max_outer;
        for (; outer < max_outer; ++outer) {
            pd_solve();
            for (size_t q = 0; q < n3; ++q) dir[q] = X[q] - Xold[q];
            if (outer == 0) broadphase(Xold, dir);
            TC toi = global_toi(Xold, X, nullptr, nullptr);
            T tt = (T)toi;
            for (size_t q = 0; q < n3; ++q) X[q] = Xold[q] + tt * dir[q];
            st.active_contacts = contacts(X);
            if (toi != TC(1) || st.active_contacts != 0) contactSeen = true;
            double res = 0;
            for (size_t q = 0; q < n3; ++q) res += (double)dir[q] * (double)dir[q];
            st.last_toi = (double)toi;
            st.last_residual = res;
            for (size_t q = 0; q < n3; ++q)
                if (!std::isfinite((double)X[q])) return PDIPC_ERR_NONFINITE;
            if (prm.fixed_outer <= 0 && res < prm.outer_tol && outer > 0) { ++outer; break; }
            std::copy(X.begin(), X.begin() + n3, Xold.begin());
        }
        // updateVelocityKernel (cu:262-281) with damping = 1 - dt
        T damping = (T)(1.0 - (double)dt);
        T invt = (T)((1.0 / (double)dt) * (double)damping);
        for (size_t q = 0; q < n3; ++q) V[q] = (X[q] - X0[q]) * invt;
        st.last_outer_iters = outer;
        st.total_outer_iters += outer;
        st.max_outer_iters = std::max(st.max_outer_iters, outer);
        st.steps_done++;
        return PDIPC_OK;
    }
    // Prediction then one outer iteration's PD solve without contact terms,
    // from a caller state; the simulation state is restored afterwards.
    int stage_pd(const double* Xin, const double* Vin, double* out) {
        if (!initialized) return PDIPC_ERR_STATE;
        std::vector<T> sx = X, sv = V;
        for (size_t q = 0; q < X.size(); ++q) X[q] = (T)Xin[q];
        for (size_t q = 0; q < V.size(); ++q) V[q] = (T)Vin[q];
        std::fill(collDiag.begin(), collDiag.end(), T(0));
        std::fill(collRhs.begin(), collRhs.end(), T(0));
        predict((T)prm.time_step);
        pd_solve();
        for (size_t q = 0; q < X.size(); ++q) out[q] = (double)X[q];
        X = sx;
        V = sv;
        return PDIPC_OK;
    }

    // ---------------- discrete adjoint of contact-free steps (two-sweep form) ----------------
    // The library's reverse pass (adjoint_kernels.cu; solver.cu adjoint_step)
    // restated sequentially on this oracle's tables.  The step's forward:
    // predict (cu:88-147), lg local steps (cu:627-790, gather form) each
    // followed by the two-sweep Chebyshev-Jacobi solve, the identity clamp of
    // a contact-free outer iteration, the velocity update (cu:262-281).
    // X, V hold the step's start state; pb, vb (3 nsim) hold dL/d(positions,
    // velocities) after the step on entry and before it on return; kb (nsim)
    // collects dL/d(strain weight).  X, V are left at the step's end.
    int adjoint_step(std::vector<T>& pb, std::vector<T>& vb, std::vector<T>& kb) {
        if (global_form != 1) return PDIPC_ERR_STATE;
        std::vector<std::vector<T>> tape;
        lgTape = &tape;
        contactSeen = false;
        const int r = step_once();
        lgTape = nullptr;
        if (r != PDIPC_OK) return r;
        if (contactSeen) return PDIPC_ERR_STATE;
        const size_t n3 = 3 * (size_t)nsim;
        const int cb = prm.cheby_iterations;
        const T w = (T)prm.jacobi_relax;
        const T dt = (T)prm.time_step;
        const T invt = (T)((1.0 / (double)dt) * (double)(T)(1.0 - (double)dt));
        std::vector<T> invD(nsim);
        for (int i = 0; i < nsim; ++i) invD[i] = T(1) / D[i];
        std::vector<T> oms;
        {
            T rho2 = (T)prm.cheby_rho;
            rho2 = rho2 * rho2;
            T om = omega_first(rho2);
            for (int it = 1; it < cb; ++it) {
                oms.push_back(om);
                om = omega_next(rho2, om);
            }
        }
        // transposed LBO weights: slot s of row i pointing at j -> weight of row j at i
        std::vector<T> lboT(lLbo.size(), T(0));
        for (int i = 0; i < nsim; ++i) {
            const int o = lOff[i];
            lboT[o] = lLbo[o];
            for (int s2 = 1; s2 < lNum[i]; ++s2) {
                const int j = lNbr[o + s2];
                for (int t = 1; t < lNum[j]; ++t)
                    if (lNbr[lOff[j] + t] == i) { lboT[o + s2] = lLbo[lOff[j] + t]; break; }
            }
        }
        auto S = [&](const std::vector<T>& z, std::vector<T>& y) { jsweep(z, y, w, invD); };
        // out (= or +=) J^T u = (1-w) u + N^T (w D^-1 u)
        // N^T as a CSR of its own (row i: the entries N_ji, ascending j), so the
        // transposed product is a gather
        std::vector<int> tPtr(nsim + 1, 0), tCol(nPtr[nsim]);
        std::vector<T> tVal(nPtr[nsim]);
        for (int e = 0; e < nPtr[nsim]; ++e) ++tPtr[nCol[e] + 1];
        for (int i = 0; i < nsim; ++i) tPtr[i + 1] += tPtr[i];
        {
            std::vector<int> fill(tPtr.begin(), tPtr.end() - 1);
            for (int j = 0; j < nsim; ++j)
                for (int e = nPtr[j]; e < nPtr[j + 1]; ++e) {
                    tCol[fill[nCol[e]]] = j;
                    tVal[fill[nCol[e]]++] = nVal[e];
                }
        }
        auto JT = [&](const std::vector<T>& u, std::vector<T>& out, bool acc) {
#pragma omp parallel for schedule(static) num_threads(threads)
            for (int i = 0; i < nsim; ++i)
                for (int k = 0; k < 3; ++k) {
                    T y = 0;
                    for (int e = tPtr[i]; e < tPtr[i + 1]; ++e) {
                        const int j = tCol[e];
                        y += tVal[e] * (w * invD[j] * u[3 * (size_t)j + k]);
                    }
                    const size_t q = 3 * (size_t)i + k;
                    out[q] = (acc ? out[q] : T(0)) + (T(1) - w) * u[q] + y;
                }
        };
        // kb_i += u_i . dS_i/dk_i: k_i sits on row i's spring entries of N and deg_i times in D_i
        auto stiff = [&](const std::vector<T>& u, const std::vector<T>& z) {
#pragma omp parallel for schedule(static) num_threads(threads)
            for (int i = 0; i < nsim; ++i) {
                const int o = lOff[i], deg = lNum[i] - 1;
                T acc = 0;
                for (int k = 0; k < 3; ++k) {
                    T nz = rhs[3 * (size_t)i + k], sz = 0;
                    for (int e = nPtr[i]; e < nPtr[i + 1]; ++e) nz += nVal[e] * z[3 * (size_t)nCol[e] + k];
                    for (int s2 = 1; s2 <= deg; ++s2) sz += z[3 * (size_t)lNbr[o + s2] + k];
                    acc += u[3 * (size_t)i + k] * (sz - T(deg) * invD[i] * nz);
                }
                kb[i] += w * invD[i] * acc;
            }
        };
        std::vector<T> r0b(n3, T(0)), X0b(n3);
        for (size_t q = 0; q < n3; ++q) {
            X0b[q] = -invt * vb[q];
            pb[q] += invt * vb[q];
        }
        std::vector<std::vector<T>> Xs(cb + 1, std::vector<T>(n3)), Ys(cb, std::vector<T>(n3));
        std::vector<std::vector<T>> Xb(cb + 1, std::vector<T>(n3));
        std::vector<T> aq, u(n3), rho(n3), rb(n3), qb(n3), tmp(n3);
        for (int l = (int)tape.size() - 1; l >= 0; --l) {
            const std::vector<T>& x = tape[l];
            std::copy(x.begin(), x.end(), X.begin());
            local_rhs(aq);
            Xs[0] = x;
            S(Xs[0], Ys[0]);
            if (cb > 1) S(Ys[0], Xs[1]);
            for (int it = 1; it < cb; ++it) {
                S(Xs[it], Ys[it]);
                if (it + 1 < cb) {
                    S(Ys[it], tmp);
                    for (size_t q = 0; q < n3; ++q) Xs[it + 1][q] = oms[it - 1] * (tmp[q] - Xs[it - 1][q]) + Xs[it - 1][q];
                }
            }
            for (int t = 0; t < cb; ++t) std::fill(Xb[t].begin(), Xb[t].end(), T(0));
            Xb[cb] = pb;
            std::fill(rho.begin(), rho.end(), T(0));
            for (int it = cb - 1; it >= 1; --it) {
                const T om = oms[it - 1];
                for (size_t q = 0; q < n3; ++q) {
                    tmp[q] = om * Xb[it + 1][q];
                    Xb[it - 1][q] += (T(1) - om) * Xb[it + 1][q];
                    rho[q] += tmp[q];
                }
                stiff(tmp, Ys[it]);
                JT(tmp, u, false);
                for (size_t q = 0; q < n3; ++q) rho[q] += u[q];
                stiff(u, Xs[it]);
                JT(u, Xb[it], true);
            }
            for (size_t q = 0; q < n3; ++q) rho[q] += Xb[1][q];
            stiff(Xb[1], Ys[0]);
            JT(Xb[1], u, false);
            for (size_t q = 0; q < n3; ++q) rho[q] += u[q];
            stiff(u, Xs[0]);
            JT(u, Xb[0], true);
            for (int i = 0; i < nsim; ++i)
                for (int k = 0; k < 3; ++k) {
                    rb[3 * (size_t)i + k] = w * invD[i] * rho[3 * (size_t)i + k];
                    r0b[3 * (size_t)i + k] += rb[3 * (size_t)i + k];
                }
            // curvature vectors: abar_k = sum_s bend_s rb_nbr(s), then through a = q c / |q|
#pragma omp parallel for schedule(static) num_threads(threads)
            for (int i = 0; i < nsim; ++i) {
                const int o = lOff[i];
                T q[3] = {0, 0, 0}, a[3] = {0, 0, 0};
                for (int s2 = 0; s2 < lNum[i]; ++s2) {
                    const int j = lNbr[o + s2];
                    for (int k = 0; k < 3; ++k) {
                        q[k] += lLbo[o + s2] * x[3 * (size_t)j + k];
                        a[k] += lBend[o + s2] * rb[3 * (size_t)j + k];
                    }
                }
                const T nrm = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
                if (nrm >= T(1e-10)) {
                    const T pr = (q[0] * a[0] + q[1] * a[1] + q[2] * a[2]) / nrm;
                    const T c = curvNorm[i] / nrm;
                    for (int k = 0; k < 3; ++k) a[k] = c * (a[k] - q[k] / nrm * pr);
                }
                for (int k = 0; k < 3; ++k) qb[3 * (size_t)i + k] = a[k];
            }
            // positions: transposed LBO gather of qb, spring projections; strain weights
#pragma omp parallel for schedule(static) num_threads(threads)
            for (int m = 0; m < nsim; ++m) {
                const int o = lOff[m];
                T acc[3];
                for (int k = 0; k < 3; ++k) acc[k] = Xb[0][3 * (size_t)m + k];
                for (int s2 = 0; s2 < lNum[m]; ++s2) {
                    const int j = lNbr[o + s2];
                    for (int k = 0; k < 3; ++k) acc[k] += lboT[o + s2] * qb[3 * (size_t)j + k];
                    if (s2 == 0) continue;
                    T d[3];
                    for (int k = 0; k < 3; ++k) d[k] = x[3 * (size_t)m + k] - x[3 * (size_t)j + k];
                    const T len = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                    const T rest = lRest[o + s2];
                    const T cm = lStrain[o] * rest, cj = lStrain[lOff[j]] * rest;
                    T uu[3], pr = 0, kr = 0;
                    for (int k = 0; k < 3; ++k) {
                        uu[k] = cm * rb[3 * (size_t)m + k] - cj * rb[3 * (size_t)j + k];
                        pr += d[k] / len * uu[k];
                        kr += rb[3 * (size_t)m + k] * d[k] / len;
                    }
                    for (int k = 0; k < 3; ++k) acc[k] += (uu[k] - d[k] / len * pr) / len;
                    kb[m] += rest * kr;
                }
                for (int k = 0; k < 3; ++k) pb[3 * (size_t)m + k] = acc[k];
            }
            // strain-limit elements: their adjoints per element, then each
            // vertex adds its elements' in ascending element order
            if (ntet > 0) {
                std::vector<T> eb(12 * (size_t)ntet);
#pragma omp parallel for schedule(static) num_threads(threads)
                for (int e = 0; e < ntet; ++e) {
                    const auto& q = tets[e];
                    const bool tri = q[3] < 0;
                    const T* xs[4];
                    const T* rs[4];
                    for (int c2 = 0; c2 < 4; ++c2) {
                        const int v = (tri && c2 == 3) ? q[0] : q[c2];
                        xs[c2] = &x[3 * (size_t)v];
                        rs[c2] = &rb[3 * (size_t)v];
                    }
                    T out[4][3];
                    elem_adjoint<T>(xs, tri, &tetIdm[9 * (size_t)e], tetW[e], rs, out);
                    for (int c2 = 0; c2 < 4; ++c2)
                        for (int k = 0; k < 3; ++k) eb[12 * (size_t)e + 3 * c2 + k] = out[c2][k];
                }
                for (int i = 0; i < nsim; ++i)
                    for (int t = vtPtr[i]; t < vtPtr[i + 1]; ++t)
                        for (int k = 0; k < 3; ++k) pb[3 * (size_t)i + k] += eb[3 * (size_t)vtIdx[t] + k];
            }
        }
        // through the prediction (pinned vertices start at x with v = 0)
        for (int i = 0; i < nsim; ++i)
            for (int k = 0; k < 3; ++k) {
                const size_t q = 3 * (size_t)i + k;
                if (pinFlag[i] != -1) {
                    pb[q] = X0b[q] + pb[q];
                    vb[q] = T(0);
                } else {
                    const T m = invMass[i] * dt;
                    const T mm = (T)(1.0 / (double)(dt * m));
                    const T y = pb[q] + mm * r0b[q];
                    pb[q] = X0b[q] + y;
                    vb[q] = dt * y;
                }
            }
        return PDIPC_OK;
    }

    // ---------------- forward-mode tangent of contact-free steps (two-sweep form) ----------------
    // The same local-global iterations as pd_solve / local_rhs / global_jj with
    // the directional derivative carried alongside: springs and curvature
    // through their normalisations, the sweeps' N, D and rhs (the strain
    // weight k_i sits on row i's spring entries of N and deg_i times in D_i).
    void pd_solve_tangent() {
        Tangent& t = *tan;
        const size_t n3 = 3 * (size_t)nsim;
        const T w = (T)prm.jacobi_relax;
        std::vector<T> invD(nsim), dInvD(nsim);
        for (int i = 0; i < nsim; ++i) {
            invD[i] = T(1) / D[i];
            dInvD[i] = -T(lNum[i] - 1) * t.dk[i] * invD[i] * invD[i];
        }
        std::vector<T> aq, da(n3), dr(n3);
        auto S = [&](const std::vector<T>& z, const std::vector<T>& dz, std::vector<T>& y, std::vector<T>& dy) {
            jsweep(z, y, w, invD);
#pragma omp parallel for schedule(static) num_threads(threads)
            for (int i = 0; i < nsim; ++i) {
                const int o = lOff[i];
                for (int k = 0; k < 3; ++k) {
                    T nz = rhs[3 * (size_t)i + k], ndz = dr[3 * (size_t)i + k], sz = 0;
                    for (int e = nPtr[i]; e < nPtr[i + 1]; ++e) {
                        nz += nVal[e] * z[3 * (size_t)nCol[e] + k];
                        ndz += nVal[e] * dz[3 * (size_t)nCol[e] + k];
                    }
                    for (int s2 = 1; s2 < lNum[i]; ++s2) sz += z[3 * (size_t)lNbr[o + s2] + k];
                    const size_t q = 3 * (size_t)i + k;
                    dy[q] = (T(1) - w) * dz[q] + w * (invD[i] * (ndz + t.dk[i] * sz) + dInvD[i] * nz);
                }
            }
        };
        for (int lg = 0; lg < prm.lg_iterations; ++lg) {
            // tangent of the curvature vectors and of the rhs at X
#pragma omp parallel for schedule(static) num_threads(threads)
            for (int i = 0; i < nsim; ++i) {
                const int o = lOff[i];
                T q[3] = {0, 0, 0}, dq[3] = {0, 0, 0};
                for (int s2 = 0; s2 < lNum[i]; ++s2) {
                    const int j = lNbr[o + s2];
                    for (int k = 0; k < 3; ++k) {
                        q[k] += lLbo[o + s2] * X[3 * (size_t)j + k];
                        dq[k] += lLbo[o + s2] * t.dP[3 * (size_t)j + k];
                    }
                }
                const T nrm = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
                if (nrm >= T(1e-10)) {
                    const T pr = (q[0] * dq[0] + q[1] * dq[1] + q[2] * dq[2]) / nrm;
                    const T c = curvNorm[i] / nrm;
                    for (int k = 0; k < 3; ++k) dq[k] = c * (dq[k] - q[k] / nrm * pr);
                }
                for (int k = 0; k < 3; ++k) da[3 * (size_t)i + k] = dq[k];
            }
#pragma omp parallel for schedule(static) num_threads(threads)
            for (int i = 0; i < nsim; ++i) {
                const int o = lOff[i];
                T r[3];
                for (int k = 0; k < 3; ++k) r[k] = t.dr0[3 * (size_t)i + k] + lBend[o] * da[3 * (size_t)i + k];
                for (int s2 = 1; s2 < lNum[i]; ++s2) {
                    const int j = lNbr[o + s2];
                    T d[3], dd[3];
                    for (int k = 0; k < 3; ++k) {
                        d[k] = X[3 * (size_t)i + k] - X[3 * (size_t)j + k];
                        dd[k] = t.dP[3 * (size_t)i + k] - t.dP[3 * (size_t)j + k];
                    }
                    const T len = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                    const T rest = lRest[o + s2];
                    const T pr = (d[0] * dd[0] + d[1] * dd[1] + d[2] * dd[2]) / len;
                    for (int k = 0; k < 3; ++k) {
                        r[k] += lStrain[o] * rest / len * (dd[k] - d[k] / len * pr);
                        r[k] += t.dk[i] * rest * d[k] / len;
                        r[k] += lBendT[o + s2] * da[3 * (size_t)j + k];
                    }
                }
                for (int k = 0; k < 3; ++k) dr[3 * (size_t)i + k] = r[k];
            }
            local_rhs(aq);
            // the two-sweep Chebyshev solve (global_jj) with tangents
            std::vector<T> xcur(X.begin(), X.begin() + n3), dxcur(t.dP.begin(), t.dP.end());
            std::vector<T> Y(n3), dY(n3), B(n3), dB(n3);
            S(xcur, dxcur, Y, dY);
            std::vector<T> prev = xcur, dprev = dxcur;
            S(Y, dY, B, dB);
            xcur = B;
            dxcur = dB;
            T rho = (T)prm.cheby_rho;
            rho = rho * rho;
            T om = omega_first(rho);
            for (int it = 1; it < prm.cheby_iterations; ++it) {
                S(xcur, dxcur, Y, dY);
                S(Y, dY, B, dB);
                for (size_t q = 0; q < n3; ++q) {
                    B[q] = om * (B[q] - prev[q]) + prev[q];
                    dB[q] = om * (dB[q] - dprev[q]) + dprev[q];
                }
                prev.swap(xcur);
                dprev.swap(dxcur);
                xcur = B;
                dxcur = dB;
                om = omega_next(rho, om);
            }
            std::copy(xcur.begin(), xcur.end(), X.begin());
            t.dP = dxcur;
        }
    }
    // A rollout of nsteps from (Xin, Vin) with the tangent (dXin, dVin, dk):
    // the final positions' and velocities' tangents.  PDIPC_ERR_STATE if an
    // outer iteration clamped the step or had contacts.
    int tangent_rollout(int nsteps, const double* Xin, const double* Vin, const double* dXin, const double* dVin,
                        const double* dkin, double* dXout, double* dVout) {
        if (!initialized) return PDIPC_ERR_STATE;
        if (global_form != 1 || ntet > 0) return PDIPC_ERR_STATE;
        if (nsteps < 1) return PDIPC_ERR_ARG;
        const size_t n3 = 3 * (size_t)nsim;
        for (size_t q = 0; q < X.size(); ++q) X[q] = (T)Xin[q];
        for (size_t q = 0; q < n3; ++q) V[q] = (T)Vin[q];
        Tangent t;
        t.dk.assign(dkin, dkin + nsim);
        std::vector<T> dX(dXin, dXin + n3), dV(dVin, dVin + n3);
        const T dt = (T)prm.time_step;
        const T invt = (T)((1.0 / (double)dt) * (double)(T)(1.0 - (double)dt));
        for (int s2 = 0; s2 < nsteps; ++s2) {
            // prediction: free vertices start at y = (v + m g) dt + x with rhs0 = y / (dt m)
            t.dP.assign(n3, T(0));
            t.dr0.assign(n3, T(0));
            for (int i = 0; i < nsim; ++i)
                for (int k = 0; k < 3; ++k) {
                    const size_t q = 3 * (size_t)i + k;
                    if (pinFlag[i] != -1) {
                        t.dP[q] = dX[q];
                    } else {
                        const T m = invMass[i] * dt;
                        t.dP[q] = dX[q] + dt * dV[q];
                        t.dr0[q] = (T)(1.0 / (double)(dt * m)) * t.dP[q];
                    }
                }
            tan = &t;
            contactSeen = false;
            const int r = step_once();
            tan = nullptr;
            if (r != PDIPC_OK) return r;
            if (contactSeen) return PDIPC_ERR_STATE;
            for (size_t q = 0; q < n3; ++q) {
                dV[q] = (t.dP[q] - dX[q]) * invt;
                dX[q] = t.dP[q];
            }
        }
        for (size_t q = 0; q < n3; ++q) {
            dXout[q] = (double)dX[q];
            dVout[q] = (double)dV[q];
        }
        return PDIPC_OK;
    }
    // A rollout of nsteps from (Xin, Vin) and its adjoint: gradients of a loss
    // with dL/d(final positions, velocities) = gx, gv with respect to the
    // initial positions, velocities and strain weights.  The state is left at
    // the rollout's end.
    int adjoint_rollout(int nsteps, const double* Xin, const double* Vin, const double* gx, const double* gv,
                        double* gx0, double* gv0, double* gk) {
        if (!initialized) return PDIPC_ERR_STATE;
        if (nsteps < 1) return PDIPC_ERR_ARG;
        const size_t n3 = 3 * (size_t)nsim;
        for (size_t q = 0; q < X.size(); ++q) X[q] = (T)Xin[q];
        for (size_t q = 0; q < n3; ++q) V[q] = (T)Vin[q];
        std::vector<std::vector<T>> xs, vs;
        for (int s2 = 0; s2 < nsteps; ++s2) {
            xs.emplace_back(X.begin(), X.begin() + n3);
            vs.emplace_back(V.begin(), V.begin() + n3);
            const int r = step_once();
            if (r != PDIPC_OK) return r;
        }
        const std::vector<T> xEnd(X.begin(), X.begin() + n3), vEnd(V.begin(), V.begin() + n3);
        std::vector<T> pb(n3), vb(n3), kb(nsim, T(0));
        for (size_t q = 0; q < n3; ++q) {
            pb[q] = (T)gx[q];
            vb[q] = gv ? (T)gv[q] : T(0);
        }
        int r = PDIPC_OK;
        for (int s2 = nsteps - 1; s2 >= 0 && r == PDIPC_OK; --s2) {
            std::copy(xs[s2].begin(), xs[s2].end(), X.begin());
            std::copy(vs[s2].begin(), vs[s2].end(), V.begin());
            r = adjoint_step(pb, vb, kb);
        }
        std::copy(xEnd.begin(), xEnd.end(), X.begin());
        std::copy(vEnd.begin(), vEnd.end(), V.begin());
        if (r != PDIPC_OK) return r;
        for (size_t q = 0; q < n3; ++q) {
            gx0[q] = (double)pb[q];
            gv0[q] = (double)vb[q];
        }
        for (int i = 0; i < nsim; ++i) gk[i] = (double)kb[i];
        return PDIPC_OK;
    }
    int step(int n) {
        if (!initialized) return PDIPC_ERR_STATE;
        st.max_outer_iters = 0;
        st.total_outer_iters = 0;
        for (int s = 0; s < n; ++s) {
            int r = step_once();
            if (r != PDIPC_OK) return r;
        }
        return PDIPC_OK;
    }
};

// ---------------- penalty / discrete-collision path ----------------
// The reference's alternative contact path (PdIpcGpuFunc.cu:2933-3740), never
// called by its step.  Restated on a Sim's tables: candidate lists of the last
// broad phase, collision faces, masses, gravity and pins.  Arithmetic in the
// CCD/contact scalar TC; forces and hits accumulate in candidate (or pair) order.
template <typename TC>
static TC pen_dot(const TC* a, const TC* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
template <typename TC>
static void pen_cross(const TC* a, const TC* b, TC* r) {
    r[0] = a[1] * b[2] - a[2] * b[1];
    r[1] = a[2] * b[0] - a[0] * b[2];
    r[2] = a[0] * b[1] - a[1] * b[0];
}
// project6 (cu:3371-3389)
template <typename TC>
static bool pen_project6(const TC* ax, const TC (*p)[3], const TC (*q)[3]) {
    TC P[3], Q[3];
    for (int j = 0; j < 3; ++j) { P[j] = pen_dot(ax, p[j]); Q[j] = pen_dot(ax, q[j]); }
    TC mx1 = P[0], mn1 = P[0], mx2 = Q[0], mn2 = Q[0];
    for (int j = 1; j < 3; ++j) {
        if (P[j] > mx1) mx1 = P[j];
        if (P[j] < mn1) mn1 = P[j];
        if (Q[j] > mx2) mx2 = Q[j];
        if (Q[j] < mn2) mn2 = Q[j];
    }
    if (mn1 > mx2) return false;
    if (mn2 > mx1) return false;
    return true;
}
// triContact (cu:3391-3468): separating axes n1, m1, e_a x f_b, e_a x n1, f_b x m1
template <typename TC>
static bool pen_tri_contact(const TC (*A)[3], const TC (*B)[3]) {
    TC p[3][3], q[3][3], e[3][3], f[3][3], n1[3], m1[3], ax[3];
    for (int j = 0; j < 3; ++j)
        for (int k = 0; k < 3; ++k) { p[j][k] = A[j][k] - A[0][k]; q[j][k] = B[j][k] - A[0][k]; }
    for (int k = 0; k < 3; ++k) {
        e[0][k] = p[1][k] - p[0][k]; e[1][k] = p[2][k] - p[1][k]; e[2][k] = p[0][k] - p[2][k];
        f[0][k] = q[1][k] - q[0][k]; f[1][k] = q[2][k] - q[1][k]; f[2][k] = q[0][k] - q[2][k];
    }
    pen_cross(e[0], e[1], n1);
    pen_cross(f[0], f[1], m1);
    if (!pen_project6(n1, p, q) || !pen_project6(m1, p, q)) return false;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) { pen_cross(e[a], f[b], ax); if (!pen_project6(ax, p, q)) return false; }
    for (int a = 0; a < 3; ++a) { pen_cross(e[a], n1, ax); if (!pen_project6(ax, p, q)) return false; }
    for (int b = 0; b < 3; ++b) { pen_cross(f[b], m1, ax); if (!pen_project6(ax, p, q)) return false; }
    return true;
}

template <typename SimT>
struct Penalty {
    using T = typename std::remove_reference<decltype(std::declval<SimT>().X)>::type::value_type;
    using TC = typename std::remove_reference<decltype(std::declval<SimT>().collMass)>::type::value_type;
    SimT& s;
    std::vector<TC> F;
    std::vector<int> times;
    explicit Penalty(SimT& sim) : s(sim), F(3 * (size_t)sim.ntot, TC(0)), times(sim.ntot, 0) {}

    void add(int i, TC fx, TC fy, TC fz) { F[3 * (size_t)i] += fx; F[3 * (size_t)i + 1] += fy; F[3 * (size_t)i + 2] += fz; }

    // prediticeDCPositionKernel (cu:2933-2981)
    void predict(const double* X, double* V, double* sn) {
        const TC dt = (TC)s.prm.time_step;
        for (int i = 0; i < s.nsim; ++i) {
            if (s.pinFlag[i] != -1) {
                for (int k = 0; k < 3; ++k) { V[3 * i + k] = 0.0; sn[3 * i + k] = (double)(TC)X[3 * i + k]; }
                continue;
            }
            const TC m = (TC)s.invMass[i] * dt;
            for (int k = 0; k < 3; ++k) {
                TC v = (TC)V[3 * i + k] + m * (TC)s.grav[3 * (size_t)i + k];
                v *= dt;
                sn[3 * i + k] = (double)((TC)X[3 * i + k] + v);
            }
        }
    }
    // computePenaltyForceKernal (cu:3013-3138)
    void ccd(const double* x0, const double* d, TC k) {
        auto one = [&](const std::array<int, 4>& c, bool isPT) {
            if (isPT ? (c[0] == c[1] || c[0] == c[2] || c[0] == c[3])
                     : (c[0] == c[2] || c[0] == c[3] || c[1] == c[2] || c[1] == c[3]))
                return;
            TC x[4][3], dx[4][3], tx[4][3];
            for (int j = 0; j < 4; ++j)
                for (int q = 0; q < 3; ++q) {
                    x[j][q] = (TC)x0[3 * (size_t)c[j] + q];
                    dx[j][q] = (TC)d[3 * (size_t)c[j] + q];
                    tx[j][q] = x[j][q] + dx[j][q];
                }
            const TC slack = (TC)1e-4;
            const bool broad = isPT ? SimT::pt_ccd_broad(x[0], x[1], x[2], x[3], dx[0], dx[1], dx[2], dx[3], slack)
                                    : SimT::ee_ccd_broad(x[0], x[1], x[2], x[3], dx[0], dx[1], dx[2], dx[3], slack);
            if (!broad) return;
            const TC toi = isPT ? s.ccd_pt(x[0], dx[0], x[1], dx[1], x[2], dx[2], x[3], dx[3])
                                : s.ccd_ee(x[0], dx[0], x[1], dx[1], x[2], dx[2], x[3], dx[3]);
            if (!(toi < (TC)1)) return;
            TC dir[3], f[3];
            if (isPT) {
                TC a, b, cc;
                const TC dist = std::sqrt(SimT::vtx_tri(tx[0], tx[1], tx[2], tx[3], &a, &b, &cc, dir));
                for (int q = 0; q < 3; ++q) f[q] = dir[q] * dist * k / (TC)3;
                add(c[0], -f[0] * (TC)3, -f[1] * (TC)3, -f[2] * (TC)3);
                for (int j = 1; j < 4; ++j) add(c[j], f[0], f[1], f[2]);
            } else {
                TC r, ss;
                const TC dist = std::sqrt(SimT::edge_edge_sq(tx[0], tx[1], tx[2], tx[3], &r, &ss, dir));
                for (int q = 0; q < 3; ++q) f[q] = dir[q] * dist * k / (TC)2;
                add(c[0], -f[0], -f[1], -f[2]);
                add(c[1], -f[0], -f[1], -f[2]);
                add(c[2], f[0], f[1], f[2]);
                add(c[3], f[0], f[1], f[2]);
            }
            for (int j = 0; j < 4; ++j) ++times[c[j]];
        };
        for (const auto& c : s.pt) one(c, true);
        for (const auto& c : s.ee) one(c, false);
    }
    // applyPenaltyForceForFloorKernal (cu:3248-3271)
    void floor(const double* x, TC k) {
        for (int i = 0; i < s.nsim; ++i) {
            const TC y = (TC)x[3 * (size_t)i + 1];
            if (y < (TC)0) {
                F[3 * (size_t)i] = 0;
                F[3 * (size_t)i + 1] = -y * k;
                F[3 * (size_t)i + 2] = 0;
                times[i] = 1;
            }
        }
    }
    // computeDcdPenaltyForceKernal (cu:3487-3688) over face pairs
    void dcd(const double* x, const int* fp, long long np, TC k, TC kself) {
        std::vector<int> model(s.ntot, 0);
        {
            int base = 0, id = 0;
            for (int pass = 0; pass < 2; ++pass)
                for (const auto& m : s.models)
                    if ((pass == 0) != m.is_static) {
                        std::fill(model.begin() + base, model.begin() + base + m.nv, id++);
                        base += m.nv;
                    }
        }
        auto normal = [](const TC (*P)[3], TC* n) {
            TC a[3], b[3];
            for (int q = 0; q < 3; ++q) { a[q] = P[1][q] - P[0][q]; b[q] = P[2][q] - P[0][q]; }
            pen_cross(a, b, n);
            const TC len = std::sqrt(pen_dot(n, n));
            for (int q = 0; q < 3; ++q) n[q] /= len;
        };
        // projectToTriangle (cu:3470-3485): the plane through the other triangle's second vertex
        auto push = [&](const std::array<int, 3>& pv, const TC (*P)[3], const std::array<int, 3>& qv, const TC (*Q)[3],
                        const TC* nq, TC stiff) {
            for (int j = 0; j < 3; ++j) {
                TC w[3], dir[3];
                for (int q = 0; q < 3; ++q) w[q] = P[j][q] - Q[1][q];
                const TC c = pen_dot(w, nq);
                for (int q = 0; q < 3; ++q) dir[q] = c * nq[q];
                const TC len = std::sqrt(pen_dot(dir, dir));
                for (int q = 0; q < 3; ++q) dir[q] /= len;
                if (pen_dot(dir, nq) < (TC)0) {
                    const TC f0 = nq[0] * len * stiff, f1 = nq[1] * len * stiff, f2 = nq[2] * len * stiff;
                    add(pv[j], f0, f1, f2);
                    for (int m = 0; m < 3; ++m) add(qv[m], -f0 / (TC)3, -f1 / (TC)3, -f2 / (TC)3);
                    ++times[pv[j]];
                    for (int m = 0; m < 3; ++m) ++times[qv[m]];
                }
            }
        };
        for (long long t = 0; t < np; ++t) {
            const auto& fa = s.faces[fp[2 * t]];
            const auto& fb = s.faces[fp[2 * t + 1]];
            bool shared = false;
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) shared |= fa[i] == fb[j];
            if (shared) continue;
            TC A[3][3], B[3][3];
            for (int j = 0; j < 3; ++j)
                for (int q = 0; q < 3; ++q) { A[j][q] = (TC)x[3 * (size_t)fa[j] + q]; B[j][q] = (TC)x[3 * (size_t)fb[j] + q]; }
            if (!pen_tri_contact<TC>(A, B)) continue;
            const TC stiff = model[fa[0]] == model[fb[0]] ? kself : k;
            TC na[3], nb[3];
            normal(A, na);
            normal(B, nb);
            if (fa[0] < s.nsim) push(fa, A, fb, B, nb, stiff);
            if (fb[0] < s.nsim) push(fb, B, fa, A, na, stiff);
        }
    }
    // uniformPenaltyForceKernal (cu:3140-3195) and the outputs
    void finish(TC damping, double* V, double* force, int* times_out) {
        for (int i = 0; i < s.nsim; ++i) {
            const int h = times[i];
            if (h == 0) continue;
            TC f[3], v[3];
            for (int q = 0; q < 3; ++q) { f[q] = F[3 * (size_t)i + q] / (TC)h; v[q] = (TC)V[3 * i + q]; }
            for (int q = 0; q < 3; ++q) F[3 * (size_t)i + q] = f[q] - damping * v[q];
            const TC len = std::sqrt(pen_dot(f, f));
            for (int q = 0; q < 3; ++q) f[q] /= len;
            const TC cc = pen_dot(v, f);
            for (int q = 0; q < 3; ++q) {
                TC vn = cc * f[q];
                TC vt = v[q] - vn;
                vn *= (TC)-0.4;
                vt = vt * (TC)0.9;
                V[3 * i + q] = (double)(vn + vt);
            }
        }
        for (size_t q = 0; q < F.size(); ++q) force[q] = (double)F[q];
        std::copy(times.begin(), times.end(), times_out);
    }
};

struct Ctx {
    int prec = 0;
    std::unique_ptr<Sim<float, float>> f32;
    std::unique_ptr<Sim<double, double>> f64;
    std::unique_ptr<Sim<float, double>> mix;
};

template <typename F>
static int dispatch(Ctx* c, F&& f) {
    if (!c) return PDIPC_ERR_ARG;
    if (c->f32) return f(*c->f32);
    if (c->f64) return f(*c->f64);
    if (c->mix) return f(*c->mix);
    return PDIPC_ERR_STATE;
}

}  // namespace orc

using orc::Ctx;

extern "C" {

void* orc_create(const pdipc_params* p, int global_form, int threads) {
    if (!p) return nullptr;
    Ctx* c = new Ctx();
    c->prec = p->precision;
    if (p->precision == PDIPC_PREC_FP64) c->f64.reset(new orc::Sim<double, double>(*p, global_form, threads));
    else if (p->precision == PDIPC_PREC_MIXED) c->mix.reset(new orc::Sim<float, double>(*p, global_form, threads));
    else c->f32.reset(new orc::Sim<float, float>(*p, global_form, threads));
    return c;
}

void orc_destroy(void* h) { delete (Ctx*)h; }

static int add_model(Ctx* c, const double* X, int nv, const int* F, int nf, bool st, double density,
                     double ks, double kb, const int* pins, int npins, double kp, int pd) {
    if (!X || !F || nv <= 0 || nf <= 0 || pd <= 0) return PDIPC_ERR_ARG;
    for (int i = 0; i < 3 * nf; ++i)
        if (F[i] < 0 || F[i] >= nv) return PDIPC_ERR_ARG;
    orc::ModelIn m;
    m.X.assign(X, X + 3 * (size_t)nv);
    m.F.assign(F, F + 3 * (size_t)nf);
    m.nv = nv; m.nf = nf; m.is_static = st;
    m.density = density; m.k_stretch = ks; m.k_bend = kb; m.k_pin = kp; m.patch_dim = pd;
    if (pins && npins > 0) m.pins.assign(pins, pins + npins);
    return orc::dispatch(c, [&](auto& s) {
        if (s.initialized) return (int)PDIPC_ERR_STATE;
        s.models.push_back(m);
        return (int)PDIPC_OK;
    });
}

int orc_add_volumetric(void* h, const double* X, int nv, const int* T, int nt, double density, double k_strain,
                       const int* pins, int npins, double kp, int pd) {
    if (!X || !T || nv <= 0 || nt <= 0 || pd <= 0) return PDIPC_ERR_ARG;
    for (int i = 0; i < 4 * nt; ++i)
        if (T[i] < 0 || T[i] >= nv) return PDIPC_ERR_ARG;
    orc::ModelIn m;
    m.X.assign(X, X + 3 * (size_t)nv);
    m.T.assign(T, T + 4 * (size_t)nt);
    m.nv = nv; m.nt = nt; m.is_volumetric = true;
    m.density = density; m.k_strain = k_strain; m.k_pin = kp; m.patch_dim = pd;
    if (pins && npins > 0) m.pins.assign(pins, pins + npins);
    return orc::dispatch((Ctx*)h, [&](auto& s) {
        if (s.initialized) return (int)PDIPC_ERR_STATE;
        s.models.push_back(m);
        return (int)PDIPC_OK;
    });
}

// tet projection of the oracle alone, for the SVD known-answer tests: n tets
// of positions x (12 doubles each: four vertices), row-major Dm^-1 (9 each),
// weights w; out receives 12 doubles per tet (w R G, vertex-major).
int orc_tet_project(int n, const double* x, const double* idm, const double* w, double* out) {
    for (int e = 0; e < n; ++e) {
        double o[4][3];
        const double* p = x + 12 * (size_t)e;
        orc::tet_project<double>(p, p + 3, p + 6, p + 9, idm + 9 * (size_t)e, w[e], o);
        for (int c = 0; c < 4; ++c)
            for (int k = 0; k < 3; ++k) out[12 * (size_t)e + 3 * c + k] = o[c][k];
    }
    return PDIPC_OK;
}

// The triangle strain projection for n triangles: x (9 per triangle: the three
// vertices), idm (4 per triangle, row-major Dm^-1), w (n); out (9 per triangle:
// the three vertices' contributions), FP64.
int orc_tri_project(int n, const double* x, const double* idm, const double* w, double* out) {
    for (int e = 0; e < n; ++e) {
        double o[4][3];
        orc::tri_project<double>(x + 9 * (size_t)e, x + 9 * (size_t)e + 3, x + 9 * (size_t)e + 6, idm + 4 * (size_t)e,
                                 w[e], o);
        for (int c = 0; c < 3; ++c)
            for (int k = 0; k < 3; ++k) out[9 * (size_t)e + 3 * c + k] = o[c][k];
    }
    return PDIPC_OK;
}
int orc_tet_surface(const double* X, int nv, const int* T, int nt, int* faces, int cap, int* nf) {
    std::vector<double> x(X, X + 3 * (size_t)nv);
    std::vector<int> t(T, T + 4 * (size_t)nt);
    auto f = orc::tet_surface(x, t, nt);
    *nf = (int)f.size();
    if ((int)f.size() > cap) return PDIPC_ERR_OVERFLOW;
    for (size_t i = 0; i < f.size(); ++i)
        for (int k = 0; k < 3; ++k) faces[3 * i + k] = f[i][k];
    return PDIPC_OK;
}

int orc_svd3(const double* F, double* U, double* s, double* V) {
    orc::svd3_onesided<double>(F, U, s, V);
    return PDIPC_OK;
}

int orc_add_cloth(void* h, const double* X, int nv, const int* F, int nf, double density, double ks, double kb,
                  const int* pins, int npins, double kp, int pd) {
    return add_model((Ctx*)h, X, nv, F, nf, false, density, ks, kb, pins, npins, kp, pd);
}
// orc_add_cloth with the per-triangle options of pdipc_add_cloth_ex (each array nf values or NULL)
int orc_add_cloth_ex(void* h, const double* X, int nv, const int* F, int nf, double density, double ks, double kb,
                     const int* pins, int npins, double kp, int pd, const double* tri_stretch, double k_tri_strain,
                     const double* tri_strain) {
    int r = add_model((Ctx*)h, X, nv, F, nf, false, density, ks, kb, pins, npins, kp, pd);
    if (r != PDIPC_OK) return r;
    return orc::dispatch((Ctx*)h, [&](auto& s) {
        orc::ModelIn& m = s.models.back();
        if (tri_stretch) m.tri_stretch.assign(tri_stretch, tri_stretch + nf);
        if (tri_strain) m.tri_strain.assign(tri_strain, tri_strain + nf);
        m.k_tri_strain = k_tri_strain;
        return (int)PDIPC_OK;
    });
}
int orc_add_static(void* h, const double* X, int nv, const int* F, int nf, int pd) {
    return add_model((Ctx*)h, X, nv, F, nf, true, 0, 0, 0, nullptr, 0, 0, pd);
}
int orc_initialize(void* h) { return orc::dispatch((Ctx*)h, [](auto& s) { return s.initialize(); }); }
int orc_step(void* h, int n) { return orc::dispatch((Ctx*)h, [&](auto& s) { return s.step(n); }); }

int orc_get_positions(void* h, double* out) {
    return orc::dispatch((Ctx*)h, [&](auto& s) {
        if (!s.initialized || !out) return (int)PDIPC_ERR_STATE;
        for (size_t q = 0; q < s.X.size(); ++q) out[q] = (double)s.X[q];
        return (int)PDIPC_OK;
    });
}
int orc_get_velocities(void* h, double* out) {
    return orc::dispatch((Ctx*)h, [&](auto& s) {
        if (!s.initialized || !out) return (int)PDIPC_ERR_STATE;
        for (size_t q = 0; q < s.V.size(); ++q) out[q] = (double)s.V[q];
        return (int)PDIPC_OK;
    });
}
int orc_set_state(void* h, const double* X, const double* V) {
    return orc::dispatch((Ctx*)h, [&](auto& s) {
        using T = typename std::remove_reference<decltype(s.X)>::type::value_type;
        if (!s.initialized || !X) return (int)PDIPC_ERR_STATE;
        for (size_t q = 0; q < s.X.size(); ++q) s.X[q] = (T)X[q];
        if (V)
            for (size_t q = 0; q < s.V.size(); ++q) s.V[q] = (T)V[q];
        return (int)PDIPC_OK;
    });
}
int orc_get_stats(void* h, pdipc_stats* out) {
    return orc::dispatch((Ctx*)h, [&](auto& s) {
        if (!out) return (int)PDIPC_ERR_ARG;
        *out = s.st;
        return (int)PDIPC_OK;
    });
}

// Broad phase on caller positions (same contract as pdipc_stage_broadphase).
int orc_broadphase(void* h, const double* xo, const double* dx, int* pairs, long long cap_pairs, long long* n_pairs,
                   int* pt, long long cap_pt, long long* n_pt, int* ee, long long cap_ee, long long* n_ee) {
    return orc::dispatch((Ctx*)h, [&](auto& s) {
        using T = typename std::remove_reference<decltype(s.X)>::type::value_type;
        if (!s.initialized) return (int)PDIPC_ERR_STATE;
        std::vector<T> a(s.X.size()), b(s.X.size());
        for (size_t q = 0; q < a.size(); ++q) { a[q] = (T)xo[q]; b[q] = (T)dx[q]; }
        s.broadphase(a, b);
        *n_pairs = (long long)s.pairs.size();
        *n_pt = (long long)s.pt.size();
        *n_ee = (long long)s.ee.size();
        if ((long long)s.pairs.size() > cap_pairs || (long long)s.pt.size() > cap_pt || (long long)s.ee.size() > cap_ee)
            return (int)PDIPC_ERR_OVERFLOW;
        for (size_t i = 0; i < s.pairs.size(); ++i) { pairs[2 * i] = s.pairs[i][0]; pairs[2 * i + 1] = s.pairs[i][1]; }
        for (size_t i = 0; i < s.pt.size(); ++i) for (int k = 0; k < 4; ++k) pt[4 * i + k] = s.pt[i][k];
        for (size_t i = 0; i < s.ee.size(); ++i) for (int k = 0; k < 4; ++k) ee[4 * i + k] = s.ee[i][k];
        return (int)PDIPC_OK;
    });
}
int orc_morton(void* h, unsigned long long* codes, int* order, int cap) {
    return orc::dispatch((Ctx*)h, [&](auto& s) {
        if (!s.initialized) return (int)PDIPC_ERR_STATE;
        if (cap < s.npatch) return (int)PDIPC_ERR_OVERFLOW;
        for (int i = 0; i < s.npatch; ++i) { codes[i] = s.morton[i]; order[i] = s.order[i]; }
        return (int)PDIPC_OK;
    });
}
int orc_toi(void* h, const double* x0, const double* x1, double* tpt, double* tee, double* tg) {
    return orc::dispatch((Ctx*)h, [&](auto& s) {
        using T = typename std::remove_reference<decltype(s.X)>::type::value_type;
        if (!s.initialized) return (int)PDIPC_ERR_STATE;
        std::vector<T> a(s.X.size()), b(s.X.size());
        for (size_t q = 0; q < a.size(); ++q) { a[q] = (T)x0[q]; b[q] = (T)x1[q]; }
        std::vector<double> vp, ve;
        double g = (double)s.global_toi(a, b, &vp, &ve);
        if (tpt) std::copy(vp.begin(), vp.end(), tpt);
        if (tee) std::copy(ve.begin(), ve.end(), tee);
        if (tg) *tg = g;
        return (int)PDIPC_OK;
    });
}
int orc_contact(void* h, const double* x, double* diag, double* rhs, long long* n_active) {
    return orc::dispatch((Ctx*)h, [&](auto& s) {
        using T = typename std::remove_reference<decltype(s.X)>::type::value_type;
        if (!s.initialized) return (int)PDIPC_ERR_STATE;
        std::vector<T> a(s.X.size());
        for (size_t q = 0; q < a.size(); ++q) a[q] = (T)x[q];
        long long na = s.contacts(a);
        if (n_active) *n_active = na;
        for (int i = 0; i < s.ntot; ++i) diag[i] = (double)s.collDiag[i];
        for (size_t q = 0; q < s.collRhs.size(); ++q) rhs[q] = (double)s.collRhs[q];
        return (int)PDIPC_OK;
    });
}

// One of the initialised tables by name, for the harness that runs the
// reference's own kernels on the same inputs (oracle/ref_harness.cpp): integer
// tables go to iout, real ones to dout (either may be NULL to ask for the
// size).  Returns the entry count, or -1 for an unknown name.
long long orc_table(void* h, const char* name, double* dout, int* iout, long long cap) {
    long long n = -1;
    orc::dispatch((Ctx*)h, [&](auto& s) {
        if (!s.initialized || !name) return (int)PDIPC_ERR_STATE;
        const std::string k(name);
        auto ints = [&](const std::vector<int>& v) {
            n = (long long)v.size();
            if (iout && n <= cap) std::copy(v.begin(), v.end(), iout);
        };
        auto reals = [&](const auto& v) {
            n = (long long)v.size();
            if (dout && n <= cap)
                for (long long q = 0; q < n; ++q) dout[q] = (double)v[q];
        };
        if (k == "lOff") ints(s.lOff);
        else if (k == "lNum") ints(s.lNum);
        else if (k == "lNbr") ints(s.lNbr);
        else if (k == "pinFlag") ints(s.pinFlag);
        else if (k == "nPtr") ints(s.nPtr);
        else if (k == "nCol") ints(s.nCol);
        else if (k == "r2Ptr") ints(s.r2Ptr);
        else if (k == "r2Col") ints(s.r2Col);
        else if (k == "r2Const") ints(s.r2Const);
        else if (k == "r2First") ints(s.r2First);
        else if (k == "pathPtr") ints(s.pathPtr);
        else if (k == "pathK") ints(s.pathK);
        else if (k == "lStrain") reals(s.lStrain);
        else if (k == "lRest") reals(s.lRest);
        else if (k == "lLbo") reals(s.lLbo);
        else if (k == "lBend") reals(s.lBend);
        else if (k == "lBendT") reals(s.lBendT);
        else if (k == "curvNorm") reals(s.curvNorm);
        else if (k == "invMass") reals(s.invMass);
        else if (k == "grav") reals(s.grav);
        else if (k == "pinStiff") reals(s.pinStiff);
        else if (k == "Delastic") reals(s.Delastic);
        else if (k == "nVal") reals(s.nVal);
        else if (k == "pathA") reals(s.pathA);
        else if (k == "collMass") reals(s.collMass);
        else if (k == "Xrest") reals(s.Xrest_all);
        return (int)PDIPC_OK;
    });
    return n;
}

int orc_penalty_predict(void* h, const double* X, double* V, double* sn) {
    return orc::dispatch((Ctx*)h, [&](auto& s) {
        if (!s.initialized) return (int)PDIPC_ERR_STATE;
        orc::Penalty<std::remove_reference_t<decltype(s)>> p(s);
        p.predict(X, V, sn);
        return (int)PDIPC_OK;
    });
}
// kind: 0 CCD candidates of the last broad phase (x, dir), 1 floor (x), 2 face pairs (x)
int orc_penalty(void* h, int kind, const double* x, const double* dir, const int* fp, long long np, double k,
                double kself, double damping, double* V, double* force, int* times) {
    return orc::dispatch((Ctx*)h, [&](auto& s) {
        if (!s.initialized) return (int)PDIPC_ERR_STATE;
        using P = orc::Penalty<std::remove_reference_t<decltype(s)>>;
        using TC = typename P::TC;
        P p(s);
        if (kind == 0) p.ccd(x, dir, (TC)k);
        else if (kind == 1) p.floor(x, (TC)k);
        else {
            for (long long i = 0; i < 2 * np; ++i)
                if (fp[i] < 0 || fp[i] >= (int)s.faces.size()) return (int)PDIPC_ERR_ARG;
            p.dcd(x, fp, np, (TC)k, (TC)kself);
        }
        p.finish((TC)damping, V, force, times);
        return (int)PDIPC_OK;
    });
}

int orc_stage_pd(void* h, const double* X, const double* V, double* out) {
    return orc::dispatch((Ctx*)h, [&](auto& s) { return s.stage_pd(X, V, out); });
}

// Forward-mode tangent of a contact-free rollout (FP64, two-sweep form only).
int orc_tangent_rollout(void* h, int nsteps, const double* X, const double* V, const double* dX, const double* dV,
                        const double* dk, double* dXout, double* dVout) {
    Ctx* c = (Ctx*)h;
    if (!c || !X || !V || !dX || !dV || !dk || !dXout || !dVout) return PDIPC_ERR_ARG;
    if (!c->f64) return PDIPC_ERR_STATE;
    return c->f64->tangent_rollout(nsteps, X, V, dX, dV, dk, dXout, dVout);
}

// Discrete adjoint of a contact-free rollout (FP64, two-sweep form only).
int orc_adjoint_rollout(void* h, int nsteps, const double* X, const double* V, const double* gx, const double* gv,
                        double* gx0, double* gv0, double* gk) {
    Ctx* c = (Ctx*)h;
    if (!c || !X || !V || !gx || !gx0 || !gv0 || !gk) return PDIPC_ERR_ARG;
    if (!c->f64) return PDIPC_ERR_STATE;
    return c->f64->adjoint_rollout(nsteps, X, V, gx, gv, gx0, gv0, gk);
}

// Topology of one standalone mesh, for the known-answer tests on the
// reference example's cached boundary.dat / patchInfo.dat.
// edges_out: 2*ne ints (cap_e pairs); patch_faces/patch_off: faces per patch
// (CSR, patch_off has npatch+1 entries, cap_p patches, cap_pf faces).
int orc_mesh_topology(const double* X, int nv, const int* F, int nf, int patch_dim, int* edges_out, int cap_e,
                      int* ne, int* patch_off, int cap_p, int* patch_faces, int cap_pf, int* np,
                      int* owned_pts_off, int* owned_pts, int* owned_edges_off, int* owned_edges) {
    orc::Topology t;
    t.nv = nv;
    t.nf = nf;
    t.faces.resize(nf);
    for (int f = 0; f < nf; ++f) t.faces[f] = {F[3 * f], F[3 * f + 1], F[3 * f + 2]};
    orc::build_edges(t);
    if (!orc::build_ownership(t)) return PDIPC_ERR_ARG;
    std::vector<double> Xv(X, X + 3 * (size_t)nv);
    orc::build_patches(t, Xv, patch_dim);
    *ne = (int)t.edges.size();
    *np = (int)t.patches.size();
    if (*ne > cap_e || *np > cap_p) return PDIPC_ERR_OVERFLOW;
    for (int e = 0; e < *ne; ++e) { edges_out[2 * e] = t.edges[e][0]; edges_out[2 * e + 1] = t.edges[e][1]; }
    int q = 0;
    patch_off[0] = 0;
    for (int p = 0; p < *np; ++p) {
        for (int f : t.patches[p]) {
            if (q >= cap_pf) return PDIPC_ERR_OVERFLOW;
            patch_faces[q++] = f;
        }
        patch_off[p + 1] = q;
    }
    if (owned_pts_off) {
        int a = 0, b = 0;
        owned_pts_off[0] = 0;
        owned_edges_off[0] = 0;
        for (int f = 0; f < nf; ++f) {
            for (int v : t.face_owned_points[f]) owned_pts[a++] = v;
            for (int e : t.face_owned_edges[f]) owned_edges[b++] = e;
            owned_pts_off[f + 1] = a;
            owned_edges_off[f + 1] = b;
        }
    }
    return PDIPC_OK;
}

}  // extern "C"
