// host_tables.h — init-time tables of the PD-IPC step, built on the host in
// FP64 and uploaded once in the working precision.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace pdipc {

struct ModelInput {
    std::vector<double> X;  // 3*nv
    std::vector<int> F;     // 3*nf (cloth, static); the boundary surface is derived for a volumetric model
    std::vector<int> T;     // 4*nt tetrahedra (volumetric model)
    int nv = 0, nf = 0, nt = 0;
    bool is_static = false;
    bool is_volumetric = false;
    double density = 0, k_stretch = 0, k_bend = 0, k_pin = 0;
    double k_strain = 0, k_volume = 0;  // volumetric: strain and (unused by the reference) volume stiffness
    // cloth: per-triangle stretch stiffness (nf, or empty: k_stretch), mapped to
    // the per-vertex spring weight as the mean over a vertex's triangles
    std::vector<double> tri_stretch;
    // cloth: per-triangle strain-limit weight per unit rest area (nf, or empty:
    // k_tri_strain everywhere; no constraint where it is 0)
    double k_tri_strain = 0;
    std::vector<double> tri_strain;
    std::vector<int> pins;
    int patch_dim = 10;
};

// Everything the device needs, in global vertex numbering: every cloth model
// in add order, then every static model in add order.
struct HostTables {
    int nsim = 0, ntot = 0;
    std::vector<double> X;  // 3*ntot initial positions
    std::vector<int> vertexModel;  // ntot: position of the vertex's model in the global order

    // per simulated vertex
    std::vector<double> mass;       // lumped area/3 * density (PdIpcClothModel.h:177-195)
    std::vector<double> Delastic;   // diagonal of the elastic system matrix (setupHessMat)
    std::vector<double> curvNorm;   // rest mean-curvature norm |sum lbo x|
    std::vector<double> strain;     // strain stiffness (slot 0 of the reference's per-slot list)
    std::vector<int> pinSlot;       // -1 or index into pinK
    std::vector<double> pinK;

    // local-step stencil per simulated vertex: [self, neighbours ascending]
    std::vector<int> lPtr, lNbr;
    std::vector<double> lRest, lLbo, lBend, lBendT;

    // tetrahedral strain constraints (solveVolumetricStrainConstraintKernel,
    // PdIpcGpuFunc.cu:439-599): global vertex ids, row-major Dm^-1 (9 per tet),
    // weight k_strain * |V|; vertex -> (tet << 2 | slot) incidence, ascending tet
    int ntet = 0;
    std::vector<int> tets;        // 4 per tet
    std::vector<double> tetIdm;   // 9 per tet
    std::vector<double> tetW;
    std::vector<int> vtPtr, vtIdx;

    // off-diagonal system matrix N = -A_offdiag, CSR with ascending columns
    std::vector<int> nPtr, nCol;
    std::vector<double> nVal;

    // collision topology
    std::vector<int> faces;  // 3 per face
    std::vector<int> edges;  // 2 per edge
    std::vector<int> pfPtr, pfIdx;  // faces of each patch
    std::vector<int> ppPtr, ppIdx;  // owned points of each patch (ascending)
    std::vector<int> pePtr, peIdx;  // owned edges of each patch (ascending)
    std::vector<int> pxPtr, pxIdx;  // every vertex touched by the patch's faces
    std::vector<uint8_t> pStatic;
    int npatch = 0;
    std::vector<double> collMassSim;  // mass for sim vertices; static ones use static_mass
};

// Builds the tables; returns an empty string or an error message.
std::string build_host_tables(const std::vector<ModelInput>& models, double gravity, HostTables& out);

// Topology of one mesh (exposed for the known-answer tests on the reference
// example's cached topology files).
struct MeshTopology {
    std::vector<int> edges;                        // 2 per edge, sorted unique (min,max)
    std::vector<std::vector<int>> point_edges;     // per vertex, ascending edge id
    std::vector<std::vector<int>> edge_faces;      // per edge, ascending face id
    std::vector<std::vector<int>> face_edges_own;  // edges owned by each face
    std::vector<std::vector<int>> face_points_own; // points owned by each face
    std::vector<std::vector<int>> patches;         // faces of each non-empty grid cell
};
std::string build_mesh_topology(const double* X, int nv, const int* F, int nf, int patch_dim, MeshTopology& t);

// Boundary surface of a tetrahedral mesh: faces of exactly one tet, turned to
// face away from that tet's centroid (PdIpcVolumetricModel::registerBoundaryInfo,
// PdIpcVolumetricModel.h:27-112), in ascending order of their sorted vertex triple.
std::string tet_boundary_faces(const double* X, int nv, const int* T, int nt, std::vector<int>& faces);

}  // namespace pdipc
