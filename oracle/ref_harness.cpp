// ref_harness.cpp — runs the reference's own PD-IPC kernels on the host
// (oracle/build_ref.py builds it with oracle/cuda_emu.h; test infrastructure).
//
// The kernels come byte for byte from Simulator/PD-IPC/PdIpcGpuFunc.cu (the
// copy in oracle/_ref/gen).  Each entry point below restates one of the
// reference's __host__ wrappers or host sequences: which kernels, in which
// order, with which launch shape and which buffer rotation; the arithmetic is
// the reference's.  Arrays are qeal (float, or double in the
// USE_DOUBLE_PRECISION build) in the reference's layouts, filled by the caller
// (oracle/refkern.py) from the oracle's initialised tables.
#include "PdIpcGpuFunc_kernels.cu"

// the two dynamic shared arrays of the broad-phase kernels (never launched here)
namespace PD_IPC {
thread_local qeal bbox[6 * 1024];
thread_local int eachPatchICPairsNum[1024];
}

using namespace PD_IPC;

namespace {

dim3 grid_for(long long n, unsigned block) { return dim3((unsigned)((n + block - 1) / block)); }

}  // namespace

extern "C" {

int ref_qeal_bytes(void) { return (int)sizeof(qeal); }

// predictiveHost (PdIpcGpuFunc.cu:150-182) with simPointsBlockSize = 128
// (PdIpcSimulator.cpp:424-425).  X, V, initRhs: 3n; inertDiag, invMass: n;
// grav, mouse, penalty: 3n; flag: n (-1 = free).
void ref_predict(int n, qeal dt, qeal* X, qeal* V, qeal* initRhs, qeal* inertDiag, qeal* grav, qeal* mouse,
                 qeal* penalty, qeal* invMass, const int* flag) {
    cuemu::launch(grid_for(n, THREADS_NUM_128), dim3(THREADS_NUM_128), [&]() {
        predictiveKernel(n, dt, X, V, initRhs, inertDiag, grav, mouse, penalty, invMass, flag);
    });
}

// PdIpcSimulator::doLocalProjection (PdIpcSimulator.cpp:1624-1681) for a cloth
// scene: rhs = initRhs, the strain and bending kernel (cu:627-728, block 128,
// cpp:428-429), the collision rhs (the cublasSaxpy of cpp:1668, when
// collRhs is not NULL) and the position constraints (cu:764-790, block 128,
// cpp:430-431).  rhs, initRhs, collRhs: 3n; pins: npins vertex ids with their
// stiffness; restPoints: 3 x (all points).
void ref_local_projection(int n, const qeal* initRhs, const qeal* strain, const qeal* bending, const int* nbrList,
                          const int* nbrNum, const int* nbrOffset, const qeal* restLen, const qeal* lbo,
                          const qeal* curvNorm, qeal* points, const qeal* collRhs, int npins, qeal* restPoints,
                          const int* pinIndex, const qeal* pinStiff, qeal* rhs) {
    std::memcpy(rhs, initRhs, sizeof(qeal) * 3 * (size_t)n);
    cuemu::launch(grid_for(n, THREADS_NUM_128), dim3(THREADS_NUM_128), [&]() {
        solveClothPointsStrainAndBendingConstraintKernel(n, strain, bending, nbrList, nbrNum, nbrOffset, restLen, lbo,
                                                         curvNorm, points, rhs);
    });
    if (collRhs)
        for (size_t q = 0; q < 3 * (size_t)n; ++q) rhs[q] = (qeal)1 * collRhs[q] + rhs[q];
    if (npins > 0)
        cuemu::launch(grid_for(npins, THREADS_NUM_128), dim3(THREADS_NUM_128), [&]() {
            solvePointsConstraintKernel(npins, restPoints, pinIndex, pinStiff, rhs);
        });
}

// updateSuperJacobiOperatorsHost (cu:976-1038) with the launch shapes of
// PdIpcSimulator.cpp:1121-1131: R1 operators, R2 path operators, R2 row
// operators, from the system diagonal sysDiag (n).
void ref_update_operators(int nR1, qeal* sysDiag, qeal* r1Value, int* r1Dii, qeal* r1Ops, int nR2Paths, qeal* aijk,
                          int* r2Dii, int* r2Djj, qeal* r2PathOps, int nR2, int* r2RowNum, int* r2RowOffset,
                          qeal* r2Const, int* r2First, qeal* r2RowOps) {
    cuemu::launch(grid_for(nR1, THREADS_NUM_128), dim3(THREADS_NUM_128),
                  [&]() { updateR1OperatorsKernel(nR1, sysDiag, r1Value, r1Dii, r1Ops); });
    cuemu::launch(grid_for(nR2Paths, THREADS_NUM_128), dim3(THREADS_NUM_128),
                  [&]() { updateR2OperatorsKernel(nR2Paths, sysDiag, aijk, r2Dii, r2Djj, r2PathOps); });
    cuemu::launch(grid_for(nR2, THREADS_NUM_128), dim3(THREADS_NUM_128), [&]() {
        updateR2RowOperatorsKernel(nR2, r2RowNum, r2RowOffset, r1Ops, r2PathOps, r2Const, r2First, r2RowOps);
    });
}

// chebyshevJacobiR2SolverHost (cu:1245-1346): the first term, one plain R2
// step, then maxIter-1 Chebyshev steps with rho 0.9992, the three iterate
// buffers rotated after every step; launch shapes of PdIpcSimulator.cpp:
// 1133-1137.  curX holds x0 on entry and, for maxIter = 15 (15 rotations of a
// 3-cycle), the result on exit; preX and nextX are scratch of 3n.
void ref_chebyshev_r2(int maxIter, int n, qeal* sysDiag, qeal* rhs, qeal* r1Ops, int* r1Index, int* r1Num,
                      int* r1Offset, qeal* firstTerm, qeal* preX, qeal* curX, qeal* nextX, qeal* r2RowOps,
                      int* r2Index, int* r2Num, int* r2Offset) {
    const long long dims = 3ll * n;
    const dim3 ftGrid = grid_for(dims * R2_SPAN, THREADS_NUM_192), itGrid = grid_for(dims * R2_SPAN, THREADS_NUM_192);
    cuemu::launch(ftGrid, dim3(THREADS_NUM_192), [&]() {
        superJacobiR2FirstTermKernel(n, sysDiag, rhs, r1Ops, r1Index, r1Num, r1Offset, firstTerm);
    });
    cuemu::launch(itGrid, dim3(THREADS_NUM_192), [&]() {
        superJacobiR2IterationKernel(n, curX, nextX, firstTerm, r2RowOps, r2Index, r2Num, r2Offset);
    });
    SwapPtr(curX, preX);
    SwapPtr(curX, nextX);
    qeal rho = 0.9992;
    rho *= rho;
    qeal omega = 2.0 / (2 - rho);
    for (int iter = 1; iter < maxIter; iter++) {
        cuemu::launch(itGrid, dim3(THREADS_NUM_192), [&]() {
            chebyshevJacobiR2IterationKernel(n, omega, firstTerm, r2RowOps, r2Index, r2Num, r2Offset, preX, curX,
                                             nextX);
        });
        omega = 4.0 / (4 - rho * omega);
        SwapPtr(curX, preX);
        SwapPtr(curX, nextX);
    }
}

// Per-candidate time of impact as getImpactOfTimeKernel (cu:2610-2704)
// decides it for one candidate (shared-vertex skip, the swept-box test with
// slack 5e-3, then the additive CCD), through the reference's own device
// functions; 1 where the kernel skips the candidate.  list: 5 ints per
// candidate [type, v0, v1, v2, v3]; x0, x1: 3 x (all points).
void ref_toi_per_candidate(int n, const int* list, const qeal* x0, const qeal* x1, qeal* toi) {
    for (int tid = 0; tid < n; ++tid) {
        const int type = list[5 * tid];
        int id[4];
        for (int c = 0; c < 4; ++c) id[c] = 3 * list[5 * tid + 1 + c];
        qeal p[4][3], d[4][3];
        for (int c = 0; c < 4; ++c)
            for (int k = 0; k < 3; ++k) {
                p[c][k] = x0[id[c] + k];
                d[c][k] = x1[id[c] + k] - p[c][k];
            }
        qeal t = 1.0;
        if (type == 0) {
            if (!(id[0] == id[1] || id[0] == id[2] || id[0] == id[3]) &&
                point_triangle_ccd_broadphase(p[0], p[1], p[2], p[3], d[0], d[1], d[2], d[3], 5e-3))
                t = ccdVertexTriangleToi(tid, p[0], d[0], p[1], d[1], p[2], d[2], p[3], d[3]);
        } else if (type == 1) {
            if (!(id[0] == id[2] || id[0] == id[3] || id[1] == id[2] || id[1] == id[3]) &&
                edge_edge_ccd_broadphase(p[0], p[1], p[2], p[3], d[0], d[1], d[2], d[3], 5e-3))
                t = ccdEdgeEdgeToi(tid, p[0], d[0], p[1], d[1], p[2], d[2], p[3], d[3]);
        }
        toi[tid] = t;
    }
}

// getImpactOfTimeHost (cu:2706-2742): the kernel with 512-thread blocks, each
// block's minimum (x 0.98 when below 1), then the smallest of them (the
// reference's cublasIsamin over positive values).  blockToi: one per block.
qeal ref_toi_global(int n, int* list, qeal* x0, qeal* x1, qeal* blockToi) {
    if (n == 0) return 1.0;
    const dim3 grid = grid_for(n, THREADS_NUM);
    cuemu::launch(grid, dim3(THREADS_NUM), [&]() { getImpactOfTimeKernel(n, list, x0, x1, blockToi); });
    qeal best = blockToi[0];
    for (unsigned b = 1; b < grid.x; ++b)
        if (std::fabs(blockToi[b]) < std::fabs(best)) best = blockToi[b];
    return best;
}

// setCollisionConstraintsHost (cu:2894-2930): the kernel with 128-thread
// blocks over the candidate list at positions x; diag (all points) and rhs
// (3 x all points) must start at zero (cpp:1733-1734).
void ref_contact(qeal dHat, qeal kappa, qeal dt, int n, int* list, qeal* x, qeal* mass, qeal* diag, qeal* rhs,
                 int nTotal) {
    if (n == 0) return;
    const qeal dHat2 = dHat * dHat;
    cuemu::launch(grid_for(n, THREADS_NUM_128), dim3(THREADS_NUM_128), [&]() {
        setCollisionConstraintsKernel(dHat, dHat2, kappa, dt, n, list, x, mass, diag, rhs, nTotal);
    });
}

}  // extern "C"
