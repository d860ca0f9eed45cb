// persistent.h — launch plan and arguments of the persistent PD solve
// (pd_persistent.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "common.cuh"

namespace pdipc {

constexpr int kMaxCheby = 64;
// warps per CTA of the persistent solve (its launch bound: 72 registers per thread)
constexpr int kMaxPersistWarps = 28;
// band path: the column-offset patterns travel in the launch's parameter space
// (read through the constant cache, off the shared-memory pipe)
constexpr int kParamPatterns = 4096;

// Slot order of the persistent solve: in every window of 64 rows, its 32 even
// rows, then its 32 odd rows (a fixed bijection of [0, 64 ceil(n / 64))).  The
// matrix slices and the rows' assignment to threads follow slot order, so the
// 32 rows of a warp are the even or the odd rows of one window.  A structured
// triangle mesh whose quads alternate their diagonal has two stencil shapes
// that alternate with the row parity: in slot order a warp's rows share one
// shape, so its column offsets are one constant-cache address and its k-th
// entries read rows two apart.  The iterates and the band in shared memory are
// in row order with swz applied: bit 0 of every row in an odd 32-row block is
// flipped, so 32 rows two apart (spanning two or three 32-row blocks) fall in
// 32 distinct shared-memory banks.  swz maps every 64-row window onto itself.
__host__ __device__ __forceinline__ int slot_of(int row) { return (row & ~63) | ((row & 1) << 5) | ((row >> 1) & 31); }
__host__ __device__ __forceinline__ int row_of(int slot) {
    return (slot & ~63) | ((slot >> 5) & 1) | ((slot & 31) << 1);
}
__host__ __device__ __forceinline__ int swz(int row) { return row ^ ((row >> 5) & 1); }

// One configuration of the persistent solve, as the autotuner names it.
struct PlanChoice {
    int rows_per_thread = 0;  // R, slices per warp; 0: one launch per sweep instead
    bool band = false;        // the iterate's column band in shared memory (correction form)
    bool l1_gather = true;
    bool local_sync = true;
};

// A launch of the plan: CTAs [cta_lo, cta_hi], rows [row0, row1).
struct PersistGroup {
    int cta_lo = 0, cta_hi = -1;
    int row0 = 0, row1 = 0;
};

struct PersistPlan {
    bool enabled = false;
    bool matrix_in_smem = false;  // values in shared memory, columns from the pattern table
    bool l1_gather = true;        // gathers may hit in L1 (else L2-only .cg loads)
    bool local_sync = true;       // CTAs wait for their row-exchange neighbours only (else grid barrier)
    int ctas = 0;
    int threads = 0;               // multiple of 32
    int rows_per_thread = 1;       // R: slices per warp
    int slices_per_cta = 0;
    size_t smem_bytes = 0;
    int patterns = 0;
    int pattern_width = 0;
    int own_max = 0;              // > 0: the CTA's column band lives in shared memory (needs local_sync)
    int halo_max = 0;
    bool band_param = true;       // band path: offset patterns in parameter space (else per CTA in shared memory)
};

// T: solver scalar; S: state scalar (T in the direct form, double in the
// correction form).
template <typename T, typename S>
struct PersistArgs {
    int nsim;
    int nslot;  // 64 ceil(nsim / 64): slots of the iterates
    int lg;
    int cheby;
    T relax;
    T omega[kMaxCheby];  // omega[it] of Chebyshev step it (it >= 1)
    long long timeout;   // barrier wait limit in clock cycles
    // state (correction form: Ph, Pl the float-float mirror of P)
    V4<S>* P;
    V4<T>* Ph;
    V4<T>* Pl;
    const V4<S>* Pold;
    const V4<S>* Xrest;
    const V4<S>* Rhs0;
    const V4<T>* CollRhs;
    const V4<T>* PinRhs;
    V4<T>* Aq;
    V4<T>* GX;   // second-sweep iterates (odd steps in GX2 on the band path), at swz(row) [nslot]
    V4<T>* GX2;
    V4<T>* GY;   // first-sweep iterates, at swz(row) [nslot]
    const T* Delastic;
    const T* Dinert;
    const T* CollDiag;
    const int* PinFlag;
    const T* PinK;
    // local step stencils: counts from the CSR row pointer, neighbours and
    // weights from the SELL-32 copy (neighbour k of row i at tOff[i >> 5] +
    // 32 k + (i & 31)), self weights per row
    const int* lPtr;
    const int* tOff;
    const int* tNbr;
    const T* tRest;
    const T* tLbo;
    const T* tBendT;
    const T* tBend0;
    const T* tLbo0;
    const T* Strain;
    const T* CurvNorm;
    // tetrahedral strain constraints: CTA c projects tets ctaTetIdx[ctaTetPtr[c] ..
    // ctaTetPtr[c + 1]) (those whose first vertex it owns) in its curvature phase;
    // rows gather their projections through vtPtr / vtIdx in the residual phase
    int ntet;
    const int4* Tets;
    const T* TetIdm;
    const T* TetW;
    V4<T>* TetOut;
    const int* vtPtr;
    const int* vtIdx;
    const int* ctaTetPtr;
    const int* ctaTetIdx;
    // matrix, SELL-32 over slots: slice s holds the rows of slots [32 s, 32 s + 32)
    const int* sliceEntry;  // SELL entry offset of every slice
    const int* sliceLen;
    const int* sCol;        // absolute columns, row order (matrix streamed from global)
    const T* sVal;
    const int* ctaSlice;    // first slice of each CTA (ctas + 1; even: CTAs own whole 64-row windows)
    const int* ctaEntry;    // first SELL entry of each CTA (ctas + 1)
    const int* rowPattern;  // pattern id of every row in the whole table (kMode 2)
    const int* rowPatLocal; // pattern id of every row in its CTA's table (kModes 1 and 3)
    const int* ctaPat;      // first pattern of every CTA's table in patLocal (ctas + 1)
    const int16_t* patLocal;  // the CTAs' tables, [patterns x pattern_width] column offsets each
    int16_t patc[kParamPatterns];  // kMode 2: the whole table (patterns x pattern_width <= kParamPatterns)
    int patW;
    // grid barrier: [0] generation, [1] arrival counter
    unsigned* bar;
    unsigned* err;
    // stop of the outer loop (null outside a step): once set, the launch
    // returns at entry, before any phase, and publishes nothing
    const OuterGate* gate;
    // neighbour synchronisation (nbr != null): CTA c publishes the number of
    // phases it completed, epoch0 + k, in flags[c] and, before phase k + 1,
    // waits until every CTA in [nbr[c].x, nbr[c].y] has published epoch0 + k
    unsigned* flags;
    const int2* nbr;
    unsigned epoch0;
    // band of the iterate in shared memory (band != null, matrix in shared
    // memory, neighbour synchronisation): CTA c's matrix rows read the rows
    // [band[c].x, band[c].y) (whole 64-row windows).  Its own rows stay in three planar arrays of
    // ownMax floats that its threads update after every sweep; the halo (the
    // columns outside its own rows, at most haloMax vertices) is copied from
    // global memory in two bulk copies per sweep
    const int2* band;
    int ownMax;
    int haloMax;
    // Launch groups: one plan covers every row and may hold more CTAs than
    // are co-resident; a launch runs CTAs [ctaLo, ctaHi] (blockIdx.x + ctaLo)
    // and updates rows [row0, row1) only, whole independent instances, so no
    // CTA waits for one outside the group (a CTA shared by two groups runs in
    // both launches, each time for its own rows).  nphases: the phase count the
    // host reserves per launch (epoch0 + nphases lies above every phase).
    int ctaLo;
    int ctaHi;
    int row0;
    int row1;
    unsigned nphases;
    // per-instance stopping (instStop != null): rows of a stopped instance
    // are not updated; a CTA without rows to update publishes its last phase
    // and returns (neighbour synchronisation only)
    const int* vInst;
    const unsigned* instStop;
};

// nullptr: no such kernel (tets need L1 gathers and at most two rows per thread;
// the band path runs the correction form).  band_param: the band path reads the
// offset patterns from parameter space (else each CTA's own table in shared memory).
const void* persistent_kernel(bool correction, bool matrix_in_smem, bool band, bool band_param, bool l1_gather,
                              int rows_per_thread, bool tets);
// the band variants (correction form), compiled in their own translation unit
const void* persistent_band_kernel(bool param_patterns, bool l1_gather, int rows_per_thread, bool tets);
// direct form (FP32 state) and correction form (FP64 state)
// (args.ctaLo .. args.ctaHi: the CTAs of this launch)
cudaError_t launch_pd_persistent(const PersistPlan& plan, const PersistArgs<float, float>& args, cudaStream_t s);
cudaError_t launch_pd_persistent(const PersistPlan& plan, const PersistArgs<float, double>& args, cudaStream_t s);

}  // namespace pdipc
