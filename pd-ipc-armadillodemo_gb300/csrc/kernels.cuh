// kernels.cuh — device state of one PD-IPC context and the launchers of every
// kernel of the step.  All launches go to the context's stream; nothing here
// synchronises.
#pragma once

#include <cstdint>
#include <mutex>

#include "common.cuh"

namespace pdipc {

// Device buffers of one context.  Vertex arrays use the global numbering
// (cloth vertices first, then static ones).  T is the solver scalar (local
// step, sweeps), TC the scalar of the state (positions, velocities, step
// direction, time of impact) and of CCD/contact: float/float reproduces the
// reference's arithmetic, double/double is the plain FP64 form, float/double
// the mixed form (FP32 arithmetic on FP64 state).
template <typename T, typename TC>
struct Dev {
    int nsim = 0, ntot = 0, nface = 0, nedge = 0, npatch = 0;

    // state
    V4<TC>* P = nullptr;      // positions [ntot]
    V4<TC>* Pold = nullptr;   // positions at the start of the outer iteration [ntot]
    V4<TC>* X0 = nullptr;     // positions at the start of the step [nsim]
    V4<TC>* Vel = nullptr;    // velocities [nsim]
    V4<TC>* Dir = nullptr;    // P - Pold before clamping [ntot]; static part stays 0
    V4<TC>* Xrest = nullptr;  // initial positions [ntot] (reset, pins)
    // correction form only: float-float mirrors (hi, lo) of P and Pold and the
    // rounded step direction, rewritten by every kernel that writes their source
    V4<T>* Ph = nullptr;      // [ntot]
    V4<T>* Pl = nullptr;      // [ntot]
    V4<T>* Poh = nullptr;     // [ntot]
    V4<T>* Pol = nullptr;     // [ntot]
    V4<T>* Dh = nullptr;      // (float) Dir [ntot]

    // solver work
    // Y, B, C: [64 ceil(nsim / 64)]; row order on the per-sweep path, slot
    // order on the persistent one (three planes of floats on its band path)
    V4<T>* Y = nullptr;      // first half of a two-sweep step
    V4<T>* B = nullptr;      // odd Chebyshev iterates
    V4<T>* Aq = nullptr;     // rescaled curvature vector per vertex [nsim]
    V4<T>* Rhs = nullptr;    // right-hand side of the current local-global iteration [nsim]
    V4<TC>* Rhs0 = nullptr;  // inertial right-hand side (m/dt^2) y [nsim]; the predicted y itself in
                             // the correction (mixed) form
    V4<T>* C = nullptr;      // even correction iterates of the correction form
    V4<T>* Grav = nullptr;   // (0, g m, 0) [nsim]
    V4<T>* PinRhs = nullptr; // k_pin * X_rest for pinned vertices, else 0 [nsim]
    T* InvMass = nullptr;    // [nsim]
    int* PinFlag = nullptr;  // -1 free, else pin slot [nsim]
    T* PinK = nullptr;       // stiffness of each pin slot
    T* Dinert = nullptr;     // m/dt^2 (0 for pinned vertices) [nsim]
    T* Delastic = nullptr;   // [nsim]
    T* InvD = nullptr;       // 1 / (elastic + inertial + collision) [nsim]
    T* CollDiag = nullptr;   // [ntot]
    V4<T>* CollRhs = nullptr;// [ntot] sum w*target; in the correction form sum w*(target - x_contact)
    TC* CollMass = nullptr;  // [ntot]

    // local-step stencils (CSR over simulated vertices): [self, neighbours ascending]
    int* lPtr = nullptr;
    int* lNbr = nullptr;
    T* lRest = nullptr;
    T* lLbo = nullptr;
    T* lBend = nullptr;
    T* lBendT = nullptr;
    T* Strain = nullptr;     // per vertex
    T* CurvNorm = nullptr;   // per vertex
    // the same stencils in SELL-32 order for the per-vertex kernels: neighbour
    // k of row i (self excluded, k < lPtr[i+1] - lPtr[i] - 1, ascending as in
    // the CSR) at tOff[i >> 5] + 32 k + (i & 31), so that a warp's k-th loads
    // are one 128-byte line; tBend0 / tLbo0 the self weights per row
    int* tOff = nullptr;
    int* tNbr = nullptr;
    T* tRest = nullptr;
    T* tLbo = nullptr;
    T* tBendT = nullptr;
    T* tBend0 = nullptr;
    T* tLbo0 = nullptr;

    // tetrahedral strain constraints: vertices, row-major Dm^-1 (9 per tet),
    // weights; per-tet projections w R G (4 per tet, vertex-major), gathered
    // per vertex through the incidence list vtIdx = 4 tet + slot (ascending tet)
    int ntet = 0;
    int4* Tets = nullptr;
    T* TetIdm = nullptr;
    T* TetW = nullptr;
    V4<T>* TetOut = nullptr;
    int* vtPtr = nullptr;
    int* vtIdx = nullptr;

    // N = -offdiag(A) in SELL-32: slice s holds rows [32 s, 32 s + 32); entry k
    // of lane r sits at sOff[s] + 32 k + r; sLen[s] entries per row.
    int nslice = 0;
    int* sOff = nullptr;
    int* sLen = nullptr;
    int* sCol = nullptr;
    T* sVal = nullptr;
    // when rows share a few column-offset lists (a structured mesh has a few
    // dozen per cloth): row i's columns are i + patOff[rowPat[i] * patW + k]
    // (int16, padded with 0: the row itself, as sCol's padding), read through
    // L1 instead of streaming sCol; null otherwise
    int* rowPat = nullptr;
    int16_t* patOff = nullptr;
    int patW = 0;

    // collision topology
    int4* Faces = nullptr;   // (v0, v1, v2, -)
    int2* Edges = nullptr;
    int* pfPtr = nullptr;
    int* pfIdx = nullptr;
    int* ppPtr = nullptr;
    int* ppIdx = nullptr;
    int* pePtr = nullptr;
    int* peIdx = nullptr;
    int* pxPtr = nullptr;
    int* pxIdx = nullptr;
    uint8_t* pStatic = nullptr;

    // patch BVH (Karras): internal nodes [0, npatch-1), leaves [npatch-1, 2 npatch-1)
    Box6<T>* PatchBox = nullptr;   // [npatch]
    Box6<T>* NodeBox = nullptr;    // [2 npatch - 1]
    int2* NodeChild = nullptr;     // [npatch - 1]
    int* NodeParent = nullptr;     // [2 npatch - 1]
    int* NodeEscape = nullptr;     // [2 npatch - 1] next node once this subtree is done (-1: end)
    int* LeafPatch = nullptr;      // [npatch] sorted order: leaf k -> patch id
    int* RefitFlag = nullptr;      // [npatch - 1]
    unsigned long long* Morton = nullptr;  // [npatch] codes by patch id

    // candidates of the current step
    int2* Pairs = nullptr;
    int64_t capPairs = 0;
    unsigned long long* PairCount = nullptr;  // pairs found by the last traversal
    int4* PT = nullptr;
    int64_t capPT = 0;
    int4* EE = nullptr;
    int64_t capEE = 0;
    int64_t nPairs = 0, nPT = 0, nEE = 0;

    // scalars
    TC* ToiMin = nullptr;    // running min over candidates (reset to 1 after use)
    TC* Toi = nullptr;       // clamped step fraction of the outer iteration
    double* ResidPart = nullptr;  // per-block partial sums of |dir|^2
    double* Resid = nullptr;      // |dir|^2
    unsigned int* ErrFlags = nullptr;
    unsigned long long* ActiveCount = nullptr;
    // set only while a step runs: the kernels of the outer loop (direction,
    // CCD, clamp, contact, copy into Pold, persistent solve) return at entry
    // once Gate->stop is set; null everywhere else (stage entry points)
    OuterGate* Gate = nullptr;

    // per-instance stopping (pdipc_params.instance_stop; null otherwise): the
    // instance (simulated model) of every vertex (-1: static), the instances'
    // vertex ranges, and per instance its stop flag (cleared outside steps),
    // residual, running time-of-impact minimum, clamp and outer-iteration count
    int ninst = 0;
    int* VInst = nullptr;          // [ntot]
    int* InstBeg = nullptr;        // [ninst + 1]
    unsigned* InstStop = nullptr;  // [ninst]
    double* InstResid = nullptr;   // [ninst]
    TC* InstToiMin = nullptr;      // [ninst]
    TC* InstToi = nullptr;         // [ninst]
    int* InstIters = nullptr;      // [ninst]
};

// Rows the per-row PD kernels skip: those of instances that have stopped
// (pdipc_params.instance_stop); stop is null when nothing is skipped.
struct RowSkip {
    const int* inst;
    const unsigned* stop;
    __device__ __forceinline__ bool operator()(int i) const { return stop && __ldg(stop + __ldg(inst + i)); }
};
template <typename T, typename TC>
inline RowSkip skip_of(const Dev<T, TC>& d) {
    return RowSkip{d.VInst, d.InstStop};
}

// The matrix N as the per-row kernels read it.
template <typename T>
struct Sell {
    const int* off;
    const int* len;
    const int* col;
    const T* val;
    const int* rowPat;      // null: columns from col
    const int16_t* patOff;
    int patW;
};
template <typename T, typename TC>
inline Sell<T> sell_of(const Dev<T, TC>& d) {
    return Sell<T>{d.sOff, d.sLen, d.sCol, d.sVal, d.rowPat, d.patOff, d.patW};
}

// Row i's stencil in the SELL-32 copy: (slot of neighbour 0, neighbour count);
// neighbour k sits at .x + 32 k.
__device__ __forceinline__ int2 stencil_of(int i, const int* __restrict__ lPtr, const int* __restrict__ tOff) {
    return make_int2(__ldg(tOff + (i >> 5)) + (i & 31), __ldg(lPtr + i + 1) - __ldg(lPtr + i) - 1);
}

// A position array and its float-float mirror (null outside the correction form).
template <typename T, typename TC>
struct Pos {
    const V4<TC>* x = nullptr;
    const V4<T>* hi = nullptr;
    const V4<T>* lo = nullptr;
};

struct SolverConsts {
    double dt, gravity, dhat, kappa, infl, relax, rho, toi_scale, ccd_slack, ccd_eta, static_mass;
    int lg, cheby, ccd_max_iter;
    // launch shapes the autotuner may change: blocks of the grid-stride
    // candidate kernels (time of impact, contact), threads per block of the
    // broad phase's traversal and expansion
    int cand_grid = 152 * 16;
    int trav_block = 128;
    int expand_block = 256;
    // 1: after the additive CCD, the FP64 coplanarity-cubic pass (pdipc_params.ccd_mode)
    int ccd_mode = 0;
};

// ---------------- PD kernels (pd_kernels.cu) ----------------
template <typename T, typename TC>
void launch_predict(const Dev<T, TC>& d, TC dt, cudaStream_t s);
template <typename T, typename TC>
void launch_diag(const Dev<T, TC>& d, cudaStream_t s);
// tet strain projections of the current positions into TetOut (no-op without tets)
template <typename T, typename TC>
void launch_tet_project(const Dev<T, TC>& d, cudaStream_t s);
template <typename T, typename TC>
void launch_local_aq(const Dev<T, TC>& d, cudaStream_t s);
// local step right-hand side fused with the first J sweep (Y = S(P))
template <typename T, typename TC>
void launch_local_rhs_sweep(const Dev<T, TC>& d, T relax, cudaStream_t s);
// out = S(src) or, with prev, out = omega (S(src) - prev) + prev (T == TC only)
template <typename T, typename TC>
void launch_sweep(const Dev<T, TC>& d, const V4<T>* src, const V4<T>* prev, V4<T>* out, T relax, T omega,
                  cudaStream_t s);
// Correction (mixed-precision) form of one local-global iteration's pieces:
// residual r0 = b - A x from relative coordinates (compensated FP32 sums) into Rhs
// and the first sweep from delta = 0 into Y.
template <typename T, typename TC>
void launch_local_residual(const Dev<T, TC>& d, T relax, cudaStream_t s);
// sweep on the correction: mode bits 1 Chebyshev, 2 the previous iterate is
// zero, 4 the result is added to the positions P instead of written to out.
template <typename T, typename TC>
void launch_sweep_delta(const Dev<T, TC>& d, int mode, const V4<T>* src, const V4<T>* prev, V4<T>* out, T relax,
                        T omega, cudaStream_t s);
template <typename T, typename TC>
void launch_direction(const Dev<T, TC>& d, cudaStream_t s);
template <typename T, typename TC>
void launch_clamp(const Dev<T, TC>& d, cudaStream_t s);
template <typename T, typename TC>
void launch_velocity(const Dev<T, TC>& d, TC invt, cudaStream_t s);
template <typename T, typename TC>
void launch_copy_old(const Dev<T, TC>& d, cudaStream_t s);
// the outer loop's stopping test on the device (d.Gate must be set, zeroed at
// the step's start): after outer iteration k = Gate->iters, stop when
// test && k > 0 && Resid < tol (the iteration index comes from the device, so
// the launch is the same in every iteration and can sit in a CUDA graph)
template <typename T, typename TC>
void launch_outer_gate(const Dev<T, TC>& d, double tol, bool test, cudaStream_t s);
// per-instance stopping: |dir|^2 of every instance into InstResid; after the
// contact pass, each running instance's test (its iteration count, then
// stop when test && outer > 0 && InstResid < tol), and the step's record in
// d.Gate (stop once every instance has stopped; resid the sum)
template <typename T, typename TC>
void launch_inst_resid(const Dev<T, TC>& d, cudaStream_t s);
template <typename T, typename TC>
void launch_inst_gate(const Dev<T, TC>& d, double tol, bool test, cudaStream_t s);
// correction form: write the float-float mirror (hi, lo; lo may be null) of n
// positions X, after a host write of X
template <typename T, typename TC>
void launch_split(const Dev<T, TC>& d, const V4<TC>* X, V4<T>* hi, V4<T>* lo, int n, cudaStream_t s);
int direction_blocks(int nsim);

// ---------------- collision kernels (collision_kernels.cu) ----------------
// swept (D != null) or static patch boxes, inflated; Xh, Dh: T-rounded copies
// of X and D when the state is wider than T (correction form), else null
template <typename T, typename TC>
void launch_patch_boxes(const Dev<T, TC>& d, const V4<TC>* X, const V4<TC>* D, const V4<T>* Xh, const V4<T>* Dh,
                        T infl, cudaStream_t s);
// init-time boxes over every vertex of the patch (AipcBvhs input, cpp:1279-1292)
template <typename T, typename TC>
void launch_patch_init_boxes(const Dev<T, TC>& d, T infl, cudaStream_t s);
// Morton codes of the patch box centres; ctr_scale[0..3] = centre xyz, scale
template <typename T, typename TC>
void launch_morton(const Dev<T, TC>& d, T* ctr_scale_dev, unsigned long long* keys, int* vals, cudaStream_t s);
template <typename T, typename TC>
void launch_karras(const Dev<T, TC>& d, const unsigned long long* sorted_codes, cudaStream_t s);
template <typename T, typename TC>
void launch_refit(const Dev<T, TC>& d, cudaStream_t s);
// overlapping patch pairs into d.Pairs[0, cap) with their point-triangle and
// edge-edge record counts; *count (zeroed by the caller) gets the full number
template <typename T, typename TC>
void launch_traverse(const Dev<T, TC>& d, int64_t* cnt_pt, int64_t* cnt_ee, int64_t cap, unsigned long long* count,
                     const SolverConsts& c, cudaStream_t s);
template <typename T, typename TC>
void launch_expand(const Dev<T, TC>& d, const int64_t* off_pt, const int64_t* off_ee, const SolverConsts& c,
                   cudaStream_t s);
template <typename T, typename TC>
void launch_toi(const Dev<T, TC>& d, Pos<T, TC> X0, Pos<T, TC> X1, const SolverConsts& c, TC* per_pt,
                TC* per_ee, cudaStream_t s);
template <typename T, typename TC>
void launch_toi_finalize(const Dev<T, TC>& d, const SolverConsts& c, cudaStream_t s);
// per-instance stopping: the per-candidate times of impact (per_pt, per_ee of
// launch_toi) reduced into every instance a candidate's vertices belong to,
// then each instance's clamp InstToi (scaled when below 1; minima reset)
template <typename T, typename TC>
void launch_inst_toi(const Dev<T, TC>& d, const TC* per_pt, const TC* per_ee, const SolverConsts& c, cudaStream_t s);
template <typename T, typename TC>
void launch_contact(const Dev<T, TC>& d, Pos<T, TC> X, const SolverConsts& c, cudaStream_t s);

// ---------------- penalty / discrete-collision stages (penalty_kernels.cu) ----------------
template <typename T, typename TC>
void launch_pen_predict(const Dev<T, TC>& d, const V4<TC>* X, V4<TC>* V, TC dt, V4<TC>* Sn, cudaStream_t s);
// over the candidate lists of the last broad phase
template <typename T, typename TC>
void launch_pen_ccd(const Dev<T, TC>& d, const V4<TC>* X0, const V4<TC>* D, TC k, TC eta, int max_iter,
                    V4<TC>* F, int* times, cudaStream_t s);
template <typename T, typename TC>
void launch_pen_floor(const Dev<T, TC>& d, const V4<TC>* X, TC k, V4<TC>* F, int* times, cudaStream_t s);
template <typename T, typename TC>
void launch_pen_dcd(const Dev<T, TC>& d, const int2* pairs, int64_t n, const int* model, const V4<TC>* X, TC k,
                    TC kself, V4<TC>* F, int* times, cudaStream_t s);
template <typename T, typename TC>
void launch_pen_uniform(const Dev<T, TC>& d, V4<TC>* F, const int* times, TC damping, V4<TC>* V, cudaStream_t s);

// ---------------- discrete adjoint of the contact-free step (adjoint_kernels.cu, FP64 only) ----------------
// transposed LBO weights per stencil slot [lPtr[nsim]] and transposed matrix
// values in the SELL layout of sVal
template <typename T, typename TC>
void launch_adj_tables(const Dev<T, TC>& d, T* lLboT, T* NTval, cudaStream_t s);
// one sweep's adjoint at input z with output adjoint scale * in:
// out (= or +=) J^T u, rho += u, kbar += dS/dk . u, other += (1 - scale) in
template <typename T, typename TC>
void launch_adj_sweep(const Dev<T, TC>& d, const T* NTval, T relax, T scale, const V4<T>* in, V4<T>* other,
                      const V4<T>* z, V4<T>* out, bool accumulate, V4<T>* rho, T* kbar, cudaStream_t s);
// the local step's adjoint at x from rho (sum of the sweeps' output adjoints):
// rb, qb scratch; r0b += w D^-1 rho; xb += d(rhs)/dx^T rb; kbar += d(rhs)/dk . rb;
// with strain-limit elements (tets, cloth triangles) their SVD-derivative
// adjoint through eb (4 per element, scratch)
template <typename T, typename TC>
void launch_adj_local(const Dev<T, TC>& d, const T* lLboT, T relax, const V4<T>* x, const V4<T>* rho, V4<T>* rb,
                      V4<T>* qb, V4<T>* r0b, V4<T>* xb, T* kbar, V4<T>* eb, cudaStream_t s);
// step output adjoints -> adjoint of the solved positions (pb) and of X0 (vb); r0b = 0
template <typename T, typename TC>
void launch_adj_step_begin(const Dev<T, TC>& d, T invt, V4<T>* pb, V4<T>* vb, V4<T>* r0b, cudaStream_t s);
// through the prediction: pb, vb := adjoints of the step's input positions and velocities
template <typename T, typename TC>
void launch_adj_step_end(const Dev<T, TC>& d, T dt, V4<T>* pb, V4<T>* vb, const V4<T>* r0b, cudaStream_t s);

// Scratch of the no-allocation per-candidate toi pass: a file-scope device array
// of kToiScratchEntries doubles (8 MiB), its address looked up once per device on
// first use.  One array per device is shared by every context of the process:
// callers hold *lock from launch until their results are back on the host.
constexpr int64_t kToiScratchEntries = int64_t(1) << 20;
struct ToiScratch {
    double* ptr = nullptr;
    int64_t entries = 0;
    std::mutex* lock = nullptr;
};
cudaError_t toi_scratch(ToiScratch* out);

// ---------------- primitives (primitives.cu) ----------------
// Exclusive scan of n int64 values (in may equal out); *total receives the sum.
// tmp must hold scan_tmp_bytes(n) bytes.
size_t scan_tmp_bytes(int64_t n);
void scan_exclusive_i64(const int64_t* in, int64_t* out, int64_t n, int64_t* total, void* tmp, cudaStream_t s);
void scan_exclusive_i32(const int* in, int* out, int n, int* total, void* tmp, cudaStream_t s);
// Stable LSD radix sort of 64-bit keys with int values (keys use the low 63 bits).
size_t sort_tmp_bytes(int n);
// stable onesweep sort by key; a timed-out look-back wait sets kErrSort in *err
void radix_sort_u64(unsigned long long* keys, int* vals, int n, void* tmp, unsigned* err, cudaStream_t s);
void launch_reduce_sum_f64(const double* part, int n, double* out, cudaStream_t s);

}  // namespace pdipc
