// pd_kernels.cu — projective-dynamics kernels of the PD-IPC cloth step.
//
// Reference kernels replaced (Simulator/PD-IPC/PdIpcGpuFunc.cu):
//   predictiveKernel :88-147                         -> k_predict
//   solveClothPointsStrainAndBendingConstraintKernel
//     :627-728 + solvePointsConstraintKernel :764-790 -> k_local_aq + k_local_rhs_sweep
//   updateR1/R2/R2Row OperatorsKernel :899-974,
//   superJacobiR2FirstTermKernel :1041-1074,
//   superJacobiR2IterationKernel :1076-1129,
//   chebyshevJacobiR2IterationKernel :1185-1242     -> k_sweep (R2 applied as two J sweeps)
//   computeDirectionKernel :185, clampDirectionKernel :222,
//   updateVelocityKernel :262, cublasSdot (cpp:1774) -> k_direction, k_clamp, k_velocity
//
// Layout: one vertex per aligned 4-vector; the local step is a gather (no
// atomics) and the system matrix is streamed from SELL-32 slices so a warp's
// column/value loads are contiguous 128-byte lines.
#include <algorithm>
#include <type_traits>

#include "kernels.cuh"
#include "svd3.cuh"

namespace pdipc {

namespace {

constexpr int kBlock = 256;

inline int blocks_for(int n, int b = kBlock) { return (n + b - 1) / b; }

// FP64 positions with FP32 arithmetic: the correction form keeps a float-float
// mirror (Ph, Pl) of P.
template <typename T, typename S>
constexpr bool kMirror = std::is_same<T, float>::value && std::is_same<S, double>::value;

__device__ __forceinline__ void store_split(V4<float>* Ph, V4<float>* Pl, int i, double x, double y, double z) {
    float h0, l0, h1, l1, h2, l2;
    split_ff(x, h0, l0);
    split_ff(y, h1, l1);
    split_ff(z, h2, l2);
    Ph[i] = V4<float>{h0, h1, h2, 0.f};
    Pl[i] = V4<float>{l0, l1, l2, 0.f};
}

// S is the state scalar (== T except in the correction form, where the
// prediction is formed in FP64 from the FP32 mass and gravity terms).
template <typename T, typename S, bool kDelta>
__global__ void k_predict(int nsim, int ntot, S dt, V4<S>* __restrict__ P, V4<S>* __restrict__ Pold,
                          V4<S>* __restrict__ X0, V4<S>* __restrict__ Vel, V4<S>* __restrict__ Rhs0,
                          T* __restrict__ Dinert, const V4<T>* __restrict__ Grav, const T* __restrict__ InvMass,
                          const int* __restrict__ PinFlag, T* __restrict__ CollDiag, V4<T>* __restrict__ CollRhs,
                          V4<T>* __restrict__ Ph, V4<T>* __restrict__ Pl, V4<T>* __restrict__ Poh,
                          V4<T>* __restrict__ Pol) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ntot) return;
    CollDiag[i] = T(0);
    CollRhs[i] = V4<T>{T(0), T(0), T(0), T(0)};
    if (i >= nsim) return;
    const V4<S> x = P[i];
    X0[i] = x;
    Pold[i] = x;
    if constexpr (kMirror<T, S>) {
        Poh[i] = Ph[i];
        Pol[i] = Pl[i];
    }
    if (PinFlag[i] != -1) {  // pinned: velocity zeroed, nothing else written
        Vel[i] = V4<S>{S(0), S(0), S(0), S(0)};
        return;
    }
    const T im = InvMass[i];
    const S m = (S)im * dt;
    const V4<S> v = Vel[i];
    const V4<T> g = Grav[i];
    S y0 = (v.x + m * (S)g.x) * dt + x.x;
    S y1 = (v.y + m * (S)g.y) * dt + x.y;
    S y2 = (v.z + m * (S)g.z) * dt + x.z;
    const S mm = S(1) / (dt * m);
    Dinert[i] = (T)(S(1) / ((S)im * dt * dt));
    if (kDelta) Rhs0[i] = V4<S>{y0, y1, y2, S(0)};
    else Rhs0[i] = V4<S>{mm * y0, mm * y1, mm * y2, S(0)};
    P[i] = V4<S>{y0, y1, y2, S(0)};
    if constexpr (kMirror<T, S>) store_split(Ph, Pl, i, y0, y1, y2);
}

template <typename T>
__global__ void k_diag(int nsim, const T* __restrict__ De, const T* __restrict__ Di, const T* __restrict__ Dc,
                       T* __restrict__ InvD) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nsim) return;
    const T d = (De[i] + Di[i]) + Dc[i];  // sysDiag = elastic + inertial (+ collision), cpp:1556-1560
    InvD[i] = T(1) / d;
}

// Tet strain projection (solveVolumetricStrainConstraintKernel,
// PdIpcGpuFunc.cu:439-599), one thread per tet; the four vertex contributions
// w R G go to TetOut and are gathered per vertex by the local-step kernels
// (the reference scatters them with atomics).  Edge vectors come from the
// float-float mirror in the correction form.
template <typename T, typename S>
__global__ void k_tet_project(int ntet, const int4* __restrict__ Tets, const T* __restrict__ Idm,
                              const T* __restrict__ W, const V4<S>* __restrict__ P, const V4<T>* __restrict__ Ph,
                              const V4<T>* __restrict__ Pl, V4<T>* __restrict__ Out, const RowSkip skip) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ntet) return;
    const int4 q = Tets[e];
    if (skip(q.x)) return;  // an element's vertices belong to one model
    // a cloth triangle's strain element has no fourth vertex (-1): its first
    // vertex stands in, so the third edge is zero and unused
    const bool tri = q.w < 0;
    const int id[4] = {q.x, q.y, q.z, tri ? q.x : q.w};
    T Ds[3][3];
    if constexpr (kMirror<T, S>) {
        const V4<T> h0 = ld4(Ph, id[0]), l0 = ld4(Pl, id[0]);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const V4<T> h = ld4(Ph, id[c + 1]), l = ld4(Pl, id[c + 1]);
            Ds[0][c] = diff_ff(h.x, l.x, h0.x, l0.x);
            Ds[1][c] = diff_ff(h.y, l.y, h0.y, l0.y);
            Ds[2][c] = diff_ff(h.z, l.z, h0.z, l0.z);
        }
    } else {
        const V4<S> x0 = ld4(P, id[0]);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const V4<S> x = ld4(P, id[c + 1]);
            Ds[0][c] = x.x - x0.x;
            Ds[1][c] = x.y - x0.y;
            Ds[2][c] = x.z - x0.z;
        }
    }
    T idm[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) idm[k] = __ldg(Idm + 9 * (size_t)e + k);
    T out[4][3];
    if (tri) {
        const T D2[3][2] = {{Ds[0][0], Ds[0][1]}, {Ds[1][0], Ds[1][1]}, {Ds[2][0], Ds[2][1]}};
        T o3[3][3];
        svd::tri_project<T>(D2, idm, __ldg(W + e), o3);
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
            for (int r = 0; r < 3; ++r) out[c][r] = o3[c][r];
        out[3][0] = out[3][1] = out[3][2] = T(0);
    } else {
        svd::tet_project<T>(Ds, idm, __ldg(W + e), out);
    }
#pragma unroll
    for (int c = 0; c < 4; ++c) Out[4 * (size_t)e + c] = V4<T>{out[c][0], out[c][1], out[c][2], T(0)};
}

// Curvature vector aq_i = sum_k lbo_ik x_k, rescaled to the rest norm
// (PdIpcGpuFunc.cu:664-699).
template <typename T>
__global__ void k_local_aq(int nsim, const V4<T>* __restrict__ P, const int* __restrict__ lPtr,
                           const int* __restrict__ tOff, const int* __restrict__ tNbr, const T* __restrict__ tLbo,
                           const T* __restrict__ tLbo0, const T* __restrict__ CurvNorm,
                           V4<T>* __restrict__ Aq, const RowSkip skip) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nsim || skip(i)) return;
    const int2 st = stencil_of(i, lPtr, tOff);
    const V4<T> x = ld4(P, i);
    const T l0 = __ldg(tLbo0 + i);
    T a0 = x.x * l0, a1 = x.y * l0, a2 = x.z * l0;
    for (int k = 0; k < st.y; ++k) {
        const int s = st.x + kSlice * k;
        const V4<T> xj = ld4(P, __ldg(tNbr + s));
        const T l = __ldg(tLbo + s);
        a0 += xj.x * l;
        a1 += xj.y * l;
        a2 += xj.z * l;
    }
    const T nrm = dsqrt(a0 * a0 + a1 * a1 + a2 * a2);
    if (nrm >= T(1e-10)) {
        const T c = __ldg(CurvNorm + i) / nrm;
        a0 *= c;
        a1 *= c;
        a2 *= c;
    }
    Aq[i] = V4<T>{a0, a1, a2, T(0)};
}

template <typename T>
__device__ __forceinline__ void sell_row(int i, const Sell<T> M, const V4<T>* __restrict__ X, T& s0, T& s1, T& s2) {
    const int sl = i >> 5, lane = i & 31;
    const int base = __ldg(M.off + sl) + lane;
    const int len = __ldg(M.len + sl);
    const int16_t* po = M.rowPat ? M.patOff + (size_t)__ldg(M.rowPat + i) * M.patW : nullptr;
    s0 = T(0);
    s1 = T(0);
    s2 = T(0);
#pragma unroll 4
    for (int k = 0; k < len; ++k) {
        const int j = po ? i + (int)__ldg(po + k) : __ldg(M.col + base + 32 * k);
        const T v = __ldg(M.val + base + 32 * k);
        const V4<T> xj = ld4(X, j);
        s0 += v * xj.x;
        s1 += v * xj.y;
        s2 += v * xj.z;
    }
}

// rhs_i = ((rhs0_i + spring_i + bend_ii aq_i + sum_k bend_ki aq_k) + contact_i) + pin_i,
// then the first weighted-Jacobi sweep Y = (1-w) x + w D^-1 (N x + rhs).
template <typename T>
__global__ void __launch_bounds__(kBlock) k_local_rhs_sweep(
    int nsim, T relax, const V4<T>* __restrict__ P, const int* __restrict__ lPtr, const int* __restrict__ tOff,
    const int* __restrict__ tNbr, const T* __restrict__ tRest, const T* __restrict__ tBend0,
    const T* __restrict__ tBendT,
    const T* __restrict__ Strain, const V4<T>* __restrict__ Aq, const V4<T>* __restrict__ Rhs0,
    const V4<T>* __restrict__ CollRhs, const V4<T>* __restrict__ PinRhs, const T* __restrict__ InvD,
    const Sell<T> M, const int* __restrict__ vtPtr, const int* __restrict__ vtIdx,
    const V4<T>* __restrict__ TetOut, V4<T>* __restrict__ Rhs, V4<T>* __restrict__ Y, const RowSkip skip) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nsim || skip(i)) return;
    const int2 st = stencil_of(i, lPtr, tOff);
    const V4<T> x = ld4(P, i);
    const T strain = __ldg(Strain + i);
    T t0 = T(0), t1 = T(0), t2 = T(0);
    for (int k = 0; k < st.y; ++k) {  // mass-spring projections (cu:670-690)
        const int s = st.x + kSlice * k;
        const V4<T> xj = ld4(P, __ldg(tNbr + s));
        const T d0 = x.x - xj.x, d1 = x.y - xj.y, d2 = x.z - xj.z;
        const T cl = dsqrt(d0 * d0 + d1 * d1 + d2 * d2);
        const T rc = strain * (__ldg(tRest + s) / cl);
        t0 += rc * d0;
        t1 += rc * d1;
        t2 += rc * d2;
    }
    const V4<T> ai = ld4(Aq, i);
    const T b0 = __ldg(tBend0 + i);
    t0 += b0 * ai.x;
    t1 += b0 * ai.y;
    t2 += b0 * ai.z;
    const V4<T> r0 = ld4(Rhs0, i);
    T r_0 = r0.x + t0, r_1 = r0.y + t1, r_2 = r0.z + t2;
    for (int k = 0; k < st.y; ++k) {  // bending terms the neighbours' stencils put on i
        const int s = st.x + kSlice * k;
        const V4<T> ak = ld4(Aq, __ldg(tNbr + s));
        const T bt = __ldg(tBendT + s);
        r_0 += bt * ak.x;
        r_1 += bt * ak.y;
        r_2 += bt * ak.z;
    }
    if (vtPtr)
        for (int q = __ldg(vtPtr + i); q < __ldg(vtPtr + i + 1); ++q) {  // tet projections, ascending tet
            const V4<T> t = ld4(TetOut, __ldg(vtIdx + q));
            r_0 += t.x;
            r_1 += t.y;
            r_2 += t.z;
        }
    const V4<T> c = ld4(CollRhs, i);
    r_0 += c.x;
    r_1 += c.y;
    r_2 += c.z;
    const V4<T> pn = ld4(PinRhs, i);
    r_0 += pn.x;
    r_1 += pn.y;
    r_2 += pn.z;
    Rhs[i] = V4<T>{r_0, r_1, r_2, T(0)};
    T s0, s1, s2;
    sell_row(i, M, P, s0, s1, s2);
    const T id = __ldg(InvD + i);
    const T om = T(1) - relax;
    Y[i] = V4<T>{om * x.x + relax * ((s0 + r_0) * id), om * x.y + relax * ((s1 + r_1) * id),
                 om * x.z + relax * ((s2 + r_2) * id), T(0)};
}

// One weighted-Jacobi sweep S(x) = (1-w) x + w D^-1 (N x + rhs); with prev it
// is the second half of a Chebyshev step: out = omega (S(src) - prev) + prev.
template <typename T, bool kCheby>
__global__ void __launch_bounds__(kBlock) k_sweep(int nsim, T relax, T omega, const V4<T>* __restrict__ src,
                                                  const V4<T>* __restrict__ prev, V4<T>* __restrict__ out,
                                                  const V4<T>* __restrict__ Rhs, const T* __restrict__ InvD,
                                                  const Sell<T> M, const RowSkip skip) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nsim || skip(i)) return;
    T s0, s1, s2;
    sell_row(i, M, src, s0, s1, s2);
    const V4<T> x = ld4(src, i);
    const V4<T> r = ld4(Rhs, i);
    const T id = __ldg(InvD + i);
    const T om = T(1) - relax;
    T y0 = om * x.x + relax * ((s0 + r.x) * id);
    T y1 = om * x.y + relax * ((s1 + r.y) * id);
    T y2 = om * x.z + relax * ((s2 + r.z) * id);
    if (kCheby) {
        const V4<T> p = ld4(prev, i);
        y0 = omega * (y0 - p.x) + p.x;
        y1 = omega * (y1 - p.y) + p.y;
        y2 = omega * (y2 - p.z) + p.z;
    }
    out[i] = V4<T>{y0, y1, y2, T(0)};
}

// Correction form, one vertex per thread.  With x the current positions,
//   r0 = b - A x
//      = Dinert (y - x) + k_pin (X_rest - x) + sum_c w_c (target_c - x_c) + Dcoll (x_c - x)
//        + springs + bending + sum_j N_ij (x_j - x)
// where x_c are the positions the contact projections were taken at (Pold).
// The elastic rows of A sum to zero (springs and the LBO stencils are
// translation invariant), which is used exactly: the rounded FP32 entries would
// otherwise add a spurious pull toward the origin.  Every large term is formed
// from a difference of nearby positions, so FP32 inputs lose nothing to
// cancellation; the sum is accumulated with compensated (TwoSum) FP32 sums.  Then the first sweep from
// delta = 0: Y = w r0 / D.  Positions are FP64 (S): the vertex's own terms
// subtract in FP64 once, the neighbour differences come from the float-float
// mirror (Ph, Pl) in FP32; each enters the FP32 arithmetic as about one rounding.
template <typename T, typename S>
__global__ void __launch_bounds__(kBlock) k_local_residual(
    int nsim, T relax, const V4<S>* __restrict__ P, const V4<T>* __restrict__ Ph, const V4<T>* __restrict__ Pl,
    const V4<S>* __restrict__ Pold, const V4<S>* __restrict__ Xrest,
    const V4<S>* __restrict__ Ypred, const T* __restrict__ Dinert, const T* __restrict__ CollDiag,
    const V4<T>* __restrict__ CollRes, const int* __restrict__ PinFlag, const T* __restrict__ PinK,
    const int* __restrict__ lPtr, const int* __restrict__ tOff, const int* __restrict__ tNbr,
    const T* __restrict__ tRest, const T* __restrict__ tBend0, const T* __restrict__ tBendT,
    const T* __restrict__ Strain,
    const V4<T>* __restrict__ Aq, const T* __restrict__ InvD,
    const Sell<T> M, const int* __restrict__ vtPtr, const int* __restrict__ vtIdx,
    const V4<T>* __restrict__ TetOut, V4<T>* __restrict__ Rhs, V4<T>* __restrict__ Y, const RowSkip skip) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nsim || skip(i)) return;
    const V4<S> x = ld4(P, i);
    Sum2 r0, r1, r2;
    {   // inertia
        const V4<S> y = ld4(Ypred, i);
        const T di = __ldg(Dinert + i);
        r0.add(di * (T)(y.x - x.x));
        r1.add(di * (T)(y.y - x.y));
        r2.add(di * (T)(y.z - x.z));
    }
    const int pf = __ldg(PinFlag + i);
    if (pf >= 0) {
        const V4<S> xr = ld4(Xrest, i);
        const T k = __ldg(PinK + pf);
        r0.add(k * (T)(xr.x - x.x));
        r1.add(k * (T)(xr.y - x.y));
        r2.add(k * (T)(xr.z - x.z));
    }
    {   // contact projections taken at Pold
        const V4<T> c = ld4(CollRes, i);
        const V4<S> xo = ld4(Pold, i);
        const T dc = __ldg(CollDiag + i);
        r0.add(c.x);
        r0.add(dc * (T)(xo.x - x.x));
        r1.add(c.y);
        r1.add(dc * (T)(xo.y - x.y));
        r2.add(c.z);
        r2.add(dc * (T)(xo.z - x.z));
    }
    const int2 st = stencil_of(i, lPtr, tOff);
    const T strain = __ldg(Strain + i);
    const V4<T> h = ld4(Ph, i), l = ld4(Pl, i);
    for (int k = 0; k < st.y; ++k) {  // mass-spring projections
        const int s = st.x + kSlice * k;
        const int j = __ldg(tNbr + s);
        const V4<T> hj = ld4(Ph, j), lj = ld4(Pl, j);
        const T d0 = diff_ff(h.x, l.x, hj.x, lj.x), d1 = diff_ff(h.y, l.y, hj.y, lj.y),
                d2 = diff_ff(h.z, l.z, hj.z, lj.z);
        const T cl = dsqrt(d0 * d0 + d1 * d1 + d2 * d2);
        const T rc = strain * (__ldg(tRest + s) / cl);
        r0.add(rc * d0);
        r1.add(rc * d1);
        r2.add(rc * d2);
    }
    {   // bending: own stencil and the neighbours' stencils
        const V4<T> ai = ld4(Aq, i);
        const T b0 = __ldg(tBend0 + i);
        r0.add(b0 * ai.x);
        r1.add(b0 * ai.y);
        r2.add(b0 * ai.z);
        for (int k = 0; k < st.y; ++k) {
            const int s = st.x + kSlice * k;
            const V4<T> ak = ld4(Aq, __ldg(tNbr + s));
            const T bt = __ldg(tBendT + s);
            r0.add(bt * ak.x);
            r1.add(bt * ak.y);
            r2.add(bt * ak.z);
        }
    }
    if (vtPtr)
        for (int q = __ldg(vtPtr + i); q < __ldg(vtPtr + i + 1); ++q) {  // tet projections w R G
            const V4<T> t = ld4(TetOut, __ldg(vtIdx + q));
            r0.add(t.x);
            r1.add(t.y);
            r2.add(t.z);
        }
    {   // sum_j N_ij (x_j - x_i)
        const int sl = i >> 5, lane = i & 31;
        const int base = __ldg(M.off + sl) + lane;
        const int len = __ldg(M.len + sl);
        const int16_t* po = M.rowPat ? M.patOff + (size_t)__ldg(M.rowPat + i) * M.patW : nullptr;
#pragma unroll 4
        for (int k = 0; k < len; ++k) {
            const int j = po ? i + (int)__ldg(po + k) : __ldg(M.col + base + 32 * k);
            const T v = __ldg(M.val + base + 32 * k);
            const V4<T> hj = ld4(Ph, j), lj = ld4(Pl, j);
            r0.add(v * diff_ff(hj.x, lj.x, h.x, l.x));
            r1.add(v * diff_ff(hj.y, lj.y, h.y, l.y));
            r2.add(v * diff_ff(hj.z, lj.z, h.z, l.z));
        }
    }
    const T f0 = r0.value(), f1 = r1.value(), f2 = r2.value();
    Rhs[i] = V4<T>{f0, f1, f2, T(0)};
    const T wid = relax * __ldg(InvD + i);
    Y[i] = V4<T>{wid * f0, wid * f1, wid * f2, T(0)};
}

// Sweep on the correction delta (rhs = residual r0).  kMode bits: 1 Chebyshev
// step omega (S(src) - prev) + prev; 2 the previous iterate is zero (so the
// step is omega S(src)); 4 the result is added to the FP64 positions P
// instead of written to out.
template <typename T, typename S, int kMode>
__global__ void __launch_bounds__(kBlock) k_sweep_delta(int nsim, T relax, T omega, const V4<T>* __restrict__ src,
                                                        const V4<T>* __restrict__ prev, V4<T>* __restrict__ out,
                                                        V4<S>* __restrict__ P, V4<T>* __restrict__ Ph,
                                                        V4<T>* __restrict__ Pl,
                                                        const V4<T>* __restrict__ Rhs, const T* __restrict__ InvD,
                                                        const Sell<T> M, const RowSkip skip) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nsim || skip(i)) return;
    T s0, s1, s2;
    sell_row(i, M, src, s0, s1, s2);
    const V4<T> x = ld4(src, i);
    const V4<T> r = ld4(Rhs, i);
    const T id = __ldg(InvD + i);
    const T om = T(1) - relax;
    T y0 = om * x.x + relax * ((s0 + r.x) * id);
    T y1 = om * x.y + relax * ((s1 + r.y) * id);
    T y2 = om * x.z + relax * ((s2 + r.z) * id);
    if (kMode & 1) {
        if (kMode & 2) {
            y0 *= omega;
            y1 *= omega;
            y2 *= omega;
        } else {
            const V4<T> p = ld4(prev, i);
            y0 = omega * (y0 - p.x) + p.x;
            y1 = omega * (y1 - p.y) + p.y;
            y2 = omega * (y2 - p.z) + p.z;
        }
    }
    if (kMode & 4) {
        const V4<S> q = P[i];
        const S n0 = q.x + (S)y0, n1 = q.y + (S)y1, n2 = q.z + (S)y2;
        P[i] = V4<S>{n0, n1, n2, S(0)};
        if constexpr (kMirror<T, S>) store_split(Ph, Pl, i, n0, n1, n2);
    } else {
        out[i] = V4<T>{y0, y1, y2, T(0)};
    }
}

// Relative form of the curvature vector for the correction form:
// aq = sum_{k>0} lbo_k (x_k - x_i), using that the LBO weights of a stencil sum
// to zero.
__global__ void k_local_aq_rel(int nsim, const V4<float>* __restrict__ Ph, const V4<float>* __restrict__ Pl,
                               const int* __restrict__ lPtr, const int* __restrict__ tOff,
                               const int* __restrict__ tNbr, const float* __restrict__ tLbo,
                               const float* __restrict__ CurvNorm,
                               V4<float>* __restrict__ Aq, const RowSkip skip) {
    using T = float;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nsim || skip(i)) return;
    const int2 st = stencil_of(i, lPtr, tOff);
    const V4<T> h = ld4(Ph, i), l = ld4(Pl, i);
    T a0 = T(0), a1 = T(0), a2 = T(0);
    for (int k = 0; k < st.y; ++k) {
        const int s = st.x + kSlice * k;
        const int j = __ldg(tNbr + s);
        const V4<T> hj = ld4(Ph, j), lj = ld4(Pl, j);
        const T w = __ldg(tLbo + s);
        a0 += w * diff_ff(hj.x, lj.x, h.x, l.x);
        a1 += w * diff_ff(hj.y, lj.y, h.y, l.y);
        a2 += w * diff_ff(hj.z, lj.z, h.z, l.z);
    }
    const T nrm = dsqrt(a0 * a0 + a1 * a1 + a2 * a2);
    if (nrm >= T(1e-10)) {
        const T c = __ldg(CurvNorm + i) / nrm;
        a0 *= c;
        a1 *= c;
        a2 *= c;
    }
    Aq[i] = V4<T>{a0, a1, a2, T(0)};
}

template <typename T, typename S>  // S: the state scalar
__global__ void k_direction(int nsim, const V4<S>* __restrict__ P, const V4<S>* __restrict__ Pold,
                            V4<S>* __restrict__ Dir, V4<T>* __restrict__ Dh, double* __restrict__ part,
                            const OuterGate* __restrict__ gate) {
    __shared__ double red[kBlock / 32];
    if (outer_stopped(gate)) return;
    double acc = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nsim; i += gridDim.x * blockDim.x) {
        const V4<S> a = P[i], b = Pold[i];
        const S d0 = a.x - b.x, d1 = a.y - b.y, d2 = a.z - b.z;
        Dir[i] = V4<S>{d0, d1, d2, S(0)};
        if constexpr (kMirror<T, S>) Dh[i] = V4<T>{(T)d0, (T)d1, (T)d2, T(0)};
        acc += (double)d0 * (double)d0 + (double)d1 * (double)d1 + (double)d2 * (double)d2;
    }
    acc = warp_sum(acc);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = threadIdx.x < kBlock / 32 ? red[threadIdx.x] : 0.0;
        v = warp_sum(v);
        if (threadIdx.x == 0) part[blockIdx.x] = v;
    }
}

template <typename T, typename S>  // S: the state scalar
__global__ void k_clamp(int nsim, const V4<S>* __restrict__ Pold, const V4<S>* __restrict__ Dir,
                        const S* __restrict__ Toi, V4<S>* __restrict__ P, V4<T>* __restrict__ Ph,
                        V4<T>* __restrict__ Pl, const OuterGate* __restrict__ gate, const int* __restrict__ VInst,
                        const S* __restrict__ InstToi) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nsim || outer_stopped(gate)) return;
    const S t = InstToi ? InstToi[VInst[i]] : *Toi;  // per-instance stopping: the instance's own clamp
    const V4<S> a = Pold[i], d = Dir[i];
    const S x = a.x + t * d.x, y = a.y + t * d.y, z = a.z + t * d.z;
    P[i] = V4<S>{x, y, z, S(0)};
    if constexpr (kMirror<T, S>) store_split(Ph, Pl, i, x, y, z);
}

// hi = rn(x); lo = rn(x - hi) unless lo is null
__global__ void k_split(int n, const V4<double>* __restrict__ X, V4<float>* __restrict__ hi,
                        V4<float>* __restrict__ lo) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const V4<double> x = X[i];
    if (lo) {
        store_split(hi, lo, i, x.x, x.y, x.z);
    } else {
        hi[i] = V4<float>{(float)x.x, (float)x.y, (float)x.z, 0.f};
    }
}

template <typename T, typename S>
__global__ void k_copy_old(int nsim, const V4<S>* __restrict__ P, V4<S>* __restrict__ Pold,
                           const V4<T>* __restrict__ Ph, const V4<T>* __restrict__ Pl, V4<T>* __restrict__ Poh,
                           V4<T>* __restrict__ Pol, const OuterGate* __restrict__ gate) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nsim || outer_stopped(gate)) return;
    Pold[i] = P[i];
    if constexpr (kMirror<T, S>) {
        Poh[i] = Ph[i];
        Pol[i] = Pl[i];
    }
}

// one thread: the stopping rule of the outer loop (PdIpcSimulator::advance,
// cpp:1683-1796: stop once |dir|^2 < tol after the first iteration)
template <typename TC>
__global__ void k_outer_gate(OuterGate* __restrict__ g, const double* __restrict__ resid, const TC* __restrict__ toi,
                             const unsigned long long* __restrict__ active, double tol, int test) {
    if (g->stop) return;
    const int outer = g->iters;  // iterations tested so far: this one's index (graph-invariant)
    const double r = *resid;
    g->resid = r;
    g->iters = outer + 1;
    g->toi = (double)*toi;
    g->active = *active;
    if (test && outer > 0 && r < tol) g->stop = 1u;
}

// Per-instance stopping: |dir|^2 of every instance, one block per instance
// over its vertex range, in a fixed order.
template <typename S>
__global__ void k_inst_resid(const int* __restrict__ beg, const V4<S>* __restrict__ Dir, double* __restrict__ resid,
                             const OuterGate* __restrict__ gate) {
    if (outer_stopped(gate)) return;
    const int k = blockIdx.x;
    double acc = 0.0;
    for (int i = beg[k] + (int)threadIdx.x; i < beg[k + 1]; i += blockDim.x) {
        const V4<S> d = Dir[i];
        acc += (double)d.x * (double)d.x + (double)d.y * (double)d.y + (double)d.z * (double)d.z;
    }
    __shared__ double red[kBlock / 32];
    acc = warp_sum(acc);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
        resid[k] = t;
    }
}

// Per-instance stopping test after outer iteration `outer` (PdIpcSimulator.cpp:
// 1776 applied to each instance): a running instance counts the iteration and
// stops when test && outer > 0 && its |dir|^2 < tol.  The step's record: the
// loop stops once every instance has; resid the sum over the instances that ran.
template <typename TC>
__global__ void k_inst_gate(int ninst, unsigned* __restrict__ stop, int* __restrict__ iters,
                            const double* __restrict__ resid, OuterGate* __restrict__ g, const TC* __restrict__ toi,
                            const unsigned long long* __restrict__ active, double tol, int test) {
    if (g->stop) return;
    const int outer = g->iters;  // read by every thread before thread 0 writes it below
    __shared__ double rsum[kBlock];
    __shared__ int running[kBlock];
    double r = 0.0;
    int run = 0;
    for (int k = threadIdx.x; k < ninst; k += blockDim.x) {
        if (stop[k]) continue;
        const double rk = resid[k];
        r += rk;
        iters[k] = outer + 1;
        if (test && outer > 0 && rk < tol) stop[k] = 1u;
        else ++run;
    }
    rsum[threadIdx.x] = r;
    running[threadIdx.x] = run;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        int n = 0;
        for (int w = 0; w < (int)blockDim.x; ++w) {
            t += rsum[w];
            n += running[w];
        }
        g->resid = t;
        g->iters = outer + 1;
        g->toi = (double)*toi;
        g->active = *active;
        if (n == 0) g->stop = 1u;
    }
}

template <typename T>
__global__ void k_velocity(int nsim, T invt, const V4<T>* __restrict__ P, const V4<T>* __restrict__ X0,
                           V4<T>* __restrict__ Vel, unsigned int* __restrict__ err) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nsim) return;
    const V4<T> a = P[i], b = X0[i];
    if (!(isfinite(a.x) && isfinite(a.y) && isfinite(a.z))) atomicOr(err, (unsigned int)kErrNonFinite);
    Vel[i] = V4<T>{(a.x - b.x) * invt, (a.y - b.y) * invt, (a.z - b.z) * invt, T(0)};
}

}  // namespace

int direction_blocks(int nsim) { return std::min(1024, std::max(1, blocks_for(nsim))); }

template <typename T, typename TC>
constexpr bool correction_form() {
    return sizeof(T) == 4 && sizeof(TC) == 8;
}

template <typename T, typename TC>
void launch_predict(const Dev<T, TC>& d, TC dt, cudaStream_t s) {
    k_predict<T, TC, correction_form<T, TC>()><<<blocks_for(d.ntot), kBlock, 0, s>>>(
        d.nsim, d.ntot, dt, d.P, d.Pold, d.X0, d.Vel, d.Rhs0, d.Dinert, d.Grav, d.InvMass, d.PinFlag, d.CollDiag,
        d.CollRhs, d.Ph, d.Pl, d.Poh, d.Pol);
}
template <typename T, typename TC>
void launch_diag(const Dev<T, TC>& d, cudaStream_t s) {
    k_diag<T><<<blocks_for(d.nsim), kBlock, 0, s>>>(d.nsim, d.Delastic, d.Dinert, d.CollDiag, d.InvD);
}
template <typename T, typename TC>
void launch_tet_project(const Dev<T, TC>& d, cudaStream_t s) {
    if (d.ntet == 0) return;
    k_tet_project<T, TC><<<blocks_for(d.ntet, 128), 128, 0, s>>>(d.ntet, d.Tets, d.TetIdm, d.TetW, d.P, d.Ph, d.Pl,
                                                                d.TetOut, skip_of(d));
}
template <typename T, typename TC>
void launch_local_aq(const Dev<T, TC>& d, cudaStream_t s) {
    if constexpr (correction_form<T, TC>())
        k_local_aq_rel<<<blocks_for(d.nsim), kBlock, 0, s>>>(d.nsim, d.Ph, d.Pl, d.lPtr, d.tOff, d.tNbr, d.tLbo,
                                                              d.CurvNorm, d.Aq, skip_of(d));
    else
        k_local_aq<T><<<blocks_for(d.nsim), kBlock, 0, s>>>(d.nsim, d.P, d.lPtr, d.tOff, d.tNbr, d.tLbo, d.tLbo0,
                                                            d.CurvNorm, d.Aq, skip_of(d));
}
template <typename T, typename TC>
void launch_local_residual(const Dev<T, TC>& d, T relax, cudaStream_t s) {
    if constexpr (kMirror<T, TC>) {
        k_local_residual<T, TC><<<blocks_for(d.nsim), kBlock, 0, s>>>(
            d.nsim, relax, d.P, d.Ph, d.Pl, d.Pold, d.Xrest, d.Rhs0, d.Dinert, d.CollDiag, d.CollRhs, d.PinFlag,
            d.PinK, d.lPtr, d.tOff, d.tNbr, d.tRest, d.tBend0, d.tBendT, d.Strain, d.Aq, d.InvD, sell_of(d), d.ntet ? d.vtPtr : nullptr, d.vtIdx, d.TetOut, d.Rhs, d.Y,
            skip_of(d));
    }
}
template <typename T, typename TC>
void launch_sweep_delta(const Dev<T, TC>& d, int mode, const V4<T>* src, const V4<T>* prev, V4<T>* out, T relax,
                        T omega, cudaStream_t s) {
    const int nb = blocks_for(d.nsim);
#define PDIPC_SWEEP_DELTA(M)                                                                                   \
    case M:                                                                                                    \
        k_sweep_delta<T, TC, M><<<nb, kBlock, 0, s>>>(d.nsim, relax, omega, src, prev, out, d.P, d.Ph, d.Pl,  \
                                                      d.Rhs, d.InvD, sell_of(d), skip_of(d));          \
        break;
    switch (mode) {
        PDIPC_SWEEP_DELTA(0)
        PDIPC_SWEEP_DELTA(1)
        PDIPC_SWEEP_DELTA(3)
        PDIPC_SWEEP_DELTA(4)
        PDIPC_SWEEP_DELTA(5)
        PDIPC_SWEEP_DELTA(7)
        default:
            break;
    }
#undef PDIPC_SWEEP_DELTA
}
template <typename T, typename TC>
void launch_local_rhs_sweep(const Dev<T, TC>& d, T relax, cudaStream_t s) {
    if constexpr (std::is_same<T, TC>::value)
        k_local_rhs_sweep<T><<<blocks_for(d.nsim), kBlock, 0, s>>>(
            d.nsim, relax, d.P, d.lPtr, d.tOff, d.tNbr, d.tRest, d.tBend0, d.tBendT, d.Strain, d.Aq, d.Rhs0, d.CollRhs,
            d.PinRhs, d.InvD, sell_of(d), d.ntet ? d.vtPtr : nullptr, d.vtIdx, d.TetOut, d.Rhs,
            d.Y, skip_of(d));
}
template <typename T, typename TC>
void launch_sweep(const Dev<T, TC>& d, const V4<T>* src, const V4<T>* prev, V4<T>* out, T relax, T omega,
                  cudaStream_t s) {
    if (prev)
        k_sweep<T, true><<<blocks_for(d.nsim), kBlock, 0, s>>>(d.nsim, relax, omega, src, prev, out, d.Rhs, d.InvD,
                                                              sell_of(d), skip_of(d));
    else
        k_sweep<T, false><<<blocks_for(d.nsim), kBlock, 0, s>>>(d.nsim, relax, omega, src, prev, out, d.Rhs,
                                                               d.InvD, sell_of(d), skip_of(d));
}
template <typename T, typename TC>
void launch_direction(const Dev<T, TC>& d, cudaStream_t s) {
    const int nb = direction_blocks(d.nsim);
    k_direction<T, TC><<<nb, kBlock, 0, s>>>(d.nsim, d.P, d.Pold, d.Dir, d.Dh, d.ResidPart, d.Gate);
    launch_reduce_sum_f64(d.ResidPart, nb, d.Resid, s);
}
template <typename T, typename TC>
void launch_clamp(const Dev<T, TC>& d, cudaStream_t s) {
    k_clamp<T, TC><<<blocks_for(d.nsim), kBlock, 0, s>>>(d.nsim, d.Pold, d.Dir, d.Toi, d.P, d.Ph, d.Pl, d.Gate,
                                                          d.VInst, d.InstStop ? d.InstToi : nullptr);
}
template <typename T, typename TC>
void launch_split(const Dev<T, TC>& d, const V4<TC>* X, V4<T>* hi, V4<T>* lo, int n, cudaStream_t s) {
    if constexpr (kMirror<T, TC>) {
        if (n > 0) k_split<<<blocks_for(n), kBlock, 0, s>>>(n, X, hi, lo);
    }
}
template <typename T, typename TC>
void launch_copy_old(const Dev<T, TC>& d, cudaStream_t s) {
    k_copy_old<T, TC><<<blocks_for(d.nsim), kBlock, 0, s>>>(d.nsim, d.P, d.Pold, d.Ph, d.Pl, d.Poh, d.Pol, d.Gate);
}
template <typename T, typename TC>
void launch_outer_gate(const Dev<T, TC>& d, double tol, bool test, cudaStream_t s) {
    k_outer_gate<TC><<<1, 1, 0, s>>>(d.Gate, d.Resid, d.Toi, d.ActiveCount, tol, test ? 1 : 0);
}
template <typename T, typename TC>
void launch_inst_resid(const Dev<T, TC>& d, cudaStream_t s) {
    if (d.ninst > 0) k_inst_resid<TC><<<d.ninst, kBlock, 0, s>>>(d.InstBeg, d.Dir, d.InstResid, d.Gate);
}
template <typename T, typename TC>
void launch_inst_gate(const Dev<T, TC>& d, double tol, bool test, cudaStream_t s) {
    k_inst_gate<TC><<<1, kBlock, 0, s>>>(d.ninst, d.InstStop, d.InstIters, d.InstResid, d.Gate, d.Toi,
                                         d.ActiveCount, tol, test ? 1 : 0);
}
template <typename T, typename TC>
void launch_velocity(const Dev<T, TC>& d, TC invt, cudaStream_t s) {
    k_velocity<TC><<<blocks_for(d.nsim), kBlock, 0, s>>>(d.nsim, invt, d.P, d.X0, d.Vel, d.ErrFlags);
}

#define PDIPC_INST_PD(T, TC)                                                                                 \
    template void launch_predict<T, TC>(const Dev<T, TC>&, TC, cudaStream_t);                                 \
    template void launch_diag<T, TC>(const Dev<T, TC>&, cudaStream_t);                                       \
    template void launch_tet_project<T, TC>(const Dev<T, TC>&, cudaStream_t);                                \
    template void launch_local_aq<T, TC>(const Dev<T, TC>&, cudaStream_t);                                   \
    template void launch_local_rhs_sweep<T, TC>(const Dev<T, TC>&, T, cudaStream_t);                         \
    template void launch_local_residual<T, TC>(const Dev<T, TC>&, T, cudaStream_t);                          \
    template void launch_sweep_delta<T, TC>(const Dev<T, TC>&, int, const V4<T>*, const V4<T>*, V4<T>*, T, T, \
                                            cudaStream_t);                                                   \
    template void launch_sweep<T, TC>(const Dev<T, TC>&, const V4<T>*, const V4<T>*, V4<T>*, T, T,           \
                                      cudaStream_t);                                                         \
    template void launch_direction<T, TC>(const Dev<T, TC>&, cudaStream_t);                                  \
    template void launch_clamp<T, TC>(const Dev<T, TC>&, cudaStream_t);                                      \
    template void launch_copy_old<T, TC>(const Dev<T, TC>&, cudaStream_t);                                   \
    template void launch_outer_gate<T, TC>(const Dev<T, TC>&, double, bool, cudaStream_t);                   \
    template void launch_inst_resid<T, TC>(const Dev<T, TC>&, cudaStream_t);                                 \
    template void launch_inst_gate<T, TC>(const Dev<T, TC>&, double, bool, cudaStream_t);                    \
    template void launch_split<T, TC>(const Dev<T, TC>&, const V4<TC>*, V4<T>*, V4<T>*, int, cudaStream_t);  \
    template void launch_velocity<T, TC>(const Dev<T, TC>&, TC, cudaStream_t);

PDIPC_INST_PD(float, float)
PDIPC_INST_PD(double, double)
PDIPC_INST_PD(float, double)

}  // namespace pdipc
