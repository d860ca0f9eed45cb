// pd_persistent.cu — one cooperative launch per outer iteration for the whole
// projective-dynamics solve (lg x [local step + 15 Chebyshev-accelerated R2
// steps as 30 weighted-Jacobi sweeps]).
//
// Replaces, for FP32 state, the per-sweep launches of pd_kernels.cu (and the
// reference's 3 + 15 launches per local-global iteration with a device
// synchronisation after each, PdIpcGpuFunc.cu:1245-1346).  Layout:
//   * every CTA owns a contiguous run of SELL-32 slices (rows); when it fits,
//     its slice of the constant off-diagonal matrix N is copied once per launch
//     into shared memory: the FP32 values, and the column offsets as a per-row
//     index into a small table of distinct offset patterns (a structured mesh
//     has a few dozen); otherwise the matrix is streamed from L2;
//   * each thread owns R rows (one per slice it handles) and keeps their
//     current/previous iterate, right-hand side and inverse diagonal in registers;
//   * only the vector being gathered crosses CTAs (through L2, and through L1
//     once the synchronisation's acquire has invalidated it), between phases;
//   * a phase ends with neighbour synchronisation (each CTA waits only for the
//     CTAs it exchanges rows with) or, optionally, a grid barrier (a
//     counter/generation pair).
// Every wait is clock-bounded: on timeout it raises kErrBarrier and every later
// wait returns at once, so the kernel always terminates.  The launch is
// cooperative (all CTAs co-resident).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <type_traits>

#include "kernels.cuh"
#include "persistent.h"

namespace pdipc {

namespace {

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Grid barrier: every CTA's thread 0 arrives on one counter; the last arrival
// resets it and bumps the generation everybody else waits on (measured 1.8 us
// on 152 CTAs; a two-level counter tree was slower).  Waits are clock-bounded:
// on timeout (or a timeout seen elsewhere) the error bit is set and the barrier
// reports failure, so every CTA returns.  bar: [0] generation, [1] counter.
// Returns false when the grid is in error.
__device__ __forceinline__ bool grid_barrier(unsigned* bar, unsigned* err, unsigned nblocks, unsigned& my_gen,
                                             long long timeout_cycles) {
    __syncthreads();
    __shared__ int ok_s;
    if (threadIdx.x == 0) {
        int ok = 1;
        if (ld_acquire_gpu(err) & kErrBarrier) {
            ok = 0;
        } else {
            const unsigned g = my_gen;
            __threadfence();
            if (atomicAdd(bar + 1, 1u) + 1u == nblocks) {
                atomicExch(bar + 1, 0u);
                __threadfence();
                atomicExch(bar, g + 1u);
            } else {
                const long long t0 = clock64();
                while (ld_acquire_gpu(bar) == g) {
                    if (clock64() - t0 > timeout_cycles || (ld_acquire_gpu(err) & kErrBarrier)) {
                        atomicOr(err, (unsigned)kErrBarrier);
                        ok = 0;
                        break;
                    }
                    __nanosleep(8);
                }
            }
            my_gen = g + 1u;
        }
        ok_s = ok;
    }
    __syncthreads();
    return ok_s != 0;
}

__device__ __forceinline__ void st_release_gpu(unsigned* p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Neighbour synchronisation: a Jacobi sweep only reads the rows of the CTAs a
// CTA's matrix rows reach, so instead of a grid barrier each CTA publishes its
// phase count and waits for those CTAs only (the range is closed under "reads
// or is read by", so no CTA overwrites rows a neighbour is still reading).
// Neighbours can then be at most one phase apart.  Lanes of warp 0 poll one
// neighbour flag each; every wait is clock-bounded and gives up, raising
// kErrBarrier, when it times out or sees the error raised elsewhere.
__device__ __forceinline__ bool nbr_barrier(unsigned* flags, unsigned* err, int cta, int2 range, unsigned epoch,
                                            long long timeout_cycles) {
    __syncthreads();
    __shared__ int nok_s;
    if (threadIdx.x < 32) {
        if (threadIdx.x == 0) {
            __threadfence();
            st_release_gpu(flags + cta, epoch);
        }
        int ok = (ld_acquire_gpu(err) & kErrBarrier) ? 0 : 1;
        for (int n = range.x + (int)threadIdx.x; ok && n <= range.y; n += 32) {
            if (n == cta) continue;
            const long long t0 = clock64();
            while ((int)(ld_acquire_gpu(flags + n) - epoch) < 0) {
                if (clock64() - t0 > timeout_cycles || (ld_acquire_gpu(err) & kErrBarrier)) {
                    atomicOr(err, (unsigned)kErrBarrier);
                    ok = 0;
                    break;
                }
                __nanosleep(8);
            }
        }
        ok = __all_sync(0xffffffffu, ok);
        if (threadIdx.x == 0) nok_s = ok;
    }
    __syncthreads();
    return nok_s != 0;
}

__device__ __forceinline__ V4<float> ldcg4(const V4<float>* p, int i) {
    const float4 v = __ldcg(reinterpret_cast<const float4*>(p) + i);
    return V4<float>{v.x, v.y, v.z, v.w};
}
__device__ __forceinline__ V4<double> ldcg4(const V4<double>* p, int i) {
    const double2* q = reinterpret_cast<const double2*>(p) + 2 * (size_t)i;
    const double2 a = __ldcg(q), b = __ldcg(q + 1);
    return V4<double>{a.x, a.y, b.x, b.y};
}
// Coherent load that may hit in L1: data written by other CTAs before a grid
// barrier is visible after it, because the barrier's gpu-scope acquire
// invalidates this SM's L1 (PTX memory model: release -> acquire -> bar.sync).
__device__ __forceinline__ V4<float> ldl14(const V4<float>* p, int i) {
    const float4 v = *(reinterpret_cast<const float4*>(p) + i);
    return V4<float>{v.x, v.y, v.z, v.w};
}
__device__ __forceinline__ V4<double> ldl14(const V4<double>* p, int i) {
    const double2* q = reinterpret_cast<const double2*>(p) + 2 * (size_t)i;
    const double2 a = q[0], b = q[1];
    return V4<double>{a.x, a.y, b.x, b.y};
}
template <bool kL1, typename X>
__device__ __forceinline__ V4<X> ldv(const V4<X>* p, int i) {
    return kL1 ? ldl14(p, i) : ldcg4(p, i);
}
__device__ __forceinline__ void stcg4(V4<float>* p, int i, float x, float y, float z) {
    __stcg(reinterpret_cast<float4*>(p) + i, make_float4(x, y, z, 0.f));
}
__device__ __forceinline__ void stcg4(V4<double>* p, int i, double x, double y, double z) {
    double2* q = reinterpret_cast<double2*>(p) + 2 * (size_t)i;
    __stcg(q, make_double2(x, y));
    __stcg(q + 1, make_double2(z, 0.0));
}

// S is the state scalar: T in the direct form, double in the correction form,
// where positions enter the FP32 arithmetic as differences formed from their
// float-float mirror (Ph, Pl): no FP64 arithmetic in the per-neighbour loops.
template <typename T, typename S, bool kCorr, bool kSmem, bool kL1, int R>
__global__ void __launch_bounds__(1024, 1) k_pd_persistent(PersistArgs<T, S> a) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int cta = blockIdx.x;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // ---- this CTA's matrix values and the offset patterns into shared memory ----
    const int eb = a.ctaEntry[cta], ee = a.ctaEntry[cta + 1];
    const int E = ee - eb;
    T* sval = reinterpret_cast<T*>(smem);
    int16_t* spat = reinterpret_cast<int16_t*>(smem + ((size_t)E * sizeof(T) + 15) / 16 * 16);
    const size_t patBytes = ((size_t)a.patterns * a.patW * sizeof(int16_t) + 15) / 16 * 16;
    T* bx = reinterpret_cast<T*>(smem + ((size_t)E * sizeof(T) + 15) / 16 * 16 + patBytes);
    T* by = bx + a.bandMax;
    T* bz = by + a.bandMax;
    const bool band = kSmem && a.band != nullptr;
    const int2 brange = band ? a.band[cta] : make_int2(0, 0);
    if (kSmem) {
        for (int q = threadIdx.x; q < E; q += blockDim.x) sval[q] = __ldg(a.sVal + eb + q);
        for (int q = threadIdx.x; q < a.patterns * a.patW; q += blockDim.x) spat[q] = __ldg(a.patOff + q);
    }
    // ---- rows owned by this thread ----
    int row[R], gb[R], sl[R], pid[R];
    bool val[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int s = a.ctaSlice[cta] + warp * R + r;  // slice index
        const bool sv = s < a.ctaSlice[cta + 1];
        row[r] = s * 32 + lane;
        val[r] = sv && row[r] < a.nsim;
        gb[r] = sv ? a.sliceEntry[s] + lane : 0;
        sl[r] = sv ? a.sliceLen[s] : 0;
        pid[r] = (kSmem && val[r]) ? a.rowPattern[row[r]] * a.patW : 0;
    }
    // entry k of owned row r: value and gathered row
    auto entry = [&](int r, int k, T& v, int& j) {
        if (kSmem) {
            v = sval[gb[r] - eb + 32 * k];
            j = row[r] + (int)spat[pid[r] + k];
        } else {
            v = __ldg(a.sVal + gb[r] + 32 * k);
            j = __ldg(a.sCol + gb[r] + 32 * k);
        }
    };
    __syncthreads();
    unsigned my_gen = 0;
    if (threadIdx.x == 0) my_gen = ld_acquire_gpu(a.bar);
    const int2 nrange = a.nbr ? a.nbr[cta] : make_int2(0, -1);
    unsigned epoch = a.epoch0;
    // end of a phase: neighbour synchronisation or the grid barrier
    auto sync = [&]() -> bool {
        if (a.nbr) return nbr_barrier(a.flags, a.err, cta, nrange, ++epoch, a.timeout);
        return grid_barrier(a.bar, a.err, gridDim.x, my_gen, a.timeout);
    };
    const T w = a.relax, om1 = T(1) - a.relax;
    T id[R];
#pragma unroll
    for (int r = 0; r < R; ++r)
        id[r] = val[r] ? T(1) / ((a.Delastic[row[r]] + a.Dinert[row[r]]) + a.CollDiag[row[r]]) : T(0);

    // stage the band of src (all threads; the caller's rows then gather from it)
    auto stage = [&](const V4<T>* src) {
        if (!band) return;
        const int n = brange.y - brange.x;
        for (int q = threadIdx.x; q < n; q += blockDim.x) {
            const V4<T> v = ldv<kL1>(src, brange.x + q);
            bx[q] = v.x;
            by[q] = v.y;
            bz[q] = v.z;
        }
        __syncthreads();
    };
    // sum_k N_ik src_k for the owned rows: matrix from shared memory, src from
    // the staged band or gathered from global memory
    auto gather = [&](const V4<T>* src, int r, T& s0, T& s1, T& s2) {
        if (band) {
            s0 = T(0);
            s1 = T(0);
            s2 = T(0);
#pragma unroll 4
            for (int k = 0; k < sl[r]; ++k) {
                T v;
                int j;
                entry(r, k, v, j);
                const int q = j - brange.x;
                s0 += v * bx[q];
                s1 += v * by[q];
                s2 += v * bz[q];
            }
            return;
        }
        s0 = T(0);
        s1 = T(0);
        s2 = T(0);
#pragma unroll 4
        for (int k = 0; k < sl[r]; ++k) {
            T v;
            int j;
            entry(r, k, v, j);
            const V4<T> xj = ldv<kL1>(src, j);
            s0 += v * xj.x;
            s1 += v * xj.y;
            s2 += v * xj.z;
        }
    };

    for (int lg = 0; lg < a.lg; ++lg) {
        // ---- curvature vectors of the owned rows ----
#pragma unroll
        for (int r = 0; r < R; ++r) {
            if (!val[r]) continue;
            const int i = row[r];
            const int b = a.lPtr[i], e = a.lPtr[i + 1];
            T a0, a1, a2;
            if constexpr (kCorr) {
                const V4<T> h = ldv<kL1>(a.Ph, i), l = ldv<kL1>(a.Pl, i);
                a0 = a1 = a2 = T(0);
                for (int s = b + 1; s < e; ++s) {
                    const int j = a.lNbr[s];
                    const V4<T> hj = ldv<kL1>(a.Ph, j), lj = ldv<kL1>(a.Pl, j);
                    const T wl = a.lLbo[s];
                    a0 += wl * diff_ff(hj.x, lj.x, h.x, l.x);
                    a1 += wl * diff_ff(hj.y, lj.y, h.y, l.y);
                    a2 += wl * diff_ff(hj.z, lj.z, h.z, l.z);
                }
            } else {
                const V4<S> x = ldv<kL1>(a.P, i);
                const T l0 = a.lLbo[b];
                a0 = x.x * l0;
                a1 = x.y * l0;
                a2 = x.z * l0;
                for (int s = b + 1; s < e; ++s) {
                    const V4<T> xj = ldv<kL1>(a.P, a.lNbr[s]);
                    const T l = a.lLbo[s];
                    a0 += xj.x * l;
                    a1 += xj.y * l;
                    a2 += xj.z * l;
                }
            }
            const T nrm = sqrtf(a0 * a0 + a1 * a1 + a2 * a2);
            if (nrm >= T(1e-10)) {
                const T c = a.CurvNorm[i] / nrm;
                a0 *= c;
                a1 *= c;
                a2 *= c;
            }
            stcg4(a.Aq, i, a0, a1, a2);
        }
        if (!sync()) return;

        // ---- right-hand side (direct) or residual (correction) of the owned rows ----
        T x0[R][3], rh[R][3];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            x0[r][0] = x0[r][1] = x0[r][2] = T(0);
            rh[r][0] = rh[r][1] = rh[r][2] = T(0);
            if (!val[r]) continue;
            const int i = row[r];
            const int b = a.lPtr[i], e = a.lPtr[i + 1];
            const V4<S> x = ldv<kL1>(a.P, i);
            const T strain = a.Strain[i];
            if constexpr (kCorr) {
                Sum2 r0, r1, r2;
                {
                    const V4<S> y = ldcg4(a.Rhs0, i);
                    const T di = a.Dinert[i];
                    r0.add(di * (T)(y.x - x.x));
                    r1.add(di * (T)(y.y - x.y));
                    r2.add(di * (T)(y.z - x.z));
                }
                const int pf = a.PinFlag[i];
                if (pf >= 0) {
                    const V4<S> xr = ldcg4(a.Xrest, i);
                    const T k = a.PinK[pf];
                    r0.add(k * (T)(xr.x - x.x));
                    r1.add(k * (T)(xr.y - x.y));
                    r2.add(k * (T)(xr.z - x.z));
                }
                {
                    const V4<T> c = ldcg4(a.CollRhs, i);
                    const V4<S> xo = ldcg4(a.Pold, i);
                    const T dc = a.CollDiag[i];
                    r0.add(c.x);
                    r0.add(dc * (T)(xo.x - x.x));
                    r1.add(c.y);
                    r1.add(dc * (T)(xo.y - x.y));
                    r2.add(c.z);
                    r2.add(dc * (T)(xo.z - x.z));
                }
                const V4<T> h = ldv<kL1>(a.Ph, i), l = ldv<kL1>(a.Pl, i);
                for (int s = b + 1; s < e; ++s) {
                    const int j = a.lNbr[s];
                    const V4<T> hj = ldv<kL1>(a.Ph, j), lj = ldv<kL1>(a.Pl, j);
                    const T d0 = diff_ff(h.x, l.x, hj.x, lj.x), d1 = diff_ff(h.y, l.y, hj.y, lj.y),
                            d2 = diff_ff(h.z, l.z, hj.z, lj.z);
                    const T cl = sqrtf(d0 * d0 + d1 * d1 + d2 * d2);
                    const T rc = strain * (a.lRest[s] / cl);
                    r0.add(rc * d0);
                    r1.add(rc * d1);
                    r2.add(rc * d2);
                }
                const V4<T> ai = ldv<kL1>(a.Aq, i);
                const T b0 = a.lBend[b];
                r0.add(b0 * ai.x);
                r1.add(b0 * ai.y);
                r2.add(b0 * ai.z);
                for (int s = b + 1; s < e; ++s) {
                    const V4<T> ak = ldv<kL1>(a.Aq, a.lNbr[s]);
                    const T bt = a.lBendT[s];
                    r0.add(bt * ak.x);
                    r1.add(bt * ak.y);
                    r2.add(bt * ak.z);
                }
                for (int k = 0; k < sl[r]; ++k) {
                    T v;
                    int j;
                    entry(r, k, v, j);
                    const V4<T> hj = ldv<kL1>(a.Ph, j), lj = ldv<kL1>(a.Pl, j);
                    r0.add(v * diff_ff(hj.x, lj.x, h.x, l.x));
                    r1.add(v * diff_ff(hj.y, lj.y, h.y, l.y));
                    r2.add(v * diff_ff(hj.z, lj.z, h.z, l.z));
                }
                rh[r][0] = r0.value();
                rh[r][1] = r1.value();
                rh[r][2] = r2.value();
            } else {
                x0[r][0] = x.x;
                x0[r][1] = x.y;
                x0[r][2] = x.z;
                T t0 = T(0), t1 = T(0), t2 = T(0);
                for (int s = b + 1; s < e; ++s) {
                    const V4<T> xj = ldv<kL1>(a.P, a.lNbr[s]);
                    const T d0 = x.x - xj.x, d1 = x.y - xj.y, d2 = x.z - xj.z;
                    const T cl = sqrtf(d0 * d0 + d1 * d1 + d2 * d2);
                    const T rc = strain * (a.lRest[s] / cl);
                    t0 += rc * d0;
                    t1 += rc * d1;
                    t2 += rc * d2;
                }
                const V4<T> ai = ldv<kL1>(a.Aq, i);
                const T b0 = a.lBend[b];
                t0 += b0 * ai.x;
                t1 += b0 * ai.y;
                t2 += b0 * ai.z;
                const V4<T> q0 = ldcg4(a.Rhs0, i);
                T u0 = q0.x + t0, u1 = q0.y + t1, u2 = q0.z + t2;
                for (int s = b + 1; s < e; ++s) {
                    const V4<T> ak = ldv<kL1>(a.Aq, a.lNbr[s]);
                    const T bt = a.lBendT[s];
                    u0 += bt * ak.x;
                    u1 += bt * ak.y;
                    u2 += bt * ak.z;
                }
                const V4<T> c = ldcg4(a.CollRhs, i);
                u0 += c.x;
                u1 += c.y;
                u2 += c.z;
                const V4<T> pn = ldcg4(a.PinRhs, i);
                u0 += pn.x;
                u1 += pn.y;
                u2 += pn.z;
                rh[r][0] = u0;
                rh[r][1] = u1;
                rh[r][2] = u2;
            }
        }

        // ---- Chebyshev-accelerated R2 iteration as two J sweeps per step ----
        // direct form: iterate on x from x0 (gathered from P);
        // correction form: iterate on delta from 0, add it to P at the end.
        T cx[R][3], px[R][3], yv[R][3];
        // first sweep: Y = S(x0)
        if constexpr (!kCorr) stage(a.P);
#pragma unroll
        for (int r = 0; r < R; ++r) {
            T s0 = T(0), s1 = T(0), s2 = T(0);
            if constexpr (kCorr) {
                cx[r][0] = cx[r][1] = cx[r][2] = T(0);
            } else {
                cx[r][0] = x0[r][0];
                cx[r][1] = x0[r][1];
                cx[r][2] = x0[r][2];
                if (val[r]) gather(a.P, r, s0, s1, s2);
            }
            yv[r][0] = om1 * cx[r][0] + w * ((s0 + rh[r][0]) * id[r]);
            yv[r][1] = om1 * cx[r][1] + w * ((s1 + rh[r][1]) * id[r]);
            yv[r][2] = om1 * cx[r][2] + w * ((s2 + rh[r][2]) * id[r]);
            if (val[r]) stcg4(a.GY, row[r], yv[r][0], yv[r][1], yv[r][2]);
        }
        if (!sync()) return;
        const int nsteps = a.cheby;
        for (int it = 0; it < nsteps; ++it) {
            const bool last = it == nsteps - 1;
            // second sweep of the step: S(Y), Chebyshev-combined except for the first step
            const T om = a.omega[it];
            stage(a.GY);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                T s0 = T(0), s1 = T(0), s2 = T(0);
                if (val[r]) gather(a.GY, r, s0, s1, s2);
                T n0 = om1 * yv[r][0] + w * ((s0 + rh[r][0]) * id[r]);
                T n1 = om1 * yv[r][1] + w * ((s1 + rh[r][1]) * id[r]);
                T n2 = om1 * yv[r][2] + w * ((s2 + rh[r][2]) * id[r]);
                if (it > 0) {
                    n0 = om * (n0 - px[r][0]) + px[r][0];
                    n1 = om * (n1 - px[r][1]) + px[r][1];
                    n2 = om * (n2 - px[r][2]) + px[r][2];
                }
                px[r][0] = cx[r][0];
                px[r][1] = cx[r][1];
                px[r][2] = cx[r][2];
                cx[r][0] = n0;
                cx[r][1] = n1;
                cx[r][2] = n2;
                if (!val[r]) continue;
                if (last) {
                    if constexpr (kCorr) {  // only this thread writes the row: its own earlier read is current
                        const V4<S> x = ldcg4(a.P, row[r]);
                        const S q0 = x.x + (S)n0, q1 = x.y + (S)n1, q2 = x.z + (S)n2;
                        stcg4(a.P, row[r], q0, q1, q2);
                        float h0, l0, h1, l1, h2, l2;
                        split_ff(q0, h0, l0);
                        split_ff(q1, h1, l1);
                        split_ff(q2, h2, l2);
                        stcg4(a.Ph, row[r], h0, h1, h2);
                        stcg4(a.Pl, row[r], l0, l1, l2);
                    } else {
                        stcg4(a.P, row[r], n0, n1, n2);
                    }
                } else {
                    stcg4(a.GX, row[r], n0, n1, n2);
                }
            }
            if (!sync()) return;
            if (last) break;
            // first sweep of the next step: Y = S(x)
            stage(a.GX);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                T s0 = T(0), s1 = T(0), s2 = T(0);
                if (val[r]) gather(a.GX, r, s0, s1, s2);
                yv[r][0] = om1 * cx[r][0] + w * ((s0 + rh[r][0]) * id[r]);
                yv[r][1] = om1 * cx[r][1] + w * ((s1 + rh[r][1]) * id[r]);
                yv[r][2] = om1 * cx[r][2] + w * ((s2 + rh[r][2]) * id[r]);
                if (val[r]) stcg4(a.GY, row[r], yv[r][0], yv[r][1], yv[r][2]);
            }
            if (!sync()) return;
        }
    }
}

template <typename T, bool kCorr, bool kSmem, bool kL1>
const void* kernel_for(int R) {
    using S = typename std::conditional<kCorr, double, T>::type;
    switch (R) {
        case 1: return (const void*)k_pd_persistent<T, S, kCorr, kSmem, kL1, 1>;
        case 2: return (const void*)k_pd_persistent<T, S, kCorr, kSmem, kL1, 2>;
        case 3: return (const void*)k_pd_persistent<T, S, kCorr, kSmem, kL1, 3>;
        default: return (const void*)k_pd_persistent<T, S, kCorr, kSmem, kL1, 4>;
    }
}

template <bool kL1>
const void* kernel_for_l1(bool correction, bool matrix_in_smem, int R) {
    if (correction)
        return matrix_in_smem ? kernel_for<float, true, true, kL1>(R) : kernel_for<float, true, false, kL1>(R);
    return matrix_in_smem ? kernel_for<float, false, true, kL1>(R) : kernel_for<float, false, false, kL1>(R);
}

}  // namespace

const void* persistent_kernel(bool correction, bool matrix_in_smem, bool l1_gather, int rows_per_thread) {
    return l1_gather ? kernel_for_l1<true>(correction, matrix_in_smem, rows_per_thread)
                     : kernel_for_l1<false>(correction, matrix_in_smem, rows_per_thread);
}

template <typename S>
cudaError_t launch_args(const PersistPlan& plan, const PersistArgs<float, S>& args, cudaStream_t s) {
    const bool correction = std::is_same<S, double>::value;
    const void* f = persistent_kernel(correction, plan.matrix_in_smem, plan.l1_gather, plan.rows_per_thread);
    void* params[] = {(void*)&args};
    return cudaLaunchCooperativeKernel(f, dim3(plan.ctas), dim3(plan.threads), params, plan.smem_bytes, s);
}

cudaError_t launch_pd_persistent(const PersistPlan& plan, const PersistArgs<float, float>& args, cudaStream_t s) {
    return launch_args(plan, args, s);
}
cudaError_t launch_pd_persistent(const PersistPlan& plan, const PersistArgs<float, double>& args, cudaStream_t s) {
    return launch_args(plan, args, s);
}

}  // namespace pdipc
