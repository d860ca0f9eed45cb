#pragma once
// pd_persistent.cuh — one cooperative launch per outer iteration for the whole
// projective-dynamics solve (lg x [local step + 15 Chebyshev-accelerated R2
// steps as 30 weighted-Jacobi sweeps]).
//
// Replaces, for FP32 solver arithmetic, the per-sweep launches of pd_kernels.cu
// (and the reference's 3 + 15 launches per local-global iteration with a device
// synchronisation after each, PdIpcGpuFunc.cu:1245-1346).  Layout:
//   * every CTA owns a contiguous run of SELL-32 slices (rows); when it fits,
//     its slice of the constant off-diagonal matrix N is copied once per launch
//     into shared memory: the FP32 values, and the column offsets as a per-row
//     index into a small table of distinct offset patterns (a structured mesh
//     has a few dozen); otherwise the matrix is streamed from L2;
//   * each thread owns R rows (one per slice it handles) and keeps their
//     right-hand side and inverse diagonal in registers;
//   * a phase ends with neighbour synchronisation (each CTA waits only for the
//     CTAs it exchanges rows with) or, optionally, a grid barrier (a
//     counter/generation pair);
//   * band path (mixed precision, kMode 2): the iterate's band of the CTA stays
//     in shared memory as three planar float arrays (own rows written by the
//     CTA's threads, the halo filled by cp.async.bulk copies from the planar
//     global iterate on an mbarrier), the offset patterns come
//     from parameter space, and one extra warp without rows publishes each
//     sweep, polls the neighbours and issues the copies while the row warps sum
//     their entries on own rows; other paths gather the iterate from global
//     memory (through L1 once the synchronisation's acquire has invalidated it).
// Every wait is clock-bounded: on timeout it raises kErrBarrier and every later
// wait returns at once, so the kernel always terminates.  The launch is
// cooperative (all CTAs co-resident).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <type_traits>

#include "kernels.cuh"
#include "persistent.h"
#include "svd3.cuh"

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

// ---- bulk copies (TMA engine) into shared memory, completed on an mbarrier ----
__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
// one arrival that also expects `bytes` of copies to complete on the barrier
__device__ __forceinline__ void mbar_arrive_expect(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
    unsigned done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}
// a plain arrival (no bytes expected): completes the phase without a copy
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}
// global -> shared bulk copy; addresses 16-byte aligned, bytes a multiple of 16
__device__ __forceinline__ void bulk_load(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

// Neighbour synchronisation: a Jacobi sweep only reads the rows of the CTAs a
// CTA's matrix rows reach, so instead of a grid barrier each CTA publishes its
// phase count and waits for those CTAs only (the range is closed under "reads
// or is read by", so no CTA overwrites rows a neighbour is still reading).
// Neighbours can then be at most one phase apart.  Publishing and waiting are
// separate steps so that a CTA can work on its own rows in between.
//
// nbr_publish: the caller has passed a __syncthreads() after its writes of the
// phase; thread 0 releases the phase count.  No separate fence: the CTA
// barrier synchronises every thread's writes with thread 0, and the release
// store at GPU scope is cumulative over what precedes it in causality order,
// so a neighbour whose acquire load reads the count sees all of them.
__device__ __forceinline__ void nbr_publish(unsigned* flags, int cta, unsigned epoch) {
    if (threadIdx.x == 0) st_release_gpu(flags + cta, epoch);
}

// nbr_wait: lanes of warp 0 poll one neighbour flag each until it reaches
// epoch; ends with __syncthreads(), after which the neighbours' writes of that
// phase are visible to every thread.  Every wait is clock-bounded and gives up,
// raising kErrBarrier, when it times out or sees the error raised elsewhere.
__device__ __forceinline__ bool nbr_wait(const unsigned* flags, unsigned* err, int cta, int2 range, unsigned epoch,
                                         long long timeout_cycles) {
    __shared__ int nok_s;
    if (threadIdx.x < 32) {
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

__device__ __forceinline__ bool nbr_barrier(unsigned* flags, unsigned* err, int cta, int2 range, unsigned epoch,
                                            long long timeout_cycles) {
    __syncthreads();
    nbr_publish(flags, cta, epoch);
    return nbr_wait(flags, err, cta, range, epoch, timeout_cycles);
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

// One tet's strain projection (solveVolumetricStrainConstraintKernel,
// PdIpcGpuFunc.cu:439-599) inside the persistent solve: Ds from the current
// positions (the float-float mirror in the correction form), w R G to TetOut.
// Out of line: it runs once per tet and local-global iteration, and its
// registers stay out of the sweeps.  Positions come from L2 (written by other
// CTAs earlier in the launch).
template <typename S, bool kCorr>
__device__ __noinline__ void tet_project_one(int e, const int4* __restrict__ Tets, const float* __restrict__ Idm,
                                             const float* __restrict__ W, const V4<S>* __restrict__ P,
                                             const V4<float>* __restrict__ Ph, const V4<float>* __restrict__ Pl,
                                             V4<float>* __restrict__ Out) {
    const int4 q = Tets[e];
    const bool tri = q.w < 0;  // a cloth triangle's strain element: no fourth vertex
    const int id[4] = {q.x, q.y, q.z, tri ? q.x : q.w};
    float Ds[3][3];
    if constexpr (kCorr) {
        const V4<float> h0 = ldcg4(Ph, id[0]), l0 = ldcg4(Pl, id[0]);
        for (int c = 0; c < 3; ++c) {
            const V4<float> h = ldcg4(Ph, id[c + 1]), l = ldcg4(Pl, id[c + 1]);
            Ds[0][c] = diff_ff(h.x, l.x, h0.x, l0.x);
            Ds[1][c] = diff_ff(h.y, l.y, h0.y, l0.y);
            Ds[2][c] = diff_ff(h.z, l.z, h0.z, l0.z);
        }
    } else {
        const V4<S> x0 = ldcg4(P, id[0]);
        for (int c = 0; c < 3; ++c) {
            const V4<S> x = ldcg4(P, id[c + 1]);
            Ds[0][c] = x.x - x0.x;
            Ds[1][c] = x.y - x0.y;
            Ds[2][c] = x.z - x0.z;
        }
    }
    float idm[9];
    for (int k = 0; k < 9; ++k) idm[k] = __ldg(Idm + 9 * (size_t)e + k);
    float out[4][3];
    if (tri) {
        const float D2[3][2] = {{Ds[0][0], Ds[0][1]}, {Ds[1][0], Ds[1][1]}, {Ds[2][0], Ds[2][1]}};
        float o3[3][3];
        svd::tri_project<float>(D2, idm, __ldg(W + e), o3);
        for (int c = 0; c < 3; ++c)
            for (int r = 0; r < 3; ++r) out[c][r] = o3[c][r];
        out[3][0] = out[3][1] = out[3][2] = 0.f;
    } else {
        svd::tet_project<float>(Ds, idm, __ldg(W + e), out);
    }
    for (int c = 0; c < 4; ++c) __stcg(reinterpret_cast<float4*>(Out) + 4 * (size_t)e + c, make_float4(out[c][0], out[c][1], out[c][2], 0.f));
}

// A CTA without rows to update in a launch (rows of other groups, or of
// stopped instances; the rule of row_valid in k_pd_persistent) takes no part:
// with neighbour synchronisation it publishes the launch's last phase at once
// (its rows are read by no row that is updated) and returns.  Out of line, so
// that the solve's register allocation does not carry it.
template <typename T, typename S, int R>
__device__ __noinline__ bool cta_idle(const PersistArgs<T, S>& a, int cta, int nrw) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    bool any = false;
    for (int r = 0; r < R; ++r) {
        const int s = a.ctaSlice[cta] + warp * R + r;
        if (warp >= nrw || s >= a.ctaSlice[cta + 1]) continue;
        const int row = row_of(s * 32 + lane);
        any = any || (row >= a.row0 && row < a.row1 && row < a.nsim &&
                      !(a.instStop && __ldg(a.instStop + __ldg(a.vInst + row))));
    }
    if (__syncthreads_or(any) || !a.nbr) return false;
    if (threadIdx.x == 0) {
        __threadfence();
        st_release_gpu(a.flags + cta, a.epoch0 + a.nphases);
    }
    return true;
}

// S is the state scalar: T in the direct form, double in the correction form,
// where positions enter the FP32 arithmetic as differences formed from their
// float-float mirror (Ph, Pl): no FP64 arithmetic in the per-neighbour loops.
// kMode bits 0-1: 0 matrix streamed from L2; 1 matrix in shared memory, gathers
// from global memory; 2 matrix and the band of the iterate in shared memory,
// offset patterns in parameter space; 3 the same with the CTA's own offset
// patterns in shared memory.  In shared memory (modes 1 and 3) a CTA keeps only
// the patterns of its own rows (ctaPat[cta] .. ctaPat[cta + 1] of patLocal),
// indexed by the rows' local ids (rowPatLocal).
// Bit 2: the scene has tets (compiled in only then: the projection's call
// costs the cloth-only kernel 7% through register allocation).
template <typename T, typename S, bool kCorr, int kMode, bool kL1, int R>
__global__ void __launch_bounds__(kMaxPersistWarps * 32, 1) k_pd_persistent(const __grid_constant__ PersistArgs<T, S> a) {
    constexpr bool kTets = (kMode & 4) != 0;
    constexpr bool kSmem = (kMode & 3) >= 1;
    constexpr bool band = (kMode & 3) >= 2;
    constexpr bool patParam = (kMode & 3) == 2;
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int abort_s;  // band path: a neighbour wait failed, every warp returns
    // the outer loop stopped at an earlier iteration: every CTA returns before
    // its first phase; flags and barrier counters stay as they are (the next
    // launch's phase numbers lie above them all the same)
    if (outer_stopped(a.gate)) return;
    const int cta = (int)blockIdx.x + a.ctaLo;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // Row r of this thread (slice ctaSlice[cta] + warp R + r, lane) is
    // updated in this launch when it is simulated, in [row0, row1) and its
    // instance has not stopped.
    const int nrw = (int)(blockDim.x >> 5) - (band ? 1 : 0);
    auto row_valid = [&](int r) -> bool {
        const int s = a.ctaSlice[cta] + warp * R + r;
        if (warp >= nrw || s >= a.ctaSlice[cta + 1]) return false;
        const int row = row_of(s * 32 + lane);
        return row >= a.row0 && row < a.row1 && row < a.nsim &&
               !(a.instStop && __ldg(a.instStop + __ldg(a.vInst + row)));
    };
    if (cta_idle<T, S, R>(a, cta, nrw)) return;
    // ---- this CTA's matrix values and the offset patterns into shared memory ----
    const int eb = a.ctaEntry[cta], ee = a.ctaEntry[cta + 1];
    const int E = ee - eb;
    T* sval = reinterpret_cast<T*>(smem);
    int16_t* spat = reinterpret_cast<int16_t*>(smem + ((size_t)E * sizeof(T) + 15) / 16 * 16);
    // this CTA's patterns (kMode 2 reads the whole table from parameter space)
    const int pat0 = (kSmem && !patParam) ? a.ctaPat[cta] : 0;
    const int npat = (kSmem && !patParam) ? a.ctaPat[cta + 1] - pat0 : 0;
    const size_t patBytes = ((size_t)npat * a.patW * sizeof(int16_t) + 15) / 16 * 16;
    // the band of the iterate, slots [brange.x, brange.y), as three planar
    // arrays of bandW floats (the own rows written by this CTA's threads after
    // every sweep, the halo on each side copied in bulk from the planar global
    // iterate), then the copies' mbarrier
    unsigned char* bandp = smem + ((size_t)E * sizeof(T) + 15) / 16 * 16 + patBytes;
    const int bandW = a.ownMax + a.haloMax;  // a multiple of 64 (whole windows)
    T* bx = reinterpret_cast<T*>(bandp);
    T* by = bx + bandW;
    T* bz = by + bandW;
    uint64_t* mbar = reinterpret_cast<uint64_t*>(bandp + (3 * (size_t)bandW * sizeof(T) + 15) / 16 * 16);
    const int2 brange = band ? a.band[cta] : make_int2(0, 0);
    if (kSmem) {
        for (int q = threadIdx.x; q < E; q += blockDim.x) sval[q] = __ldg(a.sVal + eb + q);
        for (int q = threadIdx.x; q < npat * a.patW; q += blockDim.x)
            spat[q] = __ldg(a.patLocal + (size_t)pat0 * a.patW + q);
    }
    if (band && threadIdx.x == 0) {
        mbar_init(mbar, 1);
        abort_s = 0;
    }
    // ---- rows owned by this thread: one per slice, the warp's R slices
    // consecutive; the band path's last warp has no rows ----
    // pk[r] packs the row's entry count (bits 0-9) and, on the band path, the
    // bounds of its entries on own rows (bits 10-19, 20-29).  slotof(r) is the
    // row's slot (its place in the matrix slices), rowof(r) the row itself
    // (state arrays), itof(r) = swz(rowof(r)) its place in the iterates and the band.
    const int slot0 = (a.ctaSlice[cta] + warp * R) * 32 + lane;
    auto slotof = [&](int r) { return slot0 + 32 * r; };
    auto rowof = [&](int r) { return row_of(slot0 + 32 * r); };
    auto itof = [&](int r) { return swz(row_of(slot0 + 32 * r)); };
    int gb[R], pk[R], pid[R];
    bool val[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int s = a.ctaSlice[cta] + warp * R + r;
        const bool sv = warp < nrw && s < a.ctaSlice[cta + 1];
        val[r] = row_valid(r);
        gb[r] = sv ? a.sliceEntry[s] + lane : 0;
        pk[r] = sv ? a.sliceLen[s] : 0;
        pid[r] = (kSmem && val[r]) ? (patParam ? a.rowPattern : a.rowPatLocal)[rowof(r)] * a.patW : 0;
    }
    auto slen = [&](int r) { return pk[r] & 1023; };
    // entry k of the row `row` whose SELL entries start at g (pattern p):
    // value and gathered row (a row, not a slot); entry(r, ...) for owned row r
    auto entry_at = [&](int g, int p, int row, int k, T& v, int& j) {
        if (kSmem) {
            v = sval[g - eb + 32 * k];
            j = row + (int)(patParam ? a.patc[p + k] : spat[p + k]);
        } else {
            v = __ldg(a.sVal + g + 32 * k);
            j = __ldg(a.sCol + g + 32 * k);
        }
    };
    auto entry = [&](int r, int k, T& v, int& j) { entry_at(gb[r], pid[r], rowof(r), k, v, j); };
    __syncthreads();
    unsigned my_gen = 0;
    if (threadIdx.x == 0) my_gen = ld_acquire_gpu(a.bar);
    // the neighbours within this launch's group (the instances of its rows lie inside it)
    const int2 nrange = [&]() {
        const int2 n = a.nbr ? a.nbr[cta] : make_int2(0, -1);
        return make_int2(max(n.x, a.ctaLo), min(n.y, a.ctaHi));
    }();
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
        id[r] = val[r] ? T(1) / ((a.Delastic[rowof(r)] + a.Dinert[rowof(r)]) + a.CollDiag[rowof(r)]) : T(0);

    // ---- the band: this CTA's own rows and the halo its matrix rows reach ----
    // Own slots [own0, own1) live in the planar arrays; between sweeps each
    // thread writes its rows' new values there.  The halo, slots
    // [brange.x, own0) and [own1, brange.y), is copied from global memory in
    // two bulk copies once the neighbours have published it.  A CTA owns whole
    // 64-row windows (which swz maps onto themselves), so the own and halo
    // ranges are the same in rows and in the iterates' swizzled order.
    const int own0 = a.ctaSlice[cta] * 32, own1 = min(a.ctaSlice[cta + 1] * 32, a.nslot);
    const int nlo = band ? own0 - brange.x : 0, nhi = band ? brange.y - own1 : 0;
    // The band path runs one extra warp, the last, with no rows: it publishes
    // each sweep, polls the neighbours' flags and issues the halo copies, so
    // the compute warps never wait on a flag.  Compute warps wait for a copy
    // on the mbarrier (clock-bounded); abort_s ends the launch for all warps
    // when a neighbour wait has failed.
    const bool syncw = band && warp == (int)(blockDim.x >> 5) - 1;
    const unsigned ncomp = blockDim.x - 32u;
    // barrier of the compute warps alone (band path: the sync warp does not take part)
    auto comp_bar = [&]() { asm volatile("bar.sync 1, %0;" ::"r"(ncomp) : "memory"); };
    unsigned mphase = 0;
    // sync warp: optionally wait until the neighbours have published phase
    // `epoch`, then copy the halo of src.  The whole poll has one deadline (a
    // lane that polls several neighbours does not restart its clock), so the
    // warp has either issued the copies or arrived without them within
    // a.timeout of entering; the compute warps start waiting later than that
    // and give up only after 2 * a.timeout.
    auto issue_halo = [&](const V4<T>* src, bool poll) -> bool {
        int ok = (ld_acquire_gpu(a.err) & kErrBarrier) ? 0 : 1;
        const long long t0 = clock64();
        for (int n = nrange.x + lane; poll && ok && n <= nrange.y; n += 32) {
            if (n == cta) continue;
            while ((int)(ld_acquire_gpu(a.flags + n) - epoch) < 0) {
                if (clock64() - t0 > a.timeout || (ld_acquire_gpu(a.err) & kErrBarrier)) {
                    atomicOr(a.err, (unsigned)kErrBarrier);
                    ok = 0;
                    break;
                }
                __nanosleep(8);
            }
        }
        ok = __all_sync(0xffffffffu, ok);
        if (lane == 0) {
            if (ok) {
                // the neighbours' generic-proxy writes (acquired) and this CTA's
                // earlier reads of the halo area come before the async-proxy copy
                asm volatile("fence.proxy.async.global;" ::: "memory");
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                // per plane: slots [brange.x, own0) and [own1, brange.y), all
                // offsets and sizes multiples of 64 floats (whole windows)
                mbar_arrive_expect(mbar, (unsigned)(nlo + nhi) * 3u * (unsigned)sizeof(T));
                const T* sp = reinterpret_cast<const T*>(src);
                for (int pl = 0; pl < 3; ++pl) {
                    const T* plane = sp + (size_t)pl * a.nslot;
                    T* dst = bx + (size_t)pl * bandW;
                    if (nlo > 0) bulk_load(dst, plane + brange.x, (unsigned)nlo * (unsigned)sizeof(T), mbar);
                    if (nhi > 0)
                        bulk_load(dst + (own1 - brange.x), plane + own1, (unsigned)nhi * (unsigned)sizeof(T), mbar);
                }
            } else {
                abort_s = 1;
                mbar_arrive(mbar);
            }
        }
        __syncwarp();
        return ok != 0;
    };
    // compute warps: wait for the halo copy; false when the launch is ending.
    // The phase completes either when the copies land or when the sync warp
    // gives up and arrives without copies (abort_s set first).  Past the
    // limit, the error bit makes the sync warp's poll give up at once, and
    // the warps keep waiting (bounded) for the phase: leaving earlier could
    // end the CTA while a bulk copy still writes its shared memory.  When the
    // copies did land, the sweep finishes normally and the launch ends at the
    // sync warp's next poll, which sees the error bit; so no warp returns
    // while another waits for it at a CTA barrier.
    auto halo_ready = [&]() -> bool {
        const long long t0 = clock64();
        bool raised = false;
        while (!mbar_try_wait(mbar, mphase)) {
            const long long dt = clock64() - t0;
            if (!raised && dt > 2 * a.timeout) {
                atomicOr(a.err, (unsigned)kErrBarrier);
                raised = true;
            }
            if (dt > 4 * a.timeout) return false;  // the sync warp stopped too: nothing is in flight
        }
        mphase ^= 1u;
        return *((volatile int*)&abort_s) == 0;
    };
    // Entries are in column order, so an owned row's entries split into
    // [0, kb) on the low halo, [kb, ke) on own rows and [ke, len) on the high
    // halo; the padding repeats the last entry's column with value 0.
#pragma unroll
    for (int r = 0; r < R; ++r) {
        int b = slen(r), e = slen(r);
        if (band && val[r]) {
            for (int k = 0; k < slen(r); ++k) {
                T v;
                int j;
                entry(r, k, v, j);
                if (j >= own0 && j < own1) {
                    if (b == slen(r)) b = k;
                } else if (b < slen(r) && e == slen(r)) {
                    e = k;
                }
            }
            if (b == slen(r)) {  // no own entry: split at the first column past the own block
                for (b = 0; b < slen(r); ++b) {
                    T v;
                    int j;
                    entry(r, b, v, j);
                    if (j >= own1) break;
                }
                e = b;
            }
        }
        pk[r] |= (b << 10) | (e << 20);
    }
    // entries [k0, k1) of owned row r against the band (band path: values in
    // shared memory, offsets from parameter space or shared memory); brange.x
    // is a multiple of 64, so swz(j) - brange.x = swz(j - brange.x)
    auto band_sum = [&](int r, int k0, int k1, T& s0, T& s1, T& s2) {
        const int rb = rowof(r) - brange.x;
        const T* vp = sval + (gb[r] - eb);
        const int16_t* pp = (patParam ? a.patc : spat) + pid[r];
        // unrolled by 4: 1.3-1.8% faster than by 8 at 512x512 (2: +0.7%, 3 and 6 slower, 12 spills)
#pragma unroll 4
        for (int k = k0; k < k1; ++k) {
            const T v = vp[32 * k];
            const int q = swz(rb + (int)pp[k]);
            s0 += v * bx[q];
            s1 += v * by[q];
            s2 += v * bz[q];
        }
    };
    auto own_sum = [&](int r, T& s0, T& s1, T& s2) { band_sum(r, (pk[r] >> 10) & 1023, pk[r] >> 20, s0, s1, s2); };
    auto halo_part = [&](int r, T& s0, T& s1, T& s2) {
        band_sum(r, 0, (pk[r] >> 10) & 1023, s0, s1, s2);
        band_sum(r, pk[r] >> 20, slen(r), s0, s1, s2);
    };
    // the iterates in global memory: three planes of nslot floats on the band
    // path (the halo copies take one contiguous run per plane), 4-vectors
    // elsewhere (gathered per entry)
    auto st_it = [&](V4<T>* buf, int q, T x, T y, T z) {
        if constexpr (band) {
            T* p = reinterpret_cast<T*>(buf);
            __stcg(p + q, x);
            __stcg(p + a.nslot + q, y);
            __stcg(p + 2 * (size_t)a.nslot + q, z);
        } else {
            stcg4(buf, q, x, y, z);
        }
    };
    auto ld_it = [&](const V4<T>* buf, int q) -> V4<T> {
        if constexpr (band) {
            const T* p = reinterpret_cast<const T*>(buf);
            return V4<T>{__ldcg(p + q), __ldcg(p + a.nslot + q), __ldcg(p + 2 * (size_t)a.nslot + q), T(0)};
        } else {
            return ldcg4(buf, q);
        }
    };
    // sum_k N_ik src_k for the owned rows (paths without the band): matrix
    // from shared memory or L2, src gathered from global memory, in slot order
    // (iterates) or row order (slots == false: the positions)
    auto gather = [&](const V4<T>* src, bool slots, int r, T& s0, T& s1, T& s2) {
        s0 = T(0);
        s1 = T(0);
        s2 = T(0);
#pragma unroll 4
        for (int k = 0; k < slen(r); ++k) {
            T v;
            int j;
            entry(r, k, v, j);
            const V4<T> xj = ldv<kL1>(src, slots ? swz(j) : j);
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
            const int i = rowof(r);
            const int2 st = stencil_of(i, a.lPtr, a.tOff);
            T a0, a1, a2;
            if constexpr (kCorr) {
                const V4<T> h = ldv<kL1>(a.Ph, i), l = ldv<kL1>(a.Pl, i);
                a0 = a1 = a2 = T(0);
                for (int k = 0; k < st.y; ++k) {
                    const int s = st.x + kSlice * k;
                    const int j = __ldg(a.tNbr + s);
                    const V4<T> hj = ldv<kL1>(a.Ph, j), lj = ldv<kL1>(a.Pl, j);
                    const T wl = __ldg(a.tLbo + s);
                    a0 += wl * diff_ff(hj.x, lj.x, h.x, l.x);
                    a1 += wl * diff_ff(hj.y, lj.y, h.y, l.y);
                    a2 += wl * diff_ff(hj.z, lj.z, h.z, l.z);
                }
            } else {
                const V4<S> x = ldv<kL1>(a.P, i);
                const T l0 = __ldg(a.tLbo0 + i);
                a0 = x.x * l0;
                a1 = x.y * l0;
                a2 = x.z * l0;
                for (int k = 0; k < st.y; ++k) {
                    const int s = st.x + kSlice * k;
                    const V4<T> xj = ldv<kL1>(a.P, __ldg(a.tNbr + s));
                    const T l = __ldg(a.tLbo + s);
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
        // ---- tet strain projections of the tets this CTA owns ----
        if constexpr (kTets)
            for (int q = a.ctaTetPtr[cta] + (int)threadIdx.x; q < a.ctaTetPtr[cta + 1]; q += (int)blockDim.x)
                tet_project_one<S, kCorr>(a.ctaTetIdx[q], a.Tets, a.TetIdm, a.TetW, a.P, a.Ph, a.Pl, a.TetOut);
        if (!sync()) return;

        // ---- right-hand side (direct) or residual (correction) of the owned rows ----
        // row i, whose SELL entries start at gbi (leni of them, pattern pidi):
        // its right-hand side (direct form, with its positions in xx) or its
        // residual (correction form) in rr
        auto rhs_row = [&](int i, int gbi, int leni, int pidi, T (&rr)[3], T (&xx)[3]) {
            xx[0] = xx[1] = xx[2] = T(0);
            const int2 st = stencil_of(i, a.lPtr, a.tOff);
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
                for (int k = 0; k < st.y; ++k) {
                    const int s = st.x + kSlice * k;
                    const int j = __ldg(a.tNbr + s);
                    const V4<T> hj = ldv<kL1>(a.Ph, j), lj = ldv<kL1>(a.Pl, j);
                    const T d0 = diff_ff(h.x, l.x, hj.x, lj.x), d1 = diff_ff(h.y, l.y, hj.y, lj.y),
                            d2 = diff_ff(h.z, l.z, hj.z, lj.z);
                    const T cl = sqrtf(d0 * d0 + d1 * d1 + d2 * d2);
                    const T rc = strain * (__ldg(a.tRest + s) / cl);
                    r0.add(rc * d0);
                    r1.add(rc * d1);
                    r2.add(rc * d2);
                }
                const V4<T> ai = ldv<kL1>(a.Aq, i);
                const T b0 = __ldg(a.tBend0 + i);
                r0.add(b0 * ai.x);
                r1.add(b0 * ai.y);
                r2.add(b0 * ai.z);
                for (int k = 0; k < st.y; ++k) {
                    const int s = st.x + kSlice * k;
                    const V4<T> ak = ldv<kL1>(a.Aq, __ldg(a.tNbr + s));
                    const T bt = __ldg(a.tBendT + s);
                    r0.add(bt * ak.x);
                    r1.add(bt * ak.y);
                    r2.add(bt * ak.z);
                }
                if constexpr (kTets) {
                    for (int q = a.vtPtr[i]; q < a.vtPtr[i + 1]; ++q) {  // tet projections w R G, ascending tet
                        const V4<T> t = ldcg4(a.TetOut, a.vtIdx[q]);
                        r0.add(t.x);
                        r1.add(t.y);
                        r2.add(t.z);
                    }
                }
                // unrolled by 4 so that the entries' gathers overlap (1.3% faster at
                // 512x512); the sums stay in entry order
#pragma unroll 4
                for (int k = 0; k < leni; ++k) {
                    T v;
                    int j;
                    entry_at(gbi, pidi, i, k, v, j);
                    const V4<T> hj = ldv<kL1>(a.Ph, j), lj = ldv<kL1>(a.Pl, j);
                    r0.add(v * diff_ff(hj.x, lj.x, h.x, l.x));
                    r1.add(v * diff_ff(hj.y, lj.y, h.y, l.y));
                    r2.add(v * diff_ff(hj.z, lj.z, h.z, l.z));
                }
                rr[0] = r0.value();
                rr[1] = r1.value();
                rr[2] = r2.value();
            } else {
                xx[0] = x.x;
                xx[1] = x.y;
                xx[2] = x.z;
                T t0 = T(0), t1 = T(0), t2 = T(0);
                for (int k = 0; k < st.y; ++k) {
                    const int s = st.x + kSlice * k;
                    const V4<T> xj = ldv<kL1>(a.P, __ldg(a.tNbr + s));
                    const T d0 = x.x - xj.x, d1 = x.y - xj.y, d2 = x.z - xj.z;
                    const T cl = sqrtf(d0 * d0 + d1 * d1 + d2 * d2);
                    const T rc = strain * (__ldg(a.tRest + s) / cl);
                    t0 += rc * d0;
                    t1 += rc * d1;
                    t2 += rc * d2;
                }
                const V4<T> ai = ldv<kL1>(a.Aq, i);
                const T b0 = __ldg(a.tBend0 + i);
                t0 += b0 * ai.x;
                t1 += b0 * ai.y;
                t2 += b0 * ai.z;
                const V4<T> q0 = ldcg4(a.Rhs0, i);
                T u0 = q0.x + t0, u1 = q0.y + t1, u2 = q0.z + t2;
                for (int k = 0; k < st.y; ++k) {
                    const int s = st.x + kSlice * k;
                    const V4<T> ak = ldv<kL1>(a.Aq, __ldg(a.tNbr + s));
                    const T bt = __ldg(a.tBendT + s);
                    u0 += bt * ak.x;
                    u1 += bt * ak.y;
                    u2 += bt * ak.z;
                }
                if constexpr (kTets) {
                    for (int q = a.vtPtr[i]; q < a.vtPtr[i + 1]; ++q) {  // tet projections, ascending tet
                        const V4<T> t = ldcg4(a.TetOut, a.vtIdx[q]);
                        u0 += t.x;
                        u1 += t.y;
                        u2 += t.z;
                    }
                }
                const V4<T> cr = ldcg4(a.CollRhs, i);
                u0 += cr.x;
                u1 += cr.y;
                u2 += cr.z;
                const V4<T> pn = ldcg4(a.PinRhs, i);
                u0 += pn.x;
                u1 += pn.y;
                u2 += pn.z;
                rr[0] = u0;
                rr[1] = u1;
                rr[2] = u2;
            }
        };
        T x0[R][3], rh[R][3];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            x0[r][0] = x0[r][1] = x0[r][2] = T(0);
            rh[r][0] = rh[r][1] = rh[r][2] = T(0);
            if (val[r]) rhs_row(rowof(r), gb[r], slen(r), pid[r], rh[r], x0[r]);
        }

        // ---- Chebyshev-accelerated R2 iteration as two J sweeps per step ----
        // direct form: iterate on x from x0 (gathered from P);
        // correction form: iterate on delta from 0, add it to P at the end.
        // first sweep of a step: y = S(c) from the gathered sum s and the row's own c
        auto finish_y = [&](int r, T s0, T s1, T s2, const T (&c)[3], T (&y)[3]) {
            y[0] = om1 * c[0] + w * ((s0 + rh[r][0]) * id[r]);
            y[1] = om1 * c[1] + w * ((s1 + rh[r][1]) * id[r]);
            y[2] = om1 * c[2] + w * ((s2 + rh[r][2]) * id[r]);
            if (val[r]) st_it(a.GY, itof(r), y[0], y[1], y[2]);
        };
        // second sweep of step it: S(y), Chebyshev-combined with the previous
        // second-sweep iterate p except for the first step; the last one
        // updates the positions
        auto finish_x = [&](int r, T s0, T s1, T s2, const T (&y)[3], const T (&p)[3], int it, bool last,
                            V4<T>* xout, T (&n)[3]) {
            const T om = a.omega[it];
            n[0] = om1 * y[0] + w * ((s0 + rh[r][0]) * id[r]);
            n[1] = om1 * y[1] + w * ((s1 + rh[r][1]) * id[r]);
            n[2] = om1 * y[2] + w * ((s2 + rh[r][2]) * id[r]);
            if (it > 0) {
                n[0] = om * (n[0] - p[0]) + p[0];
                n[1] = om * (n[1] - p[1]) + p[1];
                n[2] = om * (n[2] - p[2]) + p[2];
            }
            if (!val[r]) return;
            if (last) {
                if constexpr (kCorr) {  // only this thread writes the row: its own earlier read is current
                    const V4<S> x = ldcg4(a.P, rowof(r));
                    const S q0 = x.x + (S)n[0], q1 = x.y + (S)n[1], q2 = x.z + (S)n[2];
                    stcg4(a.P, rowof(r), q0, q1, q2);
                    float h0, l0, h1, l1, h2, l2;
                    split_ff(q0, h0, l0);
                    split_ff(q1, h1, l1);
                    split_ff(q2, h2, l2);
                    stcg4(a.Ph, rowof(r), h0, h1, h2);
                    stcg4(a.Pl, rowof(r), l0, l1, l2);
                } else {
                    stcg4(a.P, rowof(r), n[0], n[1], n[2]);
                }
            } else {
                st_it(xout, itof(r), n[0], n[1], n[2]);
            }
        };
        const int nsteps = a.cheby;
        if constexpr (band) {
            // The own slots always hold the latest iterate of the own rows, so a
            // row keeps only its right-hand side and partial sums in registers:
            // y and the current x come from its slot.  Second-sweep iterates
            // alternate between GX (even steps) and GX2 (odd steps), so the one
            // from two steps back that the Chebyshev combination needs is still
            // in the buffer the row overwrites (this thread's rows only); GX2
            // starts as x0 = 0.  A sweep sums a row's entries on own rows while
            // the halo is in flight, then the halo entries (correction form
            // only: the direct form keeps the reference's summation order).
            T so[R][3], nv[R][3];
            auto own_part = [&]() {
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    so[r][0] = so[r][1] = so[r][2] = T(0);
                    if (val[r]) own_sum(r, so[r][0], so[r][1], so[r][2]);
                }
            };
            auto own_slot = [&](int r, T (&c)[3]) {
                const int q = val[r] ? itof(r) - brange.x : 0;
                c[0] = bx[q];
                c[1] = by[q];
                c[2] = bz[q];
            };
            auto write_own = [&]() {
#pragma unroll
                for (int r = 0; r < R; ++r)
                    if (val[r]) {
                        const int q = itof(r) - brange.x;
                        bx[q] = nv[r][0];
                        by[q] = nv[r][1];
                        bz[q] = nv[r][2];
                    }
            };
            // end of a sweep: every row's global stores are issued and nobody
            // reads the band; the sync warp publishes the phase while the
            // compute warps move their new iterate into the own slots
            auto end_sweep = [&]() {
                __syncthreads();
                ++epoch;
                if (syncw) {
                    // release after the CTA barrier: cumulative over every
                    // thread's stores of the sweep (as in nbr_publish)
                    if (lane == 0) st_release_gpu(a.flags + cta, epoch);
                } else {
                    write_own();
                    comp_bar();
                }
            };
            // sums of a sweep for the owned rows (compute warps); false: the launch ends
            static_assert(kCorr || !band, "the band path runs the correction form");
            auto sweep_sums = [&](T (&sm)[R][3]) -> bool {
                own_part();
                if (!halo_ready()) return false;
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    sm[r][0] = so[r][0];
                    sm[r][1] = so[r][1];
                    sm[r][2] = so[r][2];
                    if (val[r]) halo_part(r, sm[r][0], sm[r][1], sm[r][2]);
                }
                return true;
            };
            // first sweep: y = S(0)
            if (!syncw) {
                const T zero[3] = {T(0), T(0), T(0)};
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    if (val[r]) st_it(a.GX2, itof(r), T(0), T(0), T(0));
                    finish_y(r, T(0), T(0), T(0), zero, nv[r]);
                }
            }
            end_sweep();
            for (int it = 0; it < nsteps; ++it) {
                const bool last = it == nsteps - 1;
                V4<T>* xb = (it & 1) ? a.GX2 : a.GX;
                // x = S(y)
                if (syncw) {
                    if (!issue_halo(a.GY, true)) return;
                } else {
                    T p[R][3], sm[R][3];
#pragma unroll
                    for (int r = 0; r < R; ++r) {
                        p[r][0] = p[r][1] = p[r][2] = T(0);
                        if (it > 0 && val[r]) {
                            const V4<T> g = ld_it(xb, itof(r));
                            p[r][0] = g.x;
                            p[r][1] = g.y;
                            p[r][2] = g.z;
                        }
                    }
                    if (!sweep_sums(sm)) return;
#pragma unroll
                    for (int r = 0; r < R; ++r) {
                        T y[3];
                        own_slot(r, y);
                        finish_x(r, sm[r][0], sm[r][1], sm[r][2], y, p[r], it, last, xb, nv[r]);
                    }
                }
                end_sweep();
                if (last) break;
                // y = S(x)
                if (syncw) {
                    if (!issue_halo(xb, true)) return;
                } else {
                    T sm[R][3];
                    if (!sweep_sums(sm)) return;
#pragma unroll
                    for (int r = 0; r < R; ++r) {
                        T c[3];
                        own_slot(r, c);
                        finish_y(r, sm[r][0], sm[r][1], sm[r][2], c, nv[r]);
                    }
                }
                end_sweep();
            }
            // the next phase reads the neighbours' positions
            if (!nbr_wait(a.flags, a.err, cta, nrange, epoch, a.timeout)) return;
        } else {
            T cx[R][3], px[R][3], yv[R][3];
#pragma unroll
            for (int r = 0; r < R; ++r) {
                T s0 = T(0), s1 = T(0), s2 = T(0);
                if constexpr (kCorr) {
                    cx[r][0] = cx[r][1] = cx[r][2] = T(0);
                } else {
                    cx[r][0] = x0[r][0];
                    cx[r][1] = x0[r][1];
                    cx[r][2] = x0[r][2];
                    if (val[r]) gather(a.P, false, r, s0, s1, s2);
                }
                finish_y(r, s0, s1, s2, cx[r], yv[r]);
            }
            if (!sync()) return;
            for (int it = 0; it < nsteps; ++it) {
                const bool last = it == nsteps - 1;
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    T s0 = T(0), s1 = T(0), s2 = T(0), n[3];
                    if (val[r]) gather(a.GY, true, r, s0, s1, s2);
                    finish_x(r, s0, s1, s2, yv[r], px[r], it, last, a.GX, n);
                    px[r][0] = cx[r][0];
                    px[r][1] = cx[r][1];
                    px[r][2] = cx[r][2];
                    cx[r][0] = n[0];
                    cx[r][1] = n[1];
                    cx[r][2] = n[2];
                }
                if (!sync()) return;
                if (last) break;
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    T s0 = T(0), s1 = T(0), s2 = T(0);
                    if (val[r]) gather(a.GX, true, r, s0, s1, s2);
                    finish_y(r, s0, s1, s2, cx[r], yv[r]);
                }
                if (!sync()) return;
            }
        }
    }
}

template <typename T, bool kCorr, int kMode, bool kL1>
const void* kernel_for(int R) {
    using S = typename std::conditional<kCorr, double, T>::type;
    switch (R) {
        case 1: return (const void*)k_pd_persistent<T, S, kCorr, kMode, kL1, 1>;
        case 2: return (const void*)k_pd_persistent<T, S, kCorr, kMode, kL1, 2>;
        case 3: return (const void*)k_pd_persistent<T, S, kCorr, kMode, kL1, 3>;
        default: return (const void*)k_pd_persistent<T, S, kCorr, kMode, kL1, 4>;
    }
}
// with tets: gathers through L1, one or two rows per thread
template <typename T, bool kCorr, int kMode>
const void* kernel_for_tets(int R) {
    using S = typename std::conditional<kCorr, double, T>::type;
    return R == 1 ? (const void*)k_pd_persistent<T, S, kCorr, kMode | 4, true, 1>
                  : (const void*)k_pd_persistent<T, S, kCorr, kMode | 4, true, 2>;
}

}  // namespace
}  // namespace pdipc
