// primitives.cu — scan, radix sort and reductions used by the broad phase.
//
// They replace the reference's thrust::exclusive_scan + device_vector element
// reads (PdIpcGpuFunc.cu:1791-1792, 1989-1990) and the CPU std::sort of the
// Morton codes (AipcBvhs.cpp:185-189).  All are deterministic.
#include <algorithm>

#include "kernels.cuh"

namespace pdipc {

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

template <typename I>
__device__ __forceinline__ I warp_incl_scan(I v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        I n = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += n;
    }
    return v;
}

// Exclusive scan of one tile; tile total to sums[blockIdx] (or *total when
// the whole input is one tile).
template <typename I>
__global__ void __launch_bounds__(kScanThreads) k_scan_tile(const I* __restrict__ in, I* __restrict__ out, int64_t n,
                                                            I* __restrict__ sums, I* __restrict__ total) {
    __shared__ I warp_tot[kScanThreads / 32];
    const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    I v[kScanItems];
    I acc = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const int64_t i = base + k;
        v[k] = i < n ? in[i] : I(0);
        acc += v[k];
    }
    const I incl = warp_incl_scan(acc);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 31) warp_tot[w] = incl;
    __syncthreads();
    if (w == 0) {
        I t = lane < kScanThreads / 32 ? warp_tot[lane] : I(0);
        t = warp_incl_scan(t);
        if (lane < kScanThreads / 32) warp_tot[lane] = t;
    }
    __syncthreads();
    I run = (w > 0 ? warp_tot[w - 1] : I(0)) + incl - acc;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const int64_t i = base + k;
        if (i < n) out[i] = run;
        run += v[k];
    }
    if (threadIdx.x == kScanThreads - 1) {
        const I tot = warp_tot[kScanThreads / 32 - 1];
        if (sums) sums[blockIdx.x] = tot;
        if (total) *total = tot;
    }
}

template <typename I>
__global__ void k_scan_add(I* __restrict__ out, int64_t n, const I* __restrict__ sums) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += sums[i / kScanTile];
}

int64_t ntiles(int64_t n) { return (n + kScanTile - 1) / kScanTile; }

template <typename I>
size_t scan_tmp_elems(int64_t n) {
    size_t e = 0;
    while (n > kScanTile) {
        n = ntiles(n);
        e += (size_t)n;
    }
    return e;
}

template <typename I>
void scan_rec(const I* in, I* out, int64_t n, I* total, I* tmp, cudaStream_t s) {
    if (n <= 0) {
        if (total) cudaMemsetAsync(total, 0, sizeof(I), s);
        return;
    }
    const int64_t nt = ntiles(n);
    if (nt == 1) {
        k_scan_tile<I><<<1, kScanThreads, 0, s>>>(in, out, n, nullptr, total);
        return;
    }
    I* sums = tmp;
    k_scan_tile<I><<<(unsigned)nt, kScanThreads, 0, s>>>(in, out, n, sums, nullptr);
    scan_rec<I>(sums, sums, nt, total, tmp + nt, s);
    k_scan_add<I><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(out, n, sums);
}

// ---------------- onesweep radix sort (64-bit keys, 8 digits of 8 bits) ----------------
// One read of the keys builds all eight digit histograms; then each digit
// pass is one kernel.  A CTA takes the next partition of 2048 keys by an
// atomic ticket (so partitions start in order), ranks its keys stably (rounds
// in index order, warps by __match_any_sync), publishes its per-digit counts,
// and looks back through the earlier partitions' published values for its
// exclusive prefix (decoupled look-back: an earlier partition publishes its
// aggregate before it looks back itself, so the chain always advances), then
// scatters.  Waits are bounded: past the limit the pass records kErrSort.
constexpr int kOsThreads = 256;
constexpr int kOsRounds = 8;
constexpr int kOsTile = kOsThreads * kOsRounds;
constexpr unsigned kOsAggregate = 1u << 30, kOsPrefix = 2u << 30, kOsValue = (1u << 30) - 1u;
constexpr long long kOsMaxSpins = 1ll << 22;

__device__ __forceinline__ unsigned os_ld_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void os_st_release(unsigned* p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__global__ void __launch_bounds__(kOsThreads) k_os_hist(const unsigned long long* __restrict__ keys, int n,
                                                        unsigned* __restrict__ hist) {
    __shared__ unsigned h[8][256];
    for (int i = threadIdx.x; i < 8 * 256; i += blockDim.x) (&h[0][0])[i] = 0u;
    __syncthreads();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const unsigned long long k = keys[i];
#pragma unroll
        for (int p = 0; p < 8; ++p) atomicAdd(&h[p][(k >> (8 * p)) & 0xffull], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 8 * 256; i += blockDim.x) {
        const unsigned c = (&h[0][0])[i];
        if (c) atomicAdd(hist + i, c);
    }
}

// exclusive scan of each pass's 256 digit counts: block p, thread d
__global__ void __launch_bounds__(256) k_os_offsets(const unsigned* __restrict__ hist, unsigned* __restrict__ off) {
    __shared__ unsigned s[256];
    const int p = blockIdx.x, d = threadIdx.x;
    const unsigned own = hist[p * 256 + d];
    s[d] = own;
    __syncthreads();
    for (int o = 1; o < 256; o <<= 1) {  // inclusive Hillis-Steele scan
        const unsigned v = d >= o ? s[d - o] : 0u;
        __syncthreads();
        s[d] += v;
        __syncthreads();
    }
    off[p * 256 + d] = s[d] - own;
}

__global__ void __launch_bounds__(kOsThreads) k_onesweep(const unsigned long long* __restrict__ kin,
                                                         const int* __restrict__ vin,
                                                         unsigned long long* __restrict__ kout,
                                                         int* __restrict__ vout, int n, int shift,
                                                         const unsigned* __restrict__ digitOff,
                                                         unsigned* __restrict__ status, unsigned* __restrict__ ticket,
                                                         unsigned* __restrict__ err) {
    __shared__ int part_s;
    __shared__ unsigned cnt[256];
    __shared__ unsigned wcnt[kOsThreads / 32][256];
    __shared__ unsigned base_s[256];
    const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
    if (tid == 0) part_s = (int)atomicAdd(ticket, 1u);
    cnt[tid] = 0u;
    __syncthreads();
    const int part = part_s;
    const int tile = part * kOsTile;
    const unsigned lt = (1u << lane) - 1u;
    unsigned long long key[kOsRounds];
    int val[kOsRounds], dig[kOsRounds];
    unsigned rank[kOsRounds];
#pragma unroll
    for (int r = 0; r < kOsRounds; ++r) {
        const int i = tile + r * kOsThreads + tid;
        const bool ok = i < n;
        key[r] = ok ? kin[i] : 0ull;
        val[r] = ok ? vin[i] : 0;
        dig[r] = ok ? (int)((key[r] >> shift) & 0xffull) : 256 + lane;  // past the end: no peers
        const unsigned peers = __match_any_sync(0xffffffffu, dig[r]);
        for (int j = lane; j < 256; j += 32) wcnt[w][j] = 0u;
        __syncwarp();
        if (ok && __popc(peers & lt) == 0) wcnt[w][dig[r]] = (unsigned)__popc(peers);
        __syncthreads();
        // thread tid owns digit tid: exclusive prefix over the warps of this round,
        // on top of the tile's count so far
        unsigned run = cnt[tid];
#pragma unroll
        for (int ww = 0; ww < kOsThreads / 32; ++ww) {
            const unsigned c = wcnt[ww][tid];
            wcnt[ww][tid] = run;
            run += c;
        }
        __syncthreads();
        rank[r] = ok ? wcnt[w][dig[r]] + (unsigned)__popc(peers & lt) : 0u;
        __syncthreads();
        cnt[tid] = run;
        __syncthreads();
    }
    // publish this partition's count of digit tid, look back for the prefix
    const unsigned local = cnt[tid];
    unsigned* st = status + (size_t)part * 256 + tid;
    unsigned before = 0u;
    if (part == 0) {
        os_st_release(st, kOsPrefix | local);
    } else {
        os_st_release(st, kOsAggregate | local);
        long long spins = 0;
        for (int j = part - 1; j >= 0;) {
            const unsigned s = os_ld_acquire(status + (size_t)j * 256 + tid);
            const unsigned f = s & ~kOsValue;
            if (f == 0u) {
                if (++spins > kOsMaxSpins) {
                    atomicOr(err, (unsigned)kErrSort);
                    break;
                }
                __nanosleep(32);
                continue;
            }
            before += s & kOsValue;
            if (f == kOsPrefix) break;
            --j;
        }
        os_st_release(st, kOsPrefix | (before + local));
    }
    base_s[tid] = digitOff[tid] + before;
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kOsRounds; ++r) {
        if (tile + r * kOsThreads + tid < n) {
            const unsigned pos = base_s[dig[r]] + rank[r];
            kout[pos] = key[r];
            vout[pos] = val[r];
        }
    }
}

__global__ void k_reduce_sum(const double* __restrict__ p, int n, double* __restrict__ out) {
    __shared__ double red[32];
    double acc = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) acc += p[i];
    acc = warp_sum(acc);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = threadIdx.x < (int)(blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
        v = warp_sum(v);
        if (threadIdx.x == 0) *out = v;
    }
}

}  // namespace

size_t scan_tmp_bytes(int64_t n) { return (scan_tmp_elems<int64_t>(n) + 2) * sizeof(int64_t); }

void scan_exclusive_i64(const int64_t* in, int64_t* out, int64_t n, int64_t* total, void* tmp, cudaStream_t s) {
    scan_rec<int64_t>(in, out, n, total, static_cast<int64_t*>(tmp), s);
}
void scan_exclusive_i32(const int* in, int* out, int n, int* total, void* tmp, cudaStream_t s) {
    scan_rec<int>(in, out, n, total, static_cast<int*>(tmp), s);
}

// scratch: alternate keys and values, then (256-aligned) the histograms and
// offsets of the 8 passes, the 8 passes' look-back status words and tickets
size_t sort_tmp_bytes(int n) {
    const size_t parts = (size_t)std::max(1, (n + kOsTile - 1) / kOsTile);
    size_t b = (size_t)n * (sizeof(unsigned long long) + sizeof(int));
    b = (b + 255) & ~(size_t)255;
    b += (2 * 8 * 256 + 8 * parts * 256 + 8) * sizeof(unsigned);
    return b + 256;
}

void radix_sort_u64(unsigned long long* keys, int* vals, int n, void* tmp, unsigned* err, cudaStream_t s) {
    if (n <= 1) return;
    const int parts = (n + kOsTile - 1) / kOsTile;
    char* t = static_cast<char*>(tmp);
    auto* k2 = reinterpret_cast<unsigned long long*>(t);
    t += (size_t)n * sizeof(unsigned long long);
    auto* v2 = reinterpret_cast<int*>(t);
    t += (size_t)n * sizeof(int);
    t = reinterpret_cast<char*>(((uintptr_t)t + 255) & ~(uintptr_t)255);
    unsigned* hist = reinterpret_cast<unsigned*>(t);
    unsigned* off = hist + 8 * 256;
    unsigned* status = off + 8 * 256;
    unsigned* tickets = status + (size_t)8 * parts * 256;
    cudaMemsetAsync(hist, 0, (2 * 8 * 256 + (size_t)8 * parts * 256 + 8) * sizeof(unsigned), s);
    k_os_hist<<<std::min(parts, 152 * 4), kOsThreads, 0, s>>>(keys, n, hist);
    k_os_offsets<<<8, 256, 0, s>>>(hist, off);
    unsigned long long *ka = keys, *kb = k2;
    int *va = vals, *vb = v2;
    for (int pass = 0; pass < 8; ++pass) {
        k_onesweep<<<parts, kOsThreads, 0, s>>>(ka, va, kb, vb, n, 8 * pass, off + 256 * pass,
                                               status + (size_t)pass * parts * 256, tickets + pass, err);
        std::swap(ka, kb);
        std::swap(va, vb);
    }
    // eight passes: the result is back in keys/vals
}

void launch_reduce_sum_f64(const double* part, int n, double* out, cudaStream_t s) {
    k_reduce_sum<<<1, 1024, 0, s>>>(part, n, out);
}

}  // namespace pdipc
