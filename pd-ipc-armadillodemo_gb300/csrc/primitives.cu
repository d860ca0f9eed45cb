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

// ---------------- radix sort ----------------
constexpr int kSortTile = 4096;
constexpr int kSortThreads = 256;

__global__ void k_hist(const unsigned long long* __restrict__ keys, int n, int shift, int nblk,
                       int* __restrict__ hist) {
    __shared__ int h[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) h[i] = 0;
    __syncthreads();
    const int base = blockIdx.x * kSortTile;
    for (int i = threadIdx.x; i < kSortTile; i += blockDim.x) {
        const int g = base + i;
        if (g < n) atomicAdd(&h[(keys[g] >> shift) & 0xff], 1);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 256; i += blockDim.x) hist[i * nblk + blockIdx.x] = h[i];
}

// One warp per tile, in order, so equal digits keep their input order.
__global__ void k_scatter(const unsigned long long* __restrict__ kin, const int* __restrict__ vin,
                          unsigned long long* __restrict__ kout, int* __restrict__ vout, int n, int shift, int nblk,
                          const int* __restrict__ off) {
    __shared__ int cnt[256];
    const int lane = threadIdx.x;
    for (int i = lane; i < 256; i += 32) cnt[i] = off[i * nblk + blockIdx.x];
    __syncwarp();
    const int base = blockIdx.x * kSortTile;
    const unsigned lt = (1u << lane) - 1u;
    for (int c = 0; c < kSortTile; c += 32) {
        const int g = base + c + lane;
        const bool ok = g < n;
        unsigned long long k = ok ? kin[g] : 0ull;
        const int v = ok ? vin[g] : 0;
        const int d = ok ? (int)((k >> shift) & 0xff) : 256 + lane;
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const int rank = __popc(peers & lt);
        int pos = 0;
        if (ok) pos = cnt[d] + rank;
        __syncwarp();
        if (ok) {
            kout[pos] = k;
            vout[pos] = v;
            if (rank == 0) cnt[d] += __popc(peers);
        }
        __syncwarp();
        if (base + c + 32 >= n) break;
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

size_t sort_tmp_bytes(int n) {
    const int nblk = std::max(1, (n + kSortTile - 1) / kSortTile);
    size_t b = 0;
    b += (size_t)n * sizeof(unsigned long long);        // alternate keys
    b += (size_t)n * sizeof(int);                       // alternate values
    b = (b + 255) & ~(size_t)255;
    b += (size_t)256 * nblk * sizeof(int);              // histograms / offsets
    b = (b + 255) & ~(size_t)255;
    b += scan_tmp_bytes((int64_t)256 * nblk);
    return b + 256;
}

void radix_sort_u64(unsigned long long* keys, int* vals, int n, void* tmp, cudaStream_t s) {
    if (n <= 1) return;
    const int nblk = (n + kSortTile - 1) / kSortTile;
    char* t = static_cast<char*>(tmp);
    auto* k2 = reinterpret_cast<unsigned long long*>(t);
    t += (size_t)n * sizeof(unsigned long long);
    auto* v2 = reinterpret_cast<int*>(t);
    t += (size_t)n * sizeof(int);
    t = reinterpret_cast<char*>(((uintptr_t)t + 255) & ~(uintptr_t)255);
    int* hist = reinterpret_cast<int*>(t);
    t += (size_t)256 * nblk * sizeof(int);
    t = reinterpret_cast<char*>(((uintptr_t)t + 255) & ~(uintptr_t)255);
    void* stmp = t;
    unsigned long long *ka = keys, *kb = k2;
    int *va = vals, *vb = v2;
    for (int pass = 0; pass < 8; ++pass) {
        const int shift = 8 * pass;
        k_hist<<<nblk, kSortThreads, 0, s>>>(ka, n, shift, nblk, hist);
        scan_exclusive_i32(hist, hist, 256 * nblk, nullptr, stmp, s);
        k_scatter<<<nblk, 32, 0, s>>>(ka, va, kb, vb, n, shift, nblk, hist);
        std::swap(ka, kb);
        std::swap(va, vb);
    }
    // eight passes: the result is back in keys/vals
}

void launch_reduce_sum_f64(const double* part, int n, double* out, cudaStream_t s) {
    k_reduce_sum<<<1, 1024, 0, s>>>(part, n, out);
}

}  // namespace pdipc
