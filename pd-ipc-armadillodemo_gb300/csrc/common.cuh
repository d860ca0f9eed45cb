// common.cuh — types and small device helpers shared by the PD-IPC kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>

namespace pdipc {

// Position-like quantities are stored one vertex per aligned 4-vector
// (x, y, z, pad) so a gather is one 16-byte (float) or two 16-byte (double)
// loads instead of the reference's three scalar loads (PdIpcGpuFunc.cu:660-662).
template <typename T>
struct alignas(4 * sizeof(T) > 16 ? 16 : 4 * sizeof(T)) V4 {
    T x, y, z, w;
};

template <typename T>
struct Box6 {  // AABB: min xyz, max xyz
    T lo[3];
    T hi[3];
};

constexpr int kWarp = 32;
constexpr int kSlice = 32;  // rows per SELL slice (one warp)

template <typename T>
__device__ __forceinline__ V4<T> ld4(const V4<T>* p, int i) {
    return p[i];
}
__device__ __forceinline__ V4<float> ld4(const V4<float>* p, int i) {
    float4 v = __ldg(reinterpret_cast<const float4*>(p) + i);
    return V4<float>{v.x, v.y, v.z, v.w};
}
__device__ __forceinline__ V4<double> ld4(const V4<double>* p, int i) {
    const double2* q = reinterpret_cast<const double2*>(p) + 2 * (size_t)i;
    double2 a = __ldg(q), b = __ldg(q + 1);
    return V4<double>{a.x, a.y, b.x, b.y};
}
// Plain (coherent) load for buffers written earlier in the same kernel or by
// other blocks of a cooperative launch.
template <typename T>
__device__ __forceinline__ V4<T> ld4c(const V4<T>* p, int i) {
    return p[i];
}

template <typename T>
__device__ __forceinline__ void st4(V4<T>* p, int i, T x, T y, T z) {
    p[i] = V4<T>{x, y, z, T(0)};
}

template <typename T>
__device__ __forceinline__ T dsqrt(T v) {
    return sqrt(v);
}
template <>
__device__ __forceinline__ float dsqrt<float>(float v) {
    return sqrtf(v);
}
template <typename T>
__device__ __forceinline__ T dlog(T v) {
    return log(v);
}
template <>
__device__ __forceinline__ float dlog<float>(float v) {
    return logf(v);
}
template <typename T>
__device__ __forceinline__ T dmin(T a, T b) {
    return fmin(a, b);
}
template <>
__device__ __forceinline__ float dmin<float>(float a, float b) {
    return fminf(a, b);
}
template <typename T>
__device__ __forceinline__ T dmax(T a, T b) {
    return fmax(a, b);
}
template <>
__device__ __forceinline__ float dmax<float>(float a, float b) {
    return fmaxf(a, b);
}

// Order-preserving integer image of a non-negative float/double, so a global
// minimum over non-negative values is one integer atomicMin.
__device__ __forceinline__ unsigned int ordered_bits(float v) { return __float_as_uint(v); }
__device__ __forceinline__ unsigned long long ordered_bits(double v) {
    return (unsigned long long)__double_as_longlong(v);
}

template <typename T>
__device__ __forceinline__ void atomic_min_nonneg(T* addr, T v);
template <>
__device__ __forceinline__ void atomic_min_nonneg<float>(float* addr, float v) {
    atomicMin(reinterpret_cast<unsigned int*>(addr), __float_as_uint(v));
}
template <>
__device__ __forceinline__ void atomic_min_nonneg<double>(double* addr, double v) {
    atomicMin(reinterpret_cast<unsigned long long*>(addr), (unsigned long long)__double_as_longlong(v));
}

template <typename T>
__device__ __forceinline__ T warp_min(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = dmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
template <typename T>
__device__ __forceinline__ T warp_max(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = dmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Compensated FP32 sum (Knuth's TwoSum): s + c carries the exact sum of the
// added terms to about twice FP32 precision, at six FP32 adds per term.
struct Sum2 {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float x) {
        const float t = s + x;
        const float bp = t - s;
        c += (s - (t - bp)) + (x - bp);
        s = t;
    }
    __device__ __forceinline__ float value() const { return s + c; }
};

// Float-float split of a double (Dekker): hi = rn(x), lo = rn(x - hi), so hi + lo
// carries x to about 2^-48 relative.  The mixed form mirrors its FP64 positions
// this way so the hot loops form position differences in FP32 only:
// (hi_j - hi_i) + (lo_j - lo_i) is the difference rounded about once to FP32
// (the hi difference of nearby values is exact by Sterbenz's lemma).  GB300's
// FP64 rate is a small fraction of its FP32 rate, so FP64 arithmetic stays out
// of the per-neighbour loops.
__device__ __forceinline__ void split_ff(double x, float& hi, float& lo) {
    hi = __double2float_rn(x);
    lo = __double2float_rn(x - (double)hi);
}
__device__ __forceinline__ float diff_ff(float hj, float lj, float hi, float li) { return (hj - hi) + (lj - li); }

// Device-side error flags (bit mask), read back by the host after a step.
enum ErrFlag : unsigned int {
    kErrNonFinite = 1u,
    kErrTraversal = 2u,
    kErrPairOverflow = 4u,
    kErrCandidateOverflow = 8u,
    kErrBarrier = 16u,  // a grid barrier of the persistent solve timed out
    kErrSort = 32u,     // a look-back wait of the radix sort timed out
};

// Stopping test of the outer loop, made on the device.  k_outer_gate writes it
// after each outer iteration's contact pass; every kernel launched by a later
// outer iteration of the step (and the iteration's own copy of the positions
// into Pold) reads `stop` at entry and returns without work once it is set.
// That lets the host enqueue outer iteration k+1 before it has read
// iteration k's residual.
struct OuterGate {
    unsigned stop;             // the stopping rule held at an earlier outer iteration
    int iters;                 // outer iterations run so far in this step
    double resid;              // |dir|^2 of the last iteration run
    double toi;                // its clamped step fraction
    unsigned long long active; // its active contact constraints
};
__device__ __forceinline__ bool outer_stopped(const OuterGate* g) { return g && g->stop; }

}  // namespace pdipc
