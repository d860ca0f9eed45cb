/*
 * cuda_emu.h — runs CUDA C kernel source on the host, for the oracle's
 * reference-kernel build only (test infrastructure; nothing in the library
 * uses it).
 *
 * The reference's kernels (Simulator/PD-IPC/PdIpcGpuFunc.cu) are plain CUDA C.
 * Compiled by a host C++ compiler with this header included first, each
 * __global__ function becomes an ordinary function, and cuemu::launch runs it
 * the way a GPU would, one block after another:
 *   - every thread of a block is a fiber (ucontext) with its own stack, and
 *     threadIdx / blockIdx / blockDim / gridDim are switched with it;
 *   - __syncthreads() suspends the fiber until every live thread of the block
 *     has reached a barrier (a thread that returned counts as arrived);
 *   - __shared__ variables are thread_local (function-local ones are static):
 *     one copy, shared by the fibers of the running block, which all run on
 *     one host thread (blocks do not overlap in time); an extern __shared__
 *     array is a thread_local array the harness defines;
 *   - atomics are plain read-modify-writes (one host thread runs every fiber),
 *     so an atomic sum adds in thread order within a block and block order
 *     across the grid: one of the orders a GPU may produce.
 * Only what the reference's cloth kernels use is provided.
 */
#ifndef ORACLE_CUDA_EMU_H
#define ORACLE_CUDA_EMU_H

#include <ucontext.h>

#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <vector>

struct uint3 {
    unsigned x, y, z;
};
struct dim3 {
    unsigned x, y, z;
    dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};
typedef int cudaError_t;
static const cudaError_t cudaSuccess = 0;
typedef struct cuemu_blas_handle* cublasHandle_t;

// the built-in variables: plain globals (not macros, so a parameter may be
// named blockDim as in the reference's headers), switched with each fiber
inline uint3 threadIdx{0, 0, 0}, blockIdx{0, 0, 0};
inline dim3 blockDim, gridDim;

namespace cuemu {

struct Fiber {
    ucontext_t ctx;
    std::vector<char> stack;
    uint3 t{0, 0, 0};
    bool done = false, waiting = false;
};

inline ucontext_t g_sched;
inline std::vector<Fiber> g_fibers;
inline Fiber* g_cur = nullptr;
inline const std::function<void()>* g_body = nullptr;
constexpr size_t kStack = 64 * 1024;

inline void fiber_main() {
    (*g_body)();
    g_cur->done = true;
    swapcontext(&g_cur->ctx, &g_sched);
}

// the calling fiber waits at the block barrier
inline void barrier() {
    g_cur->waiting = true;
    swapcontext(&g_cur->ctx, &g_sched);
}

// Runs body() as every thread of every block of grid g x block b.
inline void launch(dim3 g, dim3 b, const std::function<void()>& body) {
    ::gridDim = g;
    ::blockDim = b;
    const size_t nt = (size_t)b.x * b.y * b.z;
    if (nt == 0 || (size_t)g.x * g.y * g.z == 0) return;
    if (g_fibers.size() < nt) g_fibers.resize(nt);
    g_body = &body;
    for (unsigned bz = 0; bz < g.z; ++bz)
        for (unsigned by = 0; by < g.y; ++by)
            for (unsigned bx = 0; bx < g.x; ++bx) {
                ::blockIdx = uint3{bx, by, bz};
                for (size_t i = 0; i < nt; ++i) {
                    Fiber& f = g_fibers[i];
                    if (f.stack.size() < kStack) f.stack.resize(kStack);
                    f.t = uint3{(unsigned)(i % b.x), (unsigned)((i / b.x) % b.y), (unsigned)(i / ((size_t)b.x * b.y))};
                    f.done = false;
                    f.waiting = false;
                    getcontext(&f.ctx);
                    f.ctx.uc_stack.ss_sp = f.stack.data();
                    f.ctx.uc_stack.ss_size = f.stack.size();
                    f.ctx.uc_link = nullptr;
                    makecontext(&f.ctx, fiber_main, 0);
                }
                for (;;) {
                    size_t live = 0;
                    for (size_t i = 0; i < nt; ++i) {
                        Fiber& f = g_fibers[i];
                        if (f.done) continue;
                        if (!f.waiting) {
                            g_cur = &f;
                            ::threadIdx = f.t;
                            swapcontext(&g_sched, &f.ctx);
                        }
                        if (!f.done) ++live;
                    }
                    if (live == 0) break;
                    // every live thread is at the barrier: release them all
                    for (size_t i = 0; i < nt; ++i) g_fibers[i].waiting = false;
                }
            }
    g_cur = nullptr;
}

template <typename K, typename... A>
inline void run(dim3 g, dim3 b, K kernel, A... args) {
    const std::function<void()> body = [&]() { kernel(args...); };
    launch(g, b, body);
}

}  // namespace cuemu

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __shared__ thread_local
#define __syncthreads() ::cuemu::barrier()

// one overload per type, as CUDA declares them (an argument converts to the
// pointee's type, e.g. a double added to a float)
#define CUEMU_ATOMICS(T)                  \
    inline T atomicAdd(T* p, T v) {       \
        T o = *p;                         \
        *p = o + v;                       \
        return o;                         \
    }                                     \
    inline T atomicMin(T* p, T v) {       \
        T o = *p;                         \
        if (v < o) *p = v;                \
        return o;                         \
    }                                     \
    inline T atomicMax(T* p, T v) {       \
        T o = *p;                         \
        if (v > o) *p = v;                \
        return o;                         \
    }                                     \
    inline T atomicExch(T* p, T v) {      \
        T o = *p;                         \
        *p = v;                           \
        return o;                         \
    }
CUEMU_ATOMICS(float)
CUEMU_ATOMICS(double)
CUEMU_ATOMICS(int)
CUEMU_ATOMICS(unsigned)
CUEMU_ATOMICS(unsigned long long)
#undef CUEMU_ATOMICS
inline float rsqrtf(float x) { return 1.0f / std::sqrt(x); }
inline double rsqrt(double x) { return 1.0 / std::sqrt(x); }
inline int cudaDeviceSynchronize() { return 0; }

#endif
