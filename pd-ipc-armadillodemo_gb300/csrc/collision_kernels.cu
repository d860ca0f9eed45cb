// collision_kernels.cu — broad phase, CCD and contact projection of the
// PD-IPC cloth step.
//
// Reference kernels replaced (Simulator/PD-IPC/PdIpcGpuFunc.cu):
//   updateCcdPatchBboxesKernel :1407-1473          -> k_patch_boxes (one warp per patch)
//   AipcBvhs::init (CPU, AipcBvhs.cpp:134-213)      -> k_init_boxes, k_center_scale, k_morton,
//                                                      radix sort, k_karras (GPU LBVH build)
//   updateBvhsBboxesKernel :1506-1561 (1 block)     -> k_refit (bottom-up, atomic arrival flags)
//   findPatchsICPairsKernel :1699-1732 + thrust scan
//   + fillCompactPotentialPatchPairListKernel
//   + computeCcdPatchICPairsVfeeNumKernel :1811      -> k_traverse (one stackless pass over escape
//                                                      links, warp-ballot compaction, record counts)
//   getCcdPotentialICPairsListKernel :1838-1948     -> k_expand (one warp per 32 pairs)
//   getImpactOfTimeKernel :2610-2704 + cublasIsamin -> k_toi_* (atomic min, no host copy)
//   setCollisionConstraintsKernel :2756-2892        -> k_contact_*
//
// The set of overlapping patch pairs does not depend on the tree's shape, so
// the Karras tree reports exactly the pairs of the reference's median-split
// heap tree over the same boxes.
#include <cfloat>
#include <mutex>

#include "geometry.cuh"
#include "kernels.cuh"

namespace pdipc {

namespace {

constexpr int kBlock = 256;
inline int blocks_for(int64_t n, int b = kBlock) { return (int)std::max<int64_t>(1, (n + b - 1) / b); }
inline int grid_cap(int64_t n, int b = kBlock, int cap = 152 * 16) {
    return (int)std::min<int64_t>(cap, std::max<int64_t>(1, (n + b - 1) / b));
}

template <typename T>
__device__ __forceinline__ T tmax_val();
template <>
__device__ __forceinline__ float tmax_val<float>() { return FLT_MAX; }
template <>
__device__ __forceinline__ double tmax_val<double>() { return DBL_MAX; }

template <typename T>
__device__ __forceinline__ void warp_box_reduce(T lo[3], T hi[3]) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        lo[k] = warp_min(lo[k]);
        hi[k] = warp_max(hi[k]);
    }
}

// Swept, inflated patch AABB: per face min/max over x and x+dx of its three
// vertices, minus/plus the inflation radius (getFaceBbox, cu:1350-1375), then
// reduced over the patch's faces.  Boxes are in T: FP64 state (S) is rounded
// to T first (read from the T-rounded copies Xh, Dh when given), so the mixed
// form's boxes are the FP32 form's.  One thread per patch: a grid patch holds
// a few faces (about two on a cloth whose patch grid matches its vertex grid),
// and min/max give the same box in any order.
template <typename T, typename S>
__global__ void k_patch_boxes(int npatch, const int* __restrict__ pfPtr, const int* __restrict__ pfIdx,
                              const int4* __restrict__ Faces, const V4<S>* __restrict__ X,
                              const V4<S>* __restrict__ D, const V4<T>* __restrict__ Xh,
                              const V4<T>* __restrict__ Dh, T infl, Box6<T>* __restrict__ out) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npatch) return;
    T lo[3] = {tmax_val<T>(), tmax_val<T>(), tmax_val<T>()};
    T hi[3] = {-tmax_val<T>(), -tmax_val<T>(), -tmax_val<T>()};
    const int b = __ldg(pfPtr + p), e = __ldg(pfPtr + p + 1);
#pragma unroll 2
    for (int q = b; q < e; ++q) {
        const int4 f = Faces[pfIdx[q]];
        const int vv[3] = {f.x, f.y, f.z};
        T a[3][3], c[3][3];
        for (int j = 0; j < 3; ++j) {
            V4<T> x;
            if (Xh) {
                x = ld4(Xh, vv[j]);
            } else {
                const V4<S> xs = ld4(X, vv[j]);
                x = V4<T>{(T)xs.x, (T)xs.y, (T)xs.z, T(0)};
            }
            a[j][0] = x.x;
            a[j][1] = x.y;
            a[j][2] = x.z;
            if (D) {
                V4<T> d;
                if (Dh) {
                    d = ld4(Dh, vv[j]);
                } else {
                    const V4<S> ds = ld4(D, vv[j]);
                    d = V4<T>{(T)ds.x, (T)ds.y, (T)ds.z, T(0)};
                }
                c[j][0] = x.x + d.x;
                c[j][1] = x.y + d.y;
                c[j][2] = x.z + d.z;
            } else {
                c[j][0] = x.x;
                c[j][1] = x.y;
                c[j][2] = x.z;
            }
        }
        for (int k = 0; k < 3; ++k) {
            T mn = dmin(dmin(dmin(a[0][k], a[1][k]), a[2][k]), dmin(dmin(c[0][k], c[1][k]), c[2][k])) - infl;
            T mx = dmax(dmax(dmax(a[0][k], a[1][k]), a[2][k]), dmax(dmax(c[0][k], c[1][k]), c[2][k])) + infl;
            lo[k] = dmin(lo[k], mn);
            hi[k] = dmax(hi[k], mx);
        }
    }
    Box6<T> bx;
    for (int k = 0; k < 3; ++k) {
        bx.lo[k] = lo[k];
        bx.hi[k] = hi[k];
    }
    out[p] = bx;
}

// Init-time patch boxes over every vertex of the patch's faces, inflated
// (gpuCollisionInit, cpp:1279-1292).
template <typename T, typename S>
__global__ void k_init_boxes(int npatch, const int* __restrict__ pxPtr, const int* __restrict__ pxIdx,
                             const V4<S>* __restrict__ X, T infl, Box6<T>* __restrict__ out) {
    const int p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (p >= npatch) return;
    T lo[3] = {tmax_val<T>(), tmax_val<T>(), tmax_val<T>()};
    T hi[3] = {-tmax_val<T>(), -tmax_val<T>(), -tmax_val<T>()};
    for (int q = pxPtr[p] + lane; q < pxPtr[p + 1]; q += 32) {
        const V4<S> x = ld4(X, pxIdx[q]);
        const T xs[3] = {(T)x.x, (T)x.y, (T)x.z};
        for (int k = 0; k < 3; ++k) {
            lo[k] = dmin(lo[k], xs[k] - infl);
            hi[k] = dmax(hi[k], xs[k] + infl);
        }
    }
    warp_box_reduce(lo, hi);
    if (lane == 0) {
        Box6<T> bx;
        for (int k = 0; k < 3; ++k) {
            bx.lo[k] = lo[k];
            bx.hi[k] = hi[k];
        }
        out[p] = bx;
    }
}

// Centre of the box-centre bounds and the infinity-norm half extent
// (AipcBvhs.cpp:140-160).  One block; init-time only.
template <typename T>
__global__ void k_center_scale(int npatch, const Box6<T>* __restrict__ box, T* __restrict__ cs) {
    __shared__ T smn[3][32], smx[3][32];
    T mn[3] = {tmax_val<T>(), tmax_val<T>(), tmax_val<T>()};
    T mx[3] = {-tmax_val<T>(), -tmax_val<T>(), -tmax_val<T>()};
    for (int p = threadIdx.x; p < npatch; p += blockDim.x) {
        const Box6<T> b = box[p];
        for (int k = 0; k < 3; ++k) {
            const T c = (b.lo[k] + b.hi[k]) / T(2);
            mn[k] = dmin(mn[k], c);
            mx[k] = dmax(mx[k], c);
        }
    }
    warp_box_reduce(mn, mx);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0)
        for (int k = 0; k < 3; ++k) {
            smn[k][w] = mn[k];
            smx[k][w] = mx[k];
        }
    __syncthreads();
    if (w == 0) {
        const int nw = blockDim.x >> 5;
        for (int k = 0; k < 3; ++k) {
            mn[k] = lane < nw ? smn[k][lane] : tmax_val<T>();
            mx[k] = lane < nw ? smx[k][lane] : -tmax_val<T>();
        }
        warp_box_reduce(mn, mx);
        if (lane == 0) {
            T scale = T(0);
            for (int k = 0; k < 3; ++k) {
                const T c = (mn[k] + mx[k]) / T(2);
                cs[k] = c;
                scale = dmax(scale, fabs(mx[k] - c));
            }
            cs[3] = scale;
        }
    }
}

__device__ __forceinline__ unsigned long long spread21(unsigned long long v) {
    v &= 0x1fffffull;
    v = (v | (v << 32)) & 0x1f00000000ffffull;
    v = (v | (v << 16)) & 0x1f0000ff0000ffull;
    v = (v | (v << 8)) & 0x100f00f00f00f00full;
    v = (v | (v << 4)) & 0x10c30c30c30c30c3ull;
    v = (v | (v << 2)) & 0x1249249249249249ull;
    return v;
}
__device__ __forceinline__ unsigned long long q21(int a) {
    long long s = (long long)a + (1ll << 20);
    s = s < 0 ? 0 : (s > (1ll << 21) - 1 ? (1ll << 21) - 1 : s);
    return (unsigned long long)s;
}

// Morton code of each patch centre: centred, divided by the half extent when
// it exceeds 100, times 1000, truncated (AipcBvhs.cpp:162-183).
template <typename T>
__global__ void k_morton(int npatch, const Box6<T>* __restrict__ box, const T* __restrict__ cs,
                         unsigned long long* __restrict__ codes, unsigned long long* __restrict__ keys,
                         int* __restrict__ vals) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npatch) return;
    const Box6<T> b = box[p];
    const T scale = cs[3];
    int q[3];
    for (int k = 0; k < 3; ++k) {
        T v = (b.lo[k] + b.hi[k]) / T(2) - cs[k];
        if (scale > T(100)) v = v / scale;
        q[k] = (int)(v * T(1000));
    }
    const unsigned long long c = spread21(q21(q[0])) | (spread21(q21(q[1])) << 1) | (spread21(q21(q[2])) << 2);
    codes[p] = c;
    keys[p] = c;
    vals[p] = p;
}

__device__ __forceinline__ int kdelta(const unsigned long long* __restrict__ c, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    const unsigned long long a = c[i], b = c[j];
    if (a == b) return 64 + __clz(i ^ j);
    return __clzll(a ^ b);
}

// Karras (2012) binary radix tree over the sorted codes; equal codes are
// split by position.  Internal node i in [0, n-1), leaf k is node n-1+k.
__global__ void k_karras(int n, const unsigned long long* __restrict__ c, int2* __restrict__ child,
                         int* __restrict__ parent) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) parent[0] = -1;
    if (i >= n - 1) return;
    const int d = (kdelta(c, n, i, i + 1) - kdelta(c, n, i, i - 1)) >= 0 ? 1 : -1;
    const int dmin_ = kdelta(c, n, i, i - d);
    int lmax = 2;
    while (kdelta(c, n, i, i + lmax * d) > dmin_) lmax *= 2;
    int l = 0;
    for (int t = lmax / 2; t >= 1; t /= 2)
        if (kdelta(c, n, i, i + (l + t) * d) > dmin_) l += t;
    const int j = i + l * d;
    const int dnode = kdelta(c, n, i, j);
    int s = 0, t = l;
    do {
        t = (t + 1) >> 1;
        if (kdelta(c, n, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    const int gamma = i + s * d + min(d, 0);
    const int left = (min(i, j) == gamma) ? (n - 1 + gamma) : gamma;
    const int right = (max(i, j) == gamma + 1) ? (n - 1 + gamma + 1) : gamma + 1;
    child[i] = make_int2(left, right);
    parent[left] = i;
    parent[right] = i;
}

// Escape links of the stackless traversal: the node to visit once node c's
// subtree is done or skipped.  For a left child that is its sibling, else the
// parent's link; -1 past the root.  Computed once per tree build (refits keep
// the topology); the walk up is bounded by the tree's depth.
__global__ void k_escape(int nnodes, const int2* __restrict__ child, const int* __restrict__ parent,
                         int* __restrict__ escape) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nnodes) return;
    int x = c, e = -1;
    for (int up = 0; x > 0 && up < nnodes; ++up) {  // a tree's depth is below its node count
        const int p = parent[x];
        const int2 ch = child[p];
        if (ch.x == x) {
            e = ch.y;
            break;
        }
        x = p;
    }
    escape[c] = e;
}

template <typename T>
__device__ __forceinline__ Box6<T> load_box_cg(const Box6<T>* p) {
    Box6<T> b;
    const T* q = reinterpret_cast<const T*>(p);
    for (int k = 0; k < 3; ++k) {
        b.lo[k] = __ldcg(q + k);
        b.hi[k] = __ldcg(q + 3 + k);
    }
    return b;
}

// Bottom-up refit: the second thread to reach an internal node merges its
// children and climbs on (replaces the single-block level sweep, cu:1506-1561).
template <typename T>
__global__ void k_refit(int n, const int* __restrict__ leafPatch, const Box6<T>* __restrict__ patchBox,
                        Box6<T>* __restrict__ nodeBox, const int2* __restrict__ child,
                        const int* __restrict__ parent, int* __restrict__ flag) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int node = n - 1 + k;
    nodeBox[node] = patchBox[leafPatch[k]];
    node = parent[node];
    while (node >= 0) {
        __threadfence();
        if (atomicAdd(flag + node, 1) == 0) return;
        __threadfence();
        const int2 ch = child[node];
        const Box6<T> a = load_box_cg(nodeBox + ch.x), b = load_box_cg(nodeBox + ch.y);
        Box6<T> u;
        for (int q = 0; q < 3; ++q) {
            u.lo[q] = dmin(a.lo[q], b.lo[q]);
            u.hi[q] = dmax(a.hi[q], b.hi[q]);
        }
        nodeBox[node] = u;
        node = parent[node];
    }
}

template <typename T>
__device__ __forceinline__ bool overlap(const Box6<T>& a, const Box6<T>& b) {
    // checkOverlap (cu:1612-1625): closed intervals
    if (a.hi[0] < b.lo[0] || b.hi[0] < a.lo[0]) return false;
    if (a.hi[1] < b.lo[1] || b.hi[1] < a.lo[1]) return false;
    if (a.hi[2] < b.lo[2] || b.hi[2] < a.lo[2]) return false;
    return true;
}

// Stackless traversal, one query patch q per thread: every patch p > q whose
// box overlaps q's, skipping pairs of two static patches (they cannot move or
// receive contact forces).  Depth first, left child first, along the escape
// links.  Each warp appends its lanes' finds by ballot: one atomicAdd per
// warp and round reserves a contiguous run, so the pair stores coalesce.
// With each pair it writes the pair's record counts (points(q) x faces(p) +
// points(p) x faces(q) point-triangle, edges(q) x edges(p) edge-edge,
// computeCcdPatchICPairsVfeeNumKernel cu:1811-1836).  Finds past `cap` are
// counted, not written: the caller grows the buffers and runs the pass again.
// The pair order varies between runs (the order warps reserve their runs);
// every consumer of the list is order-free or sums with atomics anyway.
template <typename T>
__global__ void __launch_bounds__(128) k_traverse(int n, const Box6<T>* __restrict__ patchBox,
                                                  const Box6<T>* __restrict__ nodeBox,
                                                  const int2* __restrict__ child, const int* __restrict__ escape,
                                                  const int* __restrict__ leafPatch,
                                                  const uint8_t* __restrict__ pStatic, const int* __restrict__ pfPtr,
                                                  const int* __restrict__ ppPtr, const int* __restrict__ pePtr,
                                                  int2* __restrict__ out, int64_t* __restrict__ cpt,
                                                  int64_t* __restrict__ cee, int64_t cap,
                                                  unsigned long long* __restrict__ count,
                                                  unsigned int* __restrict__ err) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned lane = threadIdx.x & 31u;
    bool active = q < n && n > 1;
    // a depth-first walk visits each of the 2n-1 nodes at most once
    int budget = 2 * n;
    Box6<T> qb{};
    bool qs = false;
    int fa = 0, va = 0, ea = 0;
    if (active) {
        qb = patchBox[q];
        qs = pStatic[q] != 0;
        fa = pfPtr[q + 1] - pfPtr[q];
        va = ppPtr[q + 1] - ppPtr[q];
        ea = pePtr[q + 1] - pePtr[q];
    }
    int node = 0;
    while (__any_sync(0xffffffffu, active)) {
        int found = -1;
        while (active) {  // to this lane's next find, or to the end of its traversal
            int next;
            if (overlap(qb, nodeBox[node])) {
                if (node >= n - 1) {
                    const int p = leafPatch[node - (n - 1)];
                    if (q < p && !(qs && pStatic[p])) found = p;
                    next = escape[node];
                } else {
                    next = child[node].x;
                }
            } else {
                next = escape[node];
            }
            node = next;
            if (node < 0) active = false;
            if (--budget < 0 && active) {  // only a malformed tree gets here
                atomicOr(err, (unsigned int)kErrTraversal);
                active = false;
            }
            if (found >= 0) break;
        }
        const unsigned m = __ballot_sync(0xffffffffu, found >= 0);
        if (m == 0u) continue;
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(count, (unsigned long long)__popc(m));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (found >= 0) {
            const unsigned long long pos = base + (unsigned long long)__popc(m & ((1u << lane) - 1u));
            if (pos < (unsigned long long)cap) {
                const int p = found;
                const int64_t fb = pfPtr[p + 1] - pfPtr[p], vb = ppPtr[p + 1] - ppPtr[p],
                              eb = pePtr[p + 1] - pePtr[p];
                out[pos] = make_int2(q, p);
                cpt[pos] = (int64_t)va * fb + vb * (int64_t)fa;
                cee[pos] = (int64_t)ea * eb;
            }
        }
    }
}

// Expansion of the patch pairs into point-triangle records (points of A x
// faces of B, then points of B x faces of A, point-major) and edge-edge
// records (edges of A x edges of B), as getCcdPotentialICPairsListKernel
// (cu:1838-1948) lays them out.  A warp takes 32 consecutive pairs, whose
// records form one contiguous run of each list, and writes the run lane by
// lane (16-byte records, 512 bytes per warp store); a record finds its pair by
// a binary search over the lanes' run offsets (shuffles) and the pair's
// tables by shuffles from the owning lane.
__global__ void __launch_bounds__(kBlock) k_expand(int64_t npairs, const int2* __restrict__ pairs,
                                                   const int* __restrict__ pfPtr, const int* __restrict__ pfIdx,
                                                   const int* __restrict__ ppPtr, const int* __restrict__ ppIdx,
                                                   const int* __restrict__ pePtr, const int* __restrict__ peIdx,
                                                   const int4* __restrict__ Faces, const int2* __restrict__ Edges,
                                                   const int64_t* __restrict__ opt, const int64_t* __restrict__ oee,
                                                   int4* __restrict__ PT, int4* __restrict__ EE) {
    constexpr unsigned kAll = 0xffffffffu;
    const int64_t w0 = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) << 5;
    const int lane = threadIdx.x & 31;
    if (w0 >= npairs) return;  // whole warps only
    const int64_t t = w0 + lane;
    const int last = (npairs - w0 < 32 ? (int)(npairs - w0) : 32) - 1;
    int fa0 = 0, fa = 0, fb0 = 0, fb = 0, va0 = 0, va = 0, vb0 = 0, vb = 0, ea0 = 0, ea = 0, eb0 = 0, eb = 0;
    int64_t bp = INT64_MAX, be = INT64_MAX;
    if (lane <= last) {
        const int2 pr = pairs[t];
        fa0 = pfPtr[pr.x];
        fa = pfPtr[pr.x + 1] - fa0;
        fb0 = pfPtr[pr.y];
        fb = pfPtr[pr.y + 1] - fb0;
        va0 = ppPtr[pr.x];
        va = ppPtr[pr.x + 1] - va0;
        vb0 = ppPtr[pr.y];
        vb = ppPtr[pr.y + 1] - vb0;
        ea0 = pePtr[pr.x];
        ea = pePtr[pr.x + 1] - ea0;
        eb0 = pePtr[pr.y];
        eb = pePtr[pr.y + 1] - eb0;
        bp = opt[t];
        be = oee[t];
    }
    // the owning lane of record r: the largest lane j <= last with start_j <= r
    auto owner = [&](int64_t start, int64_t r) {
        int j = 0;
#pragma unroll
        for (int step = 16; step >= 1; step >>= 1) {
            const int c = j + step;
            const int64_t v = __shfl_sync(kAll, start, c & 31);
            if (c <= last && v <= r) j = c;
        }
        return j;
    };
    const int nab = va * fb;
    const int64_t ptBeg = __shfl_sync(kAll, bp, 0);
    const int64_t ptEnd = __shfl_sync(kAll, bp + (int64_t)nab + (int64_t)vb * fa, last);
    for (int64_t r0 = ptBeg; r0 < ptEnd; r0 += 32) {
        const int64_t r = r0 + lane;
        const int j = owner(bp, r);
        const int64_t id = r - __shfl_sync(kAll, bp, j);
        const int jnab = __shfl_sync(kAll, nab, j), jfa = __shfl_sync(kAll, fa, j), jfb = __shfl_sync(kAll, fb, j);
        const int jfa0 = __shfl_sync(kAll, fa0, j), jfb0 = __shfl_sync(kAll, fb0, j);
        const int jva0 = __shfl_sync(kAll, va0, j), jvb0 = __shfl_sync(kAll, vb0, j);
        if (r < ptEnd) {
            int v, f;
            if (id < jnab) {
                v = ppIdx[jva0 + (int)(id / jfb)];
                f = pfIdx[jfb0 + (int)(id % jfb)];
            } else {
                const int id2 = (int)(id - jnab);
                v = ppIdx[jvb0 + id2 / jfa];
                f = pfIdx[jfa0 + id2 % jfa];
            }
            const int4 F = Faces[f];
            PT[r] = make_int4(v, F.x, F.y, F.z);
        }
    }
    const int64_t eeBeg = __shfl_sync(kAll, be, 0);
    const int64_t eeEnd = __shfl_sync(kAll, be + (int64_t)ea * eb, last);
    for (int64_t r0 = eeBeg; r0 < eeEnd; r0 += 32) {
        const int64_t r = r0 + lane;
        const int j = owner(be, r);
        const int64_t id = r - __shfl_sync(kAll, be, j);
        const int jeb = __shfl_sync(kAll, eb, j), jea0 = __shfl_sync(kAll, ea0, j),
                  jeb0 = __shfl_sync(kAll, eb0, j);
        if (r < eeEnd) {
            const int2 a = Edges[peIdx[jea0 + (int)(id / jeb)]], b = Edges[peIdx[jeb0 + (int)(id % jeb)]];
            EE[r] = make_int4(a.x, a.y, b.x, b.y);
        }
    }
}

template <typename T, typename TC>
__device__ __forceinline__ void gather4(const V4<T>* __restrict__ X, const int ids[4], TC out[4][3]) {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const V4<T> v = ld4(X, ids[j]);
        out[j][0] = (TC)v.x;
        out[j][1] = (TC)v.y;
        out[j][2] = (TC)v.z;
    }
}

template <typename TC>
__device__ __forceinline__ void block_min_to(TC v, TC* dst) {
    __shared__ TC red[kBlock / 32];
    v = warp_min(v);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        TC w = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : TC(1);
        w = warp_min(w);
        if (threadIdx.x == 0 && w < TC(1)) atomic_min_nonneg(dst, w);
    }
}

// Resident blocks per SM asked of the candidate kernels: they are latency-bound
// gathers, and four blocks (64 registers) measured 25% faster than two for the
// FP32 arithmetic of the mixed and FP32 modes, despite a few spills; the FP64
// mode keeps the compiler's choice.
template <typename T>
constexpr int kCandBlocks = sizeof(T) == 4 ? 4 : 1;

// The FP64 time of impact of one candidate from the FP64 state (coordinates
// relative to its first vertex).  Out of line: few candidates reach it, and
// keeping its registers out of k_toi's main loop keeps that loop's occupancy.
template <typename TC, bool kPT>
__device__ __noinline__ TC toi_refine(const V4<TC>* __restrict__ X0, const V4<TC>* __restrict__ X1, const int* ids,
                                      TC eta, int max_iter) {
    TC xd[4][3], dd[4][3];
    const V4<TC> o = ld4(X0, ids[0]);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const V4<TC> a = ld4(X0, ids[j]), b = ld4(X1, ids[j]);
        xd[j][0] = a.x - o.x;
        xd[j][1] = a.y - o.y;
        xd[j][2] = a.z - o.z;
        dd[j][0] = b.x - a.x;
        dd[j][1] = b.y - a.y;
        dd[j][2] = b.z - a.z;
    }
    return kPT ? geo::ccd_pt<TC>(xd, dd, eta, max_iter) : geo::ccd_ee<TC>(xd, dd, eta, max_iter);
}

// Mixed mode, one candidate: the pair's coordinates relative to its first
// vertex and its motion, in FP32 from the float-float mirrors.
template <typename T>
__device__ __forceinline__ void toi_rel(const int* ids, const V4<T>* __restrict__ X0h, const V4<T>* __restrict__ X0l,
                                        const V4<T>* __restrict__ X1h, const V4<T>* __restrict__ X1l, T (&x)[4][3],
                                        T (&dx)[4][3]) {
    const V4<T> oh = ld4(X0h, ids[0]), ol = ld4(X0l, ids[0]);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const V4<T> ah = ld4(X0h, ids[j]), al = ld4(X0l, ids[j]);
        const V4<T> bh = ld4(X1h, ids[j]), bl = ld4(X1l, ids[j]);
        x[j][0] = diff_ff(ah.x, al.x, oh.x, ol.x);
        x[j][1] = diff_ff(ah.y, al.y, oh.y, ol.y);
        x[j][2] = diff_ff(ah.z, al.z, oh.z, ol.z);
        dx[j][0] = diff_ff(bh.x, bl.x, ah.x, al.x);
        dx[j][1] = diff_ff(bh.y, bl.y, ah.y, al.y);
        dx[j][2] = diff_ff(bh.z, bl.z, ah.z, al.z);
    }
}

// Mixed mode, stage 1 of a candidate: false when its time of impact is 1
// without any CCD iteration (shared vertex; the swept-box filter, first on the
// high parts alone with the distance widened past the largest effect of the
// dropped low parts (|low| <= 2^-24 |x|, plus the roundings: < 2^-18 of the
// largest coordinate), then exactly; no motion, or the CCD's box-gap exit).
template <typename T, bool kPT>
__device__ __forceinline__ bool toi_needs_ccd(const int4 c, const V4<T>* __restrict__ X0h, const V4<T>* __restrict__ X0l,
                                              const V4<T>* __restrict__ X1h, const V4<T>* __restrict__ X1l, T slack) {
    if (kPT ? (c.x == c.y || c.x == c.z || c.x == c.w) : (c.x == c.z || c.x == c.w || c.y == c.z || c.y == c.w))
        return false;
    const int ids[4] = {c.x, c.y, c.z, c.w};
    {
        T xh[4][3], dh[4][3], m = T(0);
        const V4<T> o = ld4(X0h, ids[0]);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const V4<T> ah = ld4(X0h, ids[j]), bh = ld4(X1h, ids[j]);
            xh[j][0] = ah.x - o.x;
            xh[j][1] = ah.y - o.y;
            xh[j][2] = ah.z - o.z;
            dh[j][0] = bh.x - ah.x;
            dh[j][1] = bh.y - ah.y;
            dh[j][2] = bh.z - ah.z;
            m = dmax(m, dmax(dmax(fabsf(ah.x), fabsf(ah.y)), dmax(fabsf(ah.z), fabsf(bh.x))));
            m = dmax(m, dmax(fabsf(bh.y), fabsf(bh.z)));
        }
        const T wide = slack + m * T(1.0 / 65536.0);
        if (!(kPT ? geo::pt_ccd_broad<T>(xh, dh, wide) : geo::ee_ccd_broad<T>(xh, dh, wide))) return false;
        // the CCD's box-gap exit from the high parts too: they are within
        // 2^-22 m of the exact relative coordinates and motion per component
        // (m bounds |x|), so the margins below keep it conservative; most pairs
        // settle here without loading the low parts
        const T eps = m * T(1.0 / 1048576.0);
        if (geo::ccd_trivial_approx<T, kPT>(xh, dh, T(4) * eps, T(8) * eps)) return false;
    }
    T x[4][3], dx[4][3];
    toi_rel<T>(ids, X0h, X0l, X1h, X1l, x, dx);
    if (!(kPT ? geo::pt_ccd_broad<T>(x, dx, slack) : geo::ee_ccd_broad<T>(x, dx, slack))) return false;
    return !(kPT ? geo::ccd_pt_trivial<T>(x, dx) : geo::ccd_ee_trivial<T>(x, dx));
}

// Mixed mode, stage 2: the FP32 additive CCD, and for a time of impact below 1
// its FP64 re-evaluation from the FP64 state.
template <typename T, typename TC, bool kPT>
__device__ __forceinline__ TC toi_ccd(const int4 c, const V4<TC>* __restrict__ X0, const V4<TC>* __restrict__ X1,
                                      const V4<T>* __restrict__ X0h, const V4<T>* __restrict__ X0l,
                                      const V4<T>* __restrict__ X1h, const V4<T>* __restrict__ X1l, TC eta,
                                      int max_iter) {
    const int ids[4] = {c.x, c.y, c.z, c.w};
    T x[4][3], dx[4][3];
    toi_rel<T>(ids, X0h, X0l, X1h, X1l, x, dx);
    const T tf = kPT ? geo::ccd_pt<T>(x, dx, (T)eta, max_iter) : geo::ccd_ee<T>(x, dx, (T)eta, max_iter);
    return tf < T(1) ? toi_refine<TC, kPT>(X0, X1, ids, eta, max_iter) : TC(1);
}

// getImpactOfTimeKernel (cu:2610-2704): skip pairs sharing a vertex, swept-AABB
// filter with slack, additive CCD; global minimum by integer atomicMin.
// kRel (mixed precision): coordinates relative to the pair's first vertex,
// formed in FP32 from the float-float mirrors of the FP64 state, an FP32
// additive CCD on them, and every candidate that would clamp the step
// (toi < 1) re-evaluated in FP64 from the FP64 state, so the minimum is an
// FP64 time of impact.  The stage-1 tests settle most candidates; each warp
// queues the rest in shared memory and runs the CCD iterations on 32 of them
// at a time, so they run on full warps.
template <typename T, typename TC, bool kPT, bool kRel>
__global__ void __launch_bounds__(kBlock, kCandBlocks<T>) k_toi(int64_t n, const int4* __restrict__ cand,
                                                const V4<TC>* __restrict__ X0, const V4<TC>* __restrict__ X1,
                                                const V4<T>* __restrict__ X0h, const V4<T>* __restrict__ X0l,
                                                const V4<T>* __restrict__ X1h, const V4<T>* __restrict__ X1l,
                                                TC slack, TC eta, int max_iter, TC* __restrict__ per,
                                                TC* __restrict__ toi_min, const OuterGate* __restrict__ gate) {
    if (outer_stopped(gate)) return;
    TC local = TC(1);
    if constexpr (kRel) {
        __shared__ int64_t queue[kBlock / 32][64];
        const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
        int qn = 0;
        const int64_t step = (int64_t)gridDim.x * (kBlock / 32) * 32;
        for (int64_t base = ((int64_t)blockIdx.x * (kBlock / 32) + w) * 32; base < n; base += step) {
            const int64_t t = base + lane;
            const bool need = t < n && toi_needs_ccd<T, kPT>(cand[t], X0h, X0l, X1h, X1l, (T)slack);
            if (t < n && !need && per) per[t] = TC(1);
            const unsigned m = __ballot_sync(0xffffffffu, need);
            if (need) queue[w][qn + __popc(m & ((1u << lane) - 1u))] = t;
            qn += __popc(m);
            __syncwarp();
            if (qn >= 32) {
                const int64_t tq = queue[w][lane];
                __syncwarp();
                if (lane < qn - 32) queue[w][lane] = queue[w][lane + 32];
                __syncwarp();
                qn -= 32;
                const TC toi = toi_ccd<T, TC, kPT>(cand[tq], X0, X1, X0h, X0l, X1h, X1l, eta, max_iter);
                if (per) per[tq] = toi;
                if (toi < local) local = toi;
            }
        }
        if (lane < qn) {
            const int64_t tq = queue[w][lane];
            const TC toi = toi_ccd<T, TC, kPT>(cand[tq], X0, X1, X0h, X0l, X1h, X1l, eta, max_iter);
            if (per) per[tq] = toi;
            if (toi < local) local = toi;
        }
    } else {
        for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
            const int4 c = cand[t];
            const int ids[4] = {c.x, c.y, c.z, c.w};
            TC toi = TC(1);
            const bool shared = kPT ? (c.x == c.y || c.x == c.z || c.x == c.w)
                                    : (c.x == c.z || c.x == c.w || c.y == c.z || c.y == c.w);
            if (!shared) {
                TC x[4][3], dx[4][3];
                gather4<TC, TC>(X0, ids, x);
                gather4<TC, TC>(X1, ids, dx);
#pragma unroll
                for (int j = 0; j < 4; ++j)
#pragma unroll
                    for (int k = 0; k < 3; ++k) dx[j][k] -= x[j][k];
                if (kPT) {
                    if (geo::pt_ccd_broad<TC>(x, dx, slack)) toi = geo::ccd_pt<TC>(x, dx, eta, max_iter);
                } else {
                    if (geo::ee_ccd_broad<TC>(x, dx, slack)) toi = geo::ccd_ee<TC>(x, dx, eta, max_iter);
                }
            }
            if (per) per[t] = toi;
            if (toi < local) local = toi;
        }
    }
    block_min_to(local, toi_min);
}

// ccd_mode 1: the FP64 coplanarity-cubic pass over the same candidates, after
// k_toi.  Candidates that pass the shared-vertex and swept-box tests (in
// FP64) get geo::ccd_cubic; a result below the additive CCD's lowers the
// candidate's time of impact and the running minimum.  FP64 on the GPU is
// kept to this root solve and the few candidates that reach it.
// kAlone (ccd_mode 2): no additive CCD ran, so every candidate's entry is
// written here (1 where the cubic finds no contact).
template <typename TC, bool kPT, bool kAlone>
__global__ void __launch_bounds__(kBlock) k_toi_cubic(int64_t n, const int4* __restrict__ cand,
                                                      const V4<TC>* __restrict__ X0, const V4<TC>* __restrict__ X1,
                                                      double slack, TC* __restrict__ per, TC* __restrict__ toi_min,
                                                      const OuterGate* __restrict__ gate) {
    if (outer_stopped(gate)) return;
    TC local = TC(1);
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        const int4 c = cand[t];
        if (kAlone && per) per[t] = TC(1);
        if (kPT ? (c.x == c.y || c.x == c.z || c.x == c.w) : (c.x == c.z || c.x == c.w || c.y == c.z || c.y == c.w))
            continue;
        const int ids[4] = {c.x, c.y, c.z, c.w};
        double x[4][3], d[4][3];
        gather4<TC, double>(X0, ids, x);
        gather4<TC, double>(X1, ids, d);
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int k = 0; k < 3; ++k) d[j][k] -= x[j][k];
        if (!(kPT ? geo::pt_ccd_broad<double>(x, d, slack) : geo::ee_ccd_broad<double>(x, d, slack))) continue;
        // relative to the first point: the cubic's coefficients lose nothing to large coordinates
#pragma unroll
        for (int j = 3; j >= 0; --j)
#pragma unroll
            for (int k = 0; k < 3; ++k) x[j][k] -= x[0][k];
        const TC tc = (TC)geo::ccd_cubic<kPT>(x, d);
        if (tc < TC(1)) {
            if (per && tc < per[t]) per[t] = tc;
            if (tc < local) local = tc;
        }
    }
    block_min_to(local, toi_min);
}

template <typename TC>
__global__ void k_toi_finalize(TC* __restrict__ toi_min, TC* __restrict__ toi, double scale,
                               const OuterGate* __restrict__ gate) {
    if (outer_stopped(gate)) return;
    const TC m = *toi_min;
    const TC t = (m < TC(1)) ? (TC)((double)m * scale) : TC(1);
    *toi = t;
    *toi_min = TC(1);
}

// Per-instance stopping: each candidate whose time of impact is below 1
// lowers the running minimum of every instance among its vertices (static
// vertices belong to none); then each instance's clamp.
template <typename TC>
__global__ void k_inst_toi(int64_t n, const int4* __restrict__ cand, const TC* __restrict__ per,
                           const int* __restrict__ VInst, TC* __restrict__ inst_min,
                           const OuterGate* __restrict__ gate) {
    if (outer_stopped(gate)) return;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        const TC v = per[t];
        if (!(v < TC(1))) continue;
        const int4 c = cand[t];
        const int k[4] = {VInst[c.x], VInst[c.y], VInst[c.z], VInst[c.w]};
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            bool seen = k[j] < 0;
#pragma unroll
            for (int q = 0; q < j; ++q) seen = seen || k[q] == k[j];
            if (!seen) atomic_min_nonneg(inst_min + k[j], v);
        }
    }
}
template <typename TC>
__global__ void k_inst_toi_finalize(int ninst, TC* __restrict__ inst_min, TC* __restrict__ inst_toi, double scale,
                                    const OuterGate* __restrict__ gate) {
    if (outer_stopped(gate)) return;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < ninst; k += gridDim.x * blockDim.x) {
        const TC m = inst_min[k];
        inst_toi[k] = (m < TC(1)) ? (TC)((double)m * scale) : TC(1);
        inst_min[k] = TC(1);
    }
}

// the contact pass's accumulators start from zero
template <typename T>
__global__ void k_contact_clear(int n, T* __restrict__ diag, V4<T>* __restrict__ rhs,
                                unsigned long long* __restrict__ active, const OuterGate* __restrict__ gate) {
    if (outer_stopped(gate)) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) *active = 0ull;
    if (i >= n) return;
    diag[i] = T(0);
    rhs[i] = V4<T>{T(0), T(0), T(0), T(0)};
}

template <typename TC>
struct ContactConsts {
    TC dh, dh2, kappa, dt;
};

// setCollisionConstraintsKernel (cu:2756-2892): a pair closer than dhat adds
// w = kappa b(d^2) + min(m_p, m_q)/dt^2 to the diagonal of its 4 vertices and
// w * target to their right-hand side; targets push the pair apart to dhat
// along the closest-point direction, split by the mass ratio.
// kRel (mixed precision): relative coordinates formed in FP64, an FP32 filter
// on their rounding, FP64 distance and weight for pairs within 1.1 dhat, and
// the right-hand side accumulated as w * (target - x) so the later residual
// needs no cancellation.
// One contact candidate (setCollisionConstraintsKernel, cu:2756-2892).  kStage 0:
// the whole test and, for a pair closer than dhat, its diagonal and right-hand
// side terms; 1 (mixed mode): only the shared-vertex test and the box filters on
// the high parts of the mirrors (1: the pair survives them); 2 (mixed mode): the
// rest, for a pair that survived stage 1.  Returns 1 for an active pair.
template <typename T, typename TC, bool kPT, bool kRel, int kStage>
__device__ __forceinline__ unsigned contact_candidate(const int4 c, const V4<TC>* __restrict__ X,
                                                      const V4<T>* __restrict__ Xh, const V4<T>* __restrict__ Xl,
                                                      const TC* __restrict__ mass, const ContactConsts<TC>& cc,
                                                      T* __restrict__ diag, V4<T>* __restrict__ rhs) {
    const int ids[4] = {c.x, c.y, c.z, c.w};
    if (kStage != 2 &&
        (kPT ? (c.x == c.y || c.x == c.z || c.x == c.w) : (c.x == c.z || c.x == c.w || c.y == c.z || c.y == c.w)))
        return 0u;
    TC p[4][3];
    if constexpr (kRel) {
        if (kStage != 2) {  // the box filter on the high parts alone, widened as in k_toi
            T qh[4][3], m = T(0);
            const V4<T> o = ld4(Xh, ids[0]);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const V4<T> ah = ld4(Xh, ids[j]);
                qh[j][0] = ah.x - o.x;
                qh[j][1] = ah.y - o.y;
                qh[j][2] = ah.z - o.z;
                m = dmax(m, dmax(fabsf(ah.x), dmax(fabsf(ah.y), fabsf(ah.z))));
            }
            const T wide = (T)cc.dh + m * T(1.0 / 65536.0);
            bool farh = false;
            if (kPT) {
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const T tmin = geo::mn3(qh[1][k], qh[2][k], qh[3][k]);
                    const T tmax = geo::mx3(qh[1][k], qh[2][k], qh[3][k]);
                    if ((qh[0][k] - tmax) > wide || (tmin - qh[0][k]) > wide) farh = true;
                }
            } else {
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const T mina = dmin(qh[0][k], qh[1][k]), maxa = dmax(qh[0][k], qh[1][k]);
                    const T minb = dmin(qh[2][k], qh[3][k]), maxb = dmax(qh[2][k], qh[3][k]);
                    if ((mina - maxb) > wide || (minb - maxa) > wide) farh = true;
                }
            }
            if (farh) return 0u;
            // the boxes' Euclidean gap also bounds the distance from below: a
            // pair beyond sqrt(2) dhat (after the widening) fails the filter below
            const T g = dsqrt(kPT ? geo::box_gap2<T, 1, 3>(qh, qh + 1) : geo::box_gap2<T, 2, 2>(qh, qh + 2)) -
                        T(2) * (wide - (T)cc.dh);
            if (g > T(0) && g * g > T(2) * (T)cc.dh2) return 0u;
            if (kStage == 1) return 1u;
        }
        T q[4][3];
        const V4<T> oh = ld4(Xh, ids[0]), ol = ld4(Xl, ids[0]);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const V4<T> ah = ld4(Xh, ids[j]), al = ld4(Xl, ids[j]);
            q[j][0] = diff_ff(ah.x, al.x, oh.x, ol.x);
            q[j][1] = diff_ff(ah.y, al.y, oh.y, ol.y);
            q[j][2] = diff_ff(ah.z, al.z, oh.z, ol.z);
        }
        const T dhf = (T)cc.dh;
        bool far = false;
        if (kPT) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const T tmin = geo::mn3(q[1][k], q[2][k], q[3][k]), tmax = geo::mx3(q[1][k], q[2][k], q[3][k]);
                if ((q[0][k] - tmax) > dhf || (tmin - q[0][k]) > dhf) far = true;
            }
        } else {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const T mina = dmin(q[0][k], q[1][k]), maxa = dmax(q[0][k], q[1][k]);
                const T minb = dmin(q[2][k], q[3][k]), maxb = dmax(q[2][k], q[3][k]);
                if ((mina - maxb) > dhf || (minb - maxa) > dhf) far = true;
            }
        }
        if (far) return 0u;
        T df[3], a_, b_, c_;
        const T d2f = kPT ? geo::vtx_tri<T>(q[0], q[1], q[2], q[3], &a_, &b_, &c_, df)
                          : geo::edge_edge_sq<T>(q[0], q[1], q[2], q[3], &a_, &b_, df);
        if (!(d2f < (T)(1.21 * cc.dh2))) return 0u;
        const V4<TC> o = ld4(X, ids[0]);  // close pair: FP64 relative coordinates
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const V4<TC> a = ld4(X, ids[j]);
            p[j][0] = a.x - o.x;
            p[j][1] = a.y - o.y;
            p[j][2] = a.z - o.z;
        }
    } else {
        gather4<TC, TC>(X, ids, p);
        bool far = false;
        if (kPT) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {  // point_triangle_cd_broadphase (cu:2328-2345)
                const TC tmin = geo::mn3(p[1][k], p[2][k], p[3][k]), tmax = geo::mx3(p[1][k], p[2][k], p[3][k]);
                if ((p[0][k] - tmax) > cc.dh || (tmin - p[0][k]) > cc.dh) far = true;
            }
        } else {
#pragma unroll
            for (int k = 0; k < 3; ++k) {  // edge_edge_cd_broadphase (cu:2405-2424)
                const TC mina = dmin(p[0][k], p[1][k]), maxa = dmax(p[0][k], p[1][k]);
                const TC minb = dmin(p[2][k], p[3][k]), maxb = dmax(p[2][k], p[3][k]);
                if ((mina - maxb) > cc.dh || (minb - maxa) > cc.dh) far = true;
            }
        }
        if (far) return 0u;
    }
    TC d[3], dist2, mp, mq;
    if (kPT) {
        TC a, b, cq;
        dist2 = geo::vtx_tri(p[0], p[1], p[2], p[3], &a, &b, &cq, d);
        if (dist2 >= cc.dh2) return 0u;
        mp = mass[c.x];
        mq = a * mass[c.y] + b * mass[c.z] + cq * mass[c.w];
    } else {
        TC r, s;
        dist2 = geo::edge_edge_sq(p[0], p[1], p[2], p[3], &r, &s, d);
        if (dist2 >= cc.dh2) return 0u;
        mp = (TC(1) - r) * mass[c.x] + r * mass[c.y];
        mq = (TC(1) - s) * mass[c.z] + s * mass[c.w];
    }
    TC dist = dsqrt(dist2);
    const TC t2 = dist2 - cc.dh2;
    const TC bar = -cc.kappa * t2 * t2 * dlog(dist2 / cc.dh2) / (cc.dh2 * cc.dh2);
    const TC w = bar + dmin(mp, mq) / (cc.dt * cc.dt);
    const TC rp = mq / (mp + mq), rq = mp / (mp + mq);
    const TC len = dsqrt(geo::dot3(d, d));
    for (int k = 0; k < 3; ++k) d[k] /= len;
    dist = cc.dh - dist;
    const TC dp = dist * rp, dq = dist * rq;
    for (int j = 0; j < 4; ++j) atomicAdd(diag + ids[j], (T)w);
    for (int k = 0; k < 3; ++k) {
        TC t0, t1, t2_, t3;
        if (kRel) {  // w (target - x)
            t0 = w * (dp * d[k]);
            t1 = kPT ? -w * (dq * d[k]) : w * (dp * d[k]);
            t2_ = -w * (dq * d[k]);
            t3 = -w * (dq * d[k]);
        } else {
            t0 = w * (p[0][k] + dp * d[k]);
            t1 = kPT ? w * (p[1][k] - dq * d[k]) : w * (p[1][k] + dp * d[k]);
            t2_ = w * (p[2][k] - dq * d[k]);
            t3 = w * (p[3][k] - dq * d[k]);
        }
        atomicAdd(&rhs[ids[0]].x + k, (T)t0);
        atomicAdd(&rhs[ids[1]].x + k, (T)t1);
        atomicAdd(&rhs[ids[2]].x + k, (T)t2_);
        atomicAdd(&rhs[ids[3]].x + k, (T)t3);
    }
    return 1u;
}

template <typename T, typename TC, bool kPT, bool kRel>
__global__ void __launch_bounds__(kBlock, kCandBlocks<T>) k_contact(int64_t n, const int4* __restrict__ cand,
                                                    const V4<TC>* __restrict__ X, const V4<T>* __restrict__ Xh,
                                                    const V4<T>* __restrict__ Xl, const TC* __restrict__ mass,
                                                    ContactConsts<TC> cc, T* __restrict__ diag,
                                                    V4<T>* __restrict__ rhs, unsigned long long* __restrict__ active,
                                                    const OuterGate* __restrict__ gate) {
    if (outer_stopped(gate)) return;
    unsigned int my = 0;
    if constexpr (kRel) {
        // Most candidates fail the cheap stage-1 filter.  Each warp filters 32
        // consecutive candidates at a time and queues the survivors in shared
        // memory; whenever 32 are queued the whole warp runs the rest of the
        // test on them, so the distance work runs on full warps.
        __shared__ int64_t queue[kBlock / 32][64];
        const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
        int qn = 0;
        const int64_t step = (int64_t)gridDim.x * (kBlock / 32) * 32;
        for (int64_t base = ((int64_t)blockIdx.x * (kBlock / 32) + w) * 32; base < n; base += step) {
            const int64_t t = base + lane;
            const bool pass = t < n && contact_candidate<T, TC, kPT, kRel, 1>(cand[t], X, Xh, Xl, mass, cc, diag, rhs);
            const unsigned m = __ballot_sync(0xffffffffu, pass);
            if (pass) queue[w][qn + __popc(m & ((1u << lane) - 1u))] = t;
            qn += __popc(m);
            __syncwarp();
            if (qn >= 32) {
                const int64_t tq = queue[w][lane];
                __syncwarp();
                if (lane < qn - 32) queue[w][lane] = queue[w][lane + 32];
                __syncwarp();
                qn -= 32;
                my += contact_candidate<T, TC, kPT, kRel, 2>(cand[tq], X, Xh, Xl, mass, cc, diag, rhs);
            }
        }
        if (lane < qn) my += contact_candidate<T, TC, kPT, kRel, 2>(cand[queue[w][lane]], X, Xh, Xl, mass, cc, diag, rhs);
    } else {
        for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
            my += contact_candidate<T, TC, kPT, kRel, 0>(cand[t], X, Xh, Xl, mass, cc, diag, rhs);
    }
    my = warp_sum(my);
    if ((threadIdx.x & 31) == 0 && my) atomicAdd(active, (unsigned long long)my);
}

}  // namespace

template <typename T, typename TC>
void launch_patch_boxes(const Dev<T, TC>& d, const V4<TC>* X, const V4<TC>* D, const V4<T>* Xh, const V4<T>* Dh,
                        T infl, cudaStream_t s) {
    if (d.npatch == 0) return;
    k_patch_boxes<T, TC><<<blocks_for(d.npatch, 128), 128, 0, s>>>(d.npatch, d.pfPtr, d.pfIdx, d.Faces, X, D, Xh, Dh,
                                                                  infl, d.PatchBox);
}
template <typename T, typename TC>
void launch_patch_init_boxes(const Dev<T, TC>& d, T infl, cudaStream_t s) {
    if (d.npatch == 0) return;
    k_init_boxes<T, TC><<<blocks_for((int64_t)d.npatch * 32), kBlock, 0, s>>>(d.npatch, d.pxPtr, d.pxIdx, d.P, infl,
                                                                         d.PatchBox);
}
template <typename T, typename TC>
void launch_morton(const Dev<T, TC>& d, T* cs, unsigned long long* keys, int* vals, cudaStream_t s) {
    if (d.npatch == 0) return;
    k_center_scale<T><<<1, 1024, 0, s>>>(d.npatch, d.PatchBox, cs);
    k_morton<T><<<blocks_for(d.npatch), kBlock, 0, s>>>(d.npatch, d.PatchBox, cs, d.Morton, keys, vals);
}
template <typename T, typename TC>
void launch_karras(const Dev<T, TC>& d, const unsigned long long* sorted, cudaStream_t s) {
    if (d.npatch == 0) return;
    k_karras<<<blocks_for(d.npatch), kBlock, 0, s>>>(d.npatch, sorted, d.NodeChild, d.NodeParent);
    k_escape<<<blocks_for(2 * (int64_t)d.npatch - 1), kBlock, 0, s>>>(2 * d.npatch - 1, d.NodeChild, d.NodeParent,
                                                                     d.NodeEscape);
}
template <typename T, typename TC>
void launch_refit(const Dev<T, TC>& d, cudaStream_t s) {
    if (d.npatch == 0) return;
    if (d.npatch > 1) cudaMemsetAsync(d.RefitFlag, 0, sizeof(int) * (d.npatch - 1), s);
    k_refit<T><<<blocks_for(d.npatch), kBlock, 0, s>>>(d.npatch, d.LeafPatch, d.PatchBox, d.NodeBox, d.NodeChild,
                                                       d.NodeParent, d.RefitFlag);
}
template <typename T, typename TC>
void launch_traverse(const Dev<T, TC>& d, int64_t* cpt, int64_t* cee, int64_t cap, unsigned long long* count,
                     const SolverConsts& c, cudaStream_t s) {
    if (d.npatch == 0) return;
    const int b = c.trav_block == 64 ? 64 : 128;  // within the kernel's launch bound, whole warps
    k_traverse<T><<<blocks_for(d.npatch, b), b, 0, s>>>(d.npatch, d.PatchBox, d.NodeBox, d.NodeChild, d.NodeEscape,
                                                        d.LeafPatch, d.pStatic, d.pfPtr, d.ppPtr, d.pePtr, d.Pairs,
                                                        cpt, cee, cap, count, d.ErrFlags);
}
template <typename T, typename TC>
void launch_expand(const Dev<T, TC>& d, const int64_t* opt, const int64_t* oee, const SolverConsts& c,
                   cudaStream_t s) {
    if (d.nPairs == 0) return;
    const int b = c.expand_block == 128 ? 128 : kBlock;
    // one thread per pair: each warp expands 32 consecutive pairs
    k_expand<<<blocks_for(d.nPairs, b), b, 0, s>>>(d.nPairs, d.Pairs, d.pfPtr, d.pfIdx, d.ppPtr, d.ppIdx, d.pePtr,
                                                   d.peIdx, d.Faces, d.Edges, opt, oee, d.PT, d.EE);
}
template <typename T, typename TC>
void launch_toi(const Dev<T, TC>& d, Pos<T, TC> X0, Pos<T, TC> X1, const SolverConsts& c, TC* per_pt,
                TC* per_ee, cudaStream_t s) {
    constexpr bool kRel = sizeof(T) == 4 && sizeof(TC) == 8;
    if (c.ccd_mode != 2) {  // the reference's additive CCD
        if (d.nPT > 0)
            k_toi<T, TC, true, kRel><<<grid_cap(d.nPT, kBlock, c.cand_grid), kBlock, 0, s>>>(
                d.nPT, d.PT, X0.x, X1.x, X0.hi, X0.lo, X1.hi, X1.lo, (TC)c.ccd_slack, (TC)c.ccd_eta,
                c.ccd_max_iter, per_pt, d.ToiMin, d.Gate);
        if (d.nEE > 0)
            k_toi<T, TC, false, kRel><<<grid_cap(d.nEE, kBlock, c.cand_grid), kBlock, 0, s>>>(
                d.nEE, d.EE, X0.x, X1.x, X0.hi, X0.lo, X1.hi, X1.lo, (TC)c.ccd_slack, (TC)c.ccd_eta,
                c.ccd_max_iter, per_ee, d.ToiMin, d.Gate);
    }
    if (c.ccd_mode == 1) {  // the FP64 cubic may lower it
        if (d.nPT > 0)
            k_toi_cubic<TC, true, false><<<grid_cap(d.nPT, kBlock, c.cand_grid), kBlock, 0, s>>>(
                d.nPT, d.PT, X0.x, X1.x, c.ccd_slack, per_pt, d.ToiMin, d.Gate);
        if (d.nEE > 0)
            k_toi_cubic<TC, false, false><<<grid_cap(d.nEE, kBlock, c.cand_grid), kBlock, 0, s>>>(
                d.nEE, d.EE, X0.x, X1.x, c.ccd_slack, per_ee, d.ToiMin, d.Gate);
    } else if (c.ccd_mode == 2) {  // the FP64 cubic alone: exact first-contact times
        if (d.nPT > 0)
            k_toi_cubic<TC, true, true><<<grid_cap(d.nPT, kBlock, c.cand_grid), kBlock, 0, s>>>(
                d.nPT, d.PT, X0.x, X1.x, c.ccd_slack, per_pt, d.ToiMin, d.Gate);
        if (d.nEE > 0)
            k_toi_cubic<TC, false, true><<<grid_cap(d.nEE, kBlock, c.cand_grid), kBlock, 0, s>>>(
                d.nEE, d.EE, X0.x, X1.x, c.ccd_slack, per_ee, d.ToiMin, d.Gate);
    }
}
template <typename T, typename TC>
void launch_inst_toi(const Dev<T, TC>& d, const TC* per_pt, const TC* per_ee, const SolverConsts& c, cudaStream_t s) {
    if (d.ninst == 0) return;
    if (d.nPT > 0 && per_pt)
        k_inst_toi<TC><<<grid_cap(d.nPT, kBlock, c.cand_grid), kBlock, 0, s>>>(d.nPT, d.PT, per_pt, d.VInst,
                                                                             d.InstToiMin, d.Gate);
    if (d.nEE > 0 && per_ee)
        k_inst_toi<TC><<<grid_cap(d.nEE, kBlock, c.cand_grid), kBlock, 0, s>>>(d.nEE, d.EE, per_ee, d.VInst,
                                                                             d.InstToiMin, d.Gate);
    k_inst_toi_finalize<TC><<<blocks_for(d.ninst), kBlock, 0, s>>>(d.ninst, d.InstToiMin, d.InstToi, c.toi_scale,
                                                                   d.Gate);
}
template <typename T, typename TC>
void launch_toi_finalize(const Dev<T, TC>& d, const SolverConsts& c, cudaStream_t s) {
    k_toi_finalize<TC><<<1, 1, 0, s>>>(d.ToiMin, d.Toi, c.toi_scale, d.Gate);
}
template <typename T, typename TC>
void launch_contact(const Dev<T, TC>& d, Pos<T, TC> X, const SolverConsts& c, cudaStream_t s) {
    k_contact_clear<T><<<blocks_for(d.ntot), kBlock, 0, s>>>(d.ntot, d.CollDiag, d.CollRhs, d.ActiveCount, d.Gate);
    ContactConsts<TC> cc;
    const T dh = (T)c.dhat;
    cc.dh = (TC)dh;
    cc.dh2 = (TC)(dh * dh);
    cc.kappa = (TC)(T)c.kappa;
    cc.dt = (TC)(T)c.dt;
    constexpr bool kRel = sizeof(T) == 4 && sizeof(TC) == 8;
    if (d.nPT > 0)
        k_contact<T, TC, true, kRel><<<grid_cap(d.nPT, kBlock, c.cand_grid), kBlock, 0, s>>>(d.nPT, d.PT, X.x, X.hi, X.lo, d.CollMass,
                                                                         cc, d.CollDiag, d.CollRhs, d.ActiveCount,
                                                                         d.Gate);
    if (d.nEE > 0)
        k_contact<T, TC, false, kRel><<<grid_cap(d.nEE, kBlock, c.cand_grid), kBlock, 0, s>>>(d.nEE, d.EE, X.x, X.hi, X.lo,
                                                                          d.CollMass, cc, d.CollDiag, d.CollRhs,
                                                                          d.ActiveCount, d.Gate);
}

// ---------------- no-allocation scratch of the per-candidate toi pass ----------------
// File-scope device array: module load reserves it, so the no-allocation stage
// entry needs no cudaMalloc.  Entries [0, n) are written by the toi kernels
// before they are read; nothing in it has to start at zero.
static __device__ __align__(256) double g_toi_scratch[kToiScratchEntries];

cudaError_t toi_scratch(ToiScratch* out) {
    constexpr int kMaxDevices = 64;
    static std::mutex setup;
    static std::mutex locks[kMaxDevices];
    static double* ptrs[kMaxDevices] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> g(setup);
    if (!ptrs[dev]) {  // first call on this device: look the symbol up once
        double* ptr = nullptr;
        e = cudaGetSymbolAddress((void**)&ptr, g_toi_scratch);
        if (e != cudaSuccess) return e;
        ptrs[dev] = ptr;
    }
    out->ptr = ptrs[dev];
    out->entries = kToiScratchEntries;
    out->lock = &locks[dev];
    return cudaSuccess;
}

#define PDIPC_INST_COLL(T, TC)                                                                                \
    template void launch_patch_boxes<T, TC>(const Dev<T, TC>&, const V4<TC>*, const V4<TC>*, const V4<T>*,     \
                                            const V4<T>*, T, cudaStream_t);                                   \
    template void launch_patch_init_boxes<T, TC>(const Dev<T, TC>&, T, cudaStream_t);                         \
    template void launch_morton<T, TC>(const Dev<T, TC>&, T*, unsigned long long*, int*, cudaStream_t);     \
    template void launch_karras<T, TC>(const Dev<T, TC>&, const unsigned long long*, cudaStream_t);           \
    template void launch_refit<T, TC>(const Dev<T, TC>&, cudaStream_t);                                       \
    template void launch_traverse<T, TC>(const Dev<T, TC>&, int64_t*, int64_t*, int64_t, unsigned long long*,  \
                                         const SolverConsts&, cudaStream_t);                                   \
    template void launch_expand<T, TC>(const Dev<T, TC>&, const int64_t*, const int64_t*, const SolverConsts&, \
                                       cudaStream_t);                                                          \
    template void launch_toi<T, TC>(const Dev<T, TC>&, Pos<T, TC>, Pos<T, TC>, const SolverConsts&, TC*,      \
                                    TC*, cudaStream_t);                                                       \
    template void launch_toi_finalize<T, TC>(const Dev<T, TC>&, const SolverConsts&, cudaStream_t);           \
    template void launch_inst_toi<T, TC>(const Dev<T, TC>&, const TC*, const TC*, const SolverConsts&,        \
                                         cudaStream_t);                                                      \
    template void launch_contact<T, TC>(const Dev<T, TC>&, Pos<T, TC>, const SolverConsts&, cudaStream_t);

PDIPC_INST_COLL(float, float)
PDIPC_INST_COLL(double, double)
PDIPC_INST_COLL(float, double)

}  // namespace pdipc
