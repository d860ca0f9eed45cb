// penalty_kernels.cu — the reference's penalty / discrete-collision contact path
// (PdIpcGpuFunc.cu:2933-3740).  The reference declares these kernels beside the
// IPC path but its step never calls them (PdIpcSimulator.cpp only allocates the
// zero force buffer that predictiveKernel reads), so here they are stages a
// caller runs on a context's tables: the candidate lists of the last broad
// phase, the faces, masses, gravity and pins.  State arithmetic is in the state
// scalar TC (double in the FP64 and mixed modes); forces and hit counts
// accumulate with atomics, as in the reference.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "geometry.cuh"
#include "kernels.cuh"

namespace pdipc {

namespace {

constexpr int kPenBlock = 256;
inline int pen_blocks(int64_t n) {
    return (int)std::min<int64_t>(std::max<int64_t>(1, (n + kPenBlock - 1) / kPenBlock), 152 * 16);
}

template <typename TC>
__device__ __forceinline__ void add_force(V4<TC>* F, int i, TC fx, TC fy, TC fz) {
    atomicAdd(&F[i].x, fx);
    atomicAdd(&F[i].y, fy);
    atomicAdd(&F[i].z, fz);
}

// prediticeDCPositionKernel (cu:2933-2981): sn = x + dt (v + dt m^-1 f_gravity);
// a pinned vertex keeps x and gets v = 0.
template <typename T, typename TC>
__global__ void k_pen_predict(int n, const V4<TC>* __restrict__ X, V4<TC>* __restrict__ V,
                              const V4<T>* __restrict__ Grav, const T* __restrict__ InvMass,
                              const int* __restrict__ PinFlag, TC dt, V4<TC>* __restrict__ Sn) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const V4<TC> x = X[i];
    if (PinFlag[i] != -1) {
        V[i] = V4<TC>{TC(0), TC(0), TC(0), TC(0)};
        Sn[i] = x;
        return;
    }
    const TC m = (TC)InvMass[i] * dt;
    const V4<TC> v = V[i];
    const V4<T> g = Grav[i];
    const TC vx = (v.x + m * (TC)g.x) * dt, vy = (v.y + m * (TC)g.y) * dt, vz = (v.z + m * (TC)g.z) * dt;
    Sn[i] = V4<TC>{x.x + vx, x.y + vy, x.z + vz, TC(0)};
}

// computePenaltyForceKernal (cu:3013-3138): a candidate sharing no vertex whose
// swept boxes meet within 1e-4 and whose additive CCD time of impact from x0
// along d is below 1 is pushed apart at x0 + d with stiffness * distance along
// the (unnormalised) closest-point vector: point-triangle f = n d k / 3, -3 f on
// the point and f on each face vertex; edge-edge f = n d k / 2, -f on the first
// edge and f on the second.  Every vertex of such a pair counts one hit.
template <typename TC, bool kPT>
__global__ void __launch_bounds__(kPenBlock) k_pen_ccd(int64_t n, const int4* __restrict__ cand,
                                                       const V4<TC>* __restrict__ X0, const V4<TC>* __restrict__ D,
                                                       TC k, TC eta, int max_iter, V4<TC>* __restrict__ F,
                                                       int* __restrict__ times) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        const int4 c = cand[t];
        const int ids[4] = {c.x, c.y, c.z, c.w};
        if (kPT ? (c.x == c.y || c.x == c.z || c.x == c.w) : (c.x == c.z || c.x == c.w || c.y == c.z || c.y == c.w))
            continue;
        TC x[4][3], dx[4][3];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const V4<TC> a = ld4(X0, ids[j]), b = ld4(D, ids[j]);
            x[j][0] = a.x;
            x[j][1] = a.y;
            x[j][2] = a.z;
            dx[j][0] = b.x;
            dx[j][1] = b.y;
            dx[j][2] = b.z;
        }
        if (!(kPT ? geo::pt_ccd_broad<TC>(x, dx, TC(1e-4)) : geo::ee_ccd_broad<TC>(x, dx, TC(1e-4)))) continue;
        const TC toi = kPT ? geo::ccd_pt<TC>(x, dx, eta, max_iter) : geo::ccd_ee<TC>(x, dx, eta, max_iter);
        if (!(toi < TC(1))) continue;
        TC tx[4][3];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const V4<TC> a = ld4(X0, ids[j]), b = ld4(D, ids[j]);
            tx[j][0] = a.x + b.x;
            tx[j][1] = a.y + b.y;
            tx[j][2] = a.z + b.z;
        }
        TC dir[3], f[3];
        if (kPT) {
            TC ba, bb, bc;
            const TC dist = dsqrt(geo::vtx_tri<TC>(tx[0], tx[1], tx[2], tx[3], &ba, &bb, &bc, dir));
            for (int q = 0; q < 3; ++q) f[q] = dir[q] * dist * k / TC(3);
            add_force(F, ids[0], -f[0] * TC(3), -f[1] * TC(3), -f[2] * TC(3));
            add_force(F, ids[1], f[0], f[1], f[2]);
            add_force(F, ids[2], f[0], f[1], f[2]);
            add_force(F, ids[3], f[0], f[1], f[2]);
        } else {
            TC r, s;
            const TC dist = dsqrt(geo::edge_edge_sq<TC>(tx[0], tx[1], tx[2], tx[3], &r, &s, dir));
            for (int q = 0; q < 3; ++q) f[q] = dir[q] * dist * k / TC(2);
            add_force(F, ids[0], -f[0], -f[1], -f[2]);
            add_force(F, ids[1], -f[0], -f[1], -f[2]);
            add_force(F, ids[2], f[0], f[1], f[2]);
            add_force(F, ids[3], f[0], f[1], f[2]);
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) atomicAdd(times + ids[j], 1);
    }
}

// applyPenaltyForceForFloorKernal (cu:3248-3271): a simulated vertex below
// y = 0 gets the force (0, -y k, 0) and one hit (assigned, not added).
template <typename TC>
__global__ void k_pen_floor(int n, const V4<TC>* __restrict__ X, TC k, V4<TC>* __restrict__ F,
                            int* __restrict__ times) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const TC y = X[i].y;
    if (y < TC(0)) {
        F[i] = V4<TC>{TC(0), -y * k, TC(0), TC(0)};
        times[i] = 1;
    }
}

template <typename TC>
__device__ __forceinline__ TC dot3v(const TC* a, const TC* b) {
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}
template <typename TC>
__device__ __forceinline__ void cross3v(const TC* a, const TC* b, TC* r) {
    r[0] = a[1] * b[2] - a[2] * b[1];
    r[1] = a[2] * b[0] - a[0] * b[2];
    r[2] = a[0] * b[1] - a[1] * b[0];
}
// project6 (cu:3371-3389): do the projections of the two triangles on the axis overlap?
template <typename TC>
__device__ __forceinline__ bool overlap_on(const TC* ax, const TC (*p)[3], const TC (*q)[3]) {
    const TC P1 = dot3v(ax, p[0]), P2 = dot3v(ax, p[1]), P3 = dot3v(ax, p[2]);
    const TC Q1 = dot3v(ax, q[0]), Q2 = dot3v(ax, q[1]), Q3 = dot3v(ax, q[2]);
    const TC mx1 = geo::mx3(P1, P2, P3), mn1 = geo::mn3(P1, P2, P3);
    const TC mx2 = geo::mx3(Q1, Q2, Q3), mn2 = geo::mn3(Q1, Q2, Q3);
    return !(mn1 > mx2) && !(mn2 > mx1);
}
// triContact (cu:3391-3468): separating-axis test of two triangles over the two
// normals, the nine edge-edge cross products and the six in-plane edge normals,
// in coordinates relative to the first triangle's first vertex.
template <typename TC>
__device__ bool tri_contact(const TC (*A)[3], const TC (*B)[3]) {
    TC p[3][3], q[3][3];
    for (int j = 0; j < 3; ++j)
        for (int k = 0; k < 3; ++k) {
            p[j][k] = A[j][k] - A[0][k];
            q[j][k] = B[j][k] - A[0][k];
        }
    TC e[3][3], f[3][3];
    for (int k = 0; k < 3; ++k) {
        e[0][k] = p[1][k] - p[0][k];
        e[1][k] = p[2][k] - p[1][k];
        e[2][k] = p[0][k] - p[2][k];
        f[0][k] = q[1][k] - q[0][k];
        f[1][k] = q[2][k] - q[1][k];
        f[2][k] = q[0][k] - q[2][k];
    }
    TC n1[3], m1[3], ax[3];
    cross3v(e[0], e[1], n1);
    cross3v(f[0], f[1], m1);
    if (!overlap_on(n1, p, q)) return false;
    if (!overlap_on(m1, p, q)) return false;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            cross3v(e[a], f[b], ax);
            if (!overlap_on(ax, p, q)) return false;
        }
    for (int a = 0; a < 3; ++a) {
        cross3v(e[a], n1, ax);
        if (!overlap_on(ax, p, q)) return false;
    }
    for (int b = 0; b < 3; ++b) {
        cross3v(f[b], m1, ax);
        if (!overlap_on(ax, p, q)) return false;
    }
    return true;
}
template <typename TC>
__device__ __forceinline__ void unit_normal(const TC (*T)[3], TC* n) {
    TC a[3], b[3];
    for (int k = 0; k < 3; ++k) {
        a[k] = T[1][k] - T[0][k];
        b[k] = T[2][k] - T[0][k];
    }
    cross3v(a, b, n);
    const TC len = dsqrt(dot3v(n, n));
    for (int k = 0; k < 3; ++k) n[k] /= len;
}
// Each vertex of triangle P behind the plane of Q (through Q's second vertex,
// projectToTriangle cu:3470-3485) is pushed out along Q's normal with
// stiffness * depth; Q's vertices take -1/3 of that force each.
template <typename TC>
__device__ __forceinline__ void push_out(const int* pv, const TC (*P)[3], const int* qv, const TC (*Q)[3],
                                         const TC* nq, TC k, V4<TC>* F, int* times) {
    for (int j = 0; j < 3; ++j) {
        TC w[3], dir[3];
        for (int c = 0; c < 3; ++c) w[c] = P[j][c] - Q[1][c];
        const TC cc = dot3v(w, nq);
        for (int c = 0; c < 3; ++c) dir[c] = cc * nq[c];
        const TC len = dsqrt(dot3v(dir, dir));
        for (int c = 0; c < 3; ++c) dir[c] /= len;
        if (dot3v(dir, nq) < TC(0)) {
            const TC f0 = nq[0] * len * k, f1 = nq[1] * len * k, f2 = nq[2] * len * k;
            add_force(F, pv[j], f0, f1, f2);
            for (int m = 0; m < 3; ++m) add_force(F, qv[m], -f0 / TC(3), -f1 / TC(3), -f2 / TC(3));
            atomicAdd(times + pv[j], 1);
            for (int m = 0; m < 3; ++m) atomicAdd(times + qv[m], 1);
        }
    }
}

// computeDcdPenaltyForceKernal (cu:3487-3688) over caller-supplied face pairs:
// pairs sharing no vertex that intersect push each other's vertices out; a
// triangle's own vertices move only if its first vertex is simulated; two faces
// of the same model use the self stiffness.
template <typename TC>
__global__ void __launch_bounds__(kPenBlock) k_pen_dcd(int64_t n, const int2* __restrict__ pairs,
                                                       const int4* __restrict__ Faces, const int* __restrict__ model,
                                                       int nsim, const V4<TC>* __restrict__ X, TC k, TC kself,
                                                       V4<TC>* __restrict__ F, int* __restrict__ times) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        const int2 pr = pairs[t];
        const int4 fa = Faces[pr.x], fb = Faces[pr.y];
        const int av[3] = {fa.x, fa.y, fa.z}, bv[3] = {fb.x, fb.y, fb.z};
        bool shared = false;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) shared |= av[i] == bv[j];
        if (shared) continue;
        TC A[3][3], B[3][3];
        for (int j = 0; j < 3; ++j) {
            const V4<TC> a = ld4(X, av[j]), b = ld4(X, bv[j]);
            A[j][0] = a.x;
            A[j][1] = a.y;
            A[j][2] = a.z;
            B[j][0] = b.x;
            B[j][1] = b.y;
            B[j][2] = b.z;
        }
        if (!tri_contact<TC>(A, B)) continue;
        const TC stiff = model[av[0]] == model[bv[0]] ? kself : k;
        TC na[3], nb[3];
        unit_normal<TC>(A, na);
        unit_normal<TC>(B, nb);
        if (av[0] < nsim) push_out<TC>(av, A, bv, B, nb, stiff, F, times);
        if (bv[0] < nsim) push_out<TC>(bv, B, av, A, na, stiff, F, times);
    }
}

// uniformPenaltyForceKernal (cu:3140-3195): the force of a hit vertex is averaged
// over its hits, minus damping * v; its velocity keeps 0.9 of the part across
// the averaged force and -0.4 of the part along it.
template <typename TC>
__global__ void k_pen_uniform(int n, V4<TC>* __restrict__ F, const int* __restrict__ times, TC damping,
                              V4<TC>* __restrict__ V) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int h = times[i];
    if (h == 0) return;
    const V4<TC> f4 = F[i];
    TC f[3] = {f4.x / (TC)h, f4.y / (TC)h, f4.z / (TC)h};
    const V4<TC> v4 = V[i];
    const TC v[3] = {v4.x, v4.y, v4.z};
    F[i] = V4<TC>{f[0] - damping * v[0], f[1] - damping * v[1], f[2] - damping * v[2], TC(0)};
    const TC len = dsqrt(dot3v(f, f));
    for (int k = 0; k < 3; ++k) f[k] /= len;
    const TC cc = dot3v(v, f);
    TC vn[3], vt[3];
    for (int k = 0; k < 3; ++k) {
        vn[k] = cc * f[k];
        vt[k] = v[k] - vn[k];
        vn[k] *= TC(-0.4);
        vt[k] = vt[k] * TC(0.9);
    }
    V[i] = V4<TC>{vn[0] + vt[0], vn[1] + vt[1], vn[2] + vt[2], TC(0)};
}

}  // namespace

template <typename T, typename TC>
void launch_pen_predict(const Dev<T, TC>& d, const V4<TC>* X, V4<TC>* V, TC dt, V4<TC>* Sn, cudaStream_t s) {
    if (d.nsim == 0) return;
    k_pen_predict<T, TC><<<pen_blocks(d.nsim), kPenBlock, 0, s>>>(d.nsim, X, V, d.Grav, d.InvMass, d.PinFlag, dt,
                                                                   Sn);
}

template <typename T, typename TC>
void launch_pen_ccd(const Dev<T, TC>& d, const V4<TC>* X0, const V4<TC>* D, TC k, TC eta, int max_iter,
                    V4<TC>* F, int* times, cudaStream_t s) {
    if (d.nPT > 0)
        k_pen_ccd<TC, true><<<pen_blocks(d.nPT), kPenBlock, 0, s>>>(d.nPT, d.PT, X0, D, k, eta, max_iter, F, times);
    if (d.nEE > 0)
        k_pen_ccd<TC, false><<<pen_blocks(d.nEE), kPenBlock, 0, s>>>(d.nEE, d.EE, X0, D, k, eta, max_iter, F, times);
}

template <typename T, typename TC>
void launch_pen_floor(const Dev<T, TC>& d, const V4<TC>* X, TC k, V4<TC>* F, int* times, cudaStream_t s) {
    if (d.nsim == 0) return;
    k_pen_floor<TC><<<pen_blocks(d.nsim), kPenBlock, 0, s>>>(d.nsim, X, k, F, times);
}

template <typename T, typename TC>
void launch_pen_dcd(const Dev<T, TC>& d, const int2* pairs, int64_t n, const int* model, const V4<TC>* X, TC k,
                    TC kself, V4<TC>* F, int* times, cudaStream_t s) {
    if (n <= 0) return;
    k_pen_dcd<TC><<<pen_blocks(n), kPenBlock, 0, s>>>(n, pairs, d.Faces, model, d.nsim, X, k, kself, F, times);
}

template <typename T, typename TC>
void launch_pen_uniform(const Dev<T, TC>& d, V4<TC>* F, const int* times, TC damping, V4<TC>* V, cudaStream_t s) {
    if (d.nsim == 0) return;
    k_pen_uniform<TC><<<pen_blocks(d.nsim), kPenBlock, 0, s>>>(d.nsim, F, times, damping, V);
}

#define PDIPC_INST_PEN(T, TC)                                                                                     \
    template void launch_pen_predict<T, TC>(const Dev<T, TC>&, const V4<TC>*, V4<TC>*, TC, V4<TC>*, cudaStream_t); \
    template void launch_pen_ccd<T, TC>(const Dev<T, TC>&, const V4<TC>*, const V4<TC>*, TC, TC, int, V4<TC>*,      \
                                        int*, cudaStream_t);                                                       \
    template void launch_pen_floor<T, TC>(const Dev<T, TC>&, const V4<TC>*, TC, V4<TC>*, int*, cudaStream_t);      \
    template void launch_pen_dcd<T, TC>(const Dev<T, TC>&, const int2*, int64_t, const int*, const V4<TC>*, TC, TC, \
                                        V4<TC>*, int*, cudaStream_t);                                              \
    template void launch_pen_uniform<T, TC>(const Dev<T, TC>&, V4<TC>*, const int*, TC, V4<TC>*, cudaStream_t);

PDIPC_INST_PEN(float, float)
PDIPC_INST_PEN(double, double)
PDIPC_INST_PEN(float, double)

}  // namespace pdipc
