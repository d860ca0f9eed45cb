// geometry.cuh — closest-point distances, swept-AABB filters and additive CCD
// of the reference (Simulator/PD-IPC/PdIpcGpuFunc.cu:2152-2607), templated on
// the scalar so the same code runs in float (reference arithmetic) or double.
#pragma once

#include "common.cuh"

namespace pdipc {
namespace geo {

template <typename R>
struct P3 {
    R v[3];
};

template <typename R>
__device__ __forceinline__ R dot3(const R* a, const R* b) {
    R s = R(0);
    s += a[0] * b[0];
    s += a[1] * b[1];
    s += a[2] * b[2];
    return s;
}
template <typename R>
__device__ __forceinline__ void sub3(const R* a, const R* b, R* r) {
    r[0] = a[0] - b[0];
    r[1] = a[1] - b[1];
    r[2] = a[2] - b[2];
}
template <typename R>
__device__ __forceinline__ void cross3(const R* a, const R* b, R* r) {
    r[0] = a[1] * b[2] - b[1] * a[2];
    r[1] = a[2] * b[0] - b[2] * a[0];
    r[2] = a[0] * b[1] - b[0] * a[1];
}

// VertexEdgeSqDistance (cu:2155-2175)
template <typename R>
__device__ __forceinline__ R vtx_edge_sq(const R* v, const R* ea, const R* eb, R* r) {
    R va[3], ba[3], d[3];
    sub3(v, ea, va);
    sub3(eb, ea, ba);
    const R vb = dot3(va, ba), bb = dot3(ba, ba);
    if (vb < R(0)) *r = R(0);
    else if (vb > bb) *r = R(1);
    else *r = vb / bb;
    for (int k = 0; k < 3; ++k) d[k] = v[k] - (ea[k] * (R(1) - *r) + eb[k] * *r);
    return dot3(d, d);
}

// EdgeEdgeSqDistance (cu:2177-2237): d = closest(a) - closest(b)
template <typename R>
__device__ __forceinline__ R edge_edge_sq(const R* xi, const R* xj, const R* xa, const R* xb, R* r, R* s, R* d) {
    R xba[3], xji[3], xai[3], tmp[3];
    sub3(xb, xa, xba);
    sub3(xj, xi, xji);
    sub3(xa, xi, xai);
    cross3(xji, xba, d);
    const R nn = dot3(d, d);
    cross3(xai, xji, tmp);
    const R w_aiji = dot3(d, tmp);
    cross3(xai, xba, tmp);
    const R w_aiba = dot3(d, tmp);
    if (nn > R(1e-24f) && w_aiji >= R(0) && w_aiji <= nn && w_aiba >= R(0) && w_aiba <= nn) {
        *r = w_aiba / nn;
        *s = w_aiji / nn;
    } else {
        R best = R(999999999), dd, v;
        if (w_aiba < R(0) && ((dd = vtx_edge_sq(xi, xa, xb, &v)) < best)) { best = dd; *r = R(0); *s = v; }
        if (w_aiba > nn && ((dd = vtx_edge_sq(xj, xa, xb, &v)) < best)) { best = dd; *r = R(1); *s = v; }
        if (w_aiji < R(0) && ((dd = vtx_edge_sq(xa, xi, xj, &v)) < best)) { best = dd; *r = v; *s = R(0); }
        if (w_aiji > nn && ((dd = vtx_edge_sq(xb, xi, xj, &v)) < best)) { best = dd; *r = v; *s = R(1); }
    }
    for (int k = 0; k < 3; ++k) d[k] = xi[k] * (R(1) - *r) + xj[k] * *r - xa[k] * (R(1) - *s) - xb[k] * *s;
    return dot3(d, d);
}

// VertexTriangleDistance (cu:2239-2292): d = x - closest point on the triangle
template <typename R>
__device__ __forceinline__ R vtx_tri(const R* xi, const R* xa, const R* xb, const R* xc, R* ba, R* bb, R* bc, R* d) {
    R xba[3], xca[3], xia[3], tmp[3];
    sub3(xb, xa, xba);
    sub3(xc, xa, xca);
    sub3(xi, xa, xia);
    cross3(xba, xca, d);
    const R nn = dot3(d, d);
    cross3(xia, xca, tmp);
    const R w_iaca = dot3(d, tmp);
    cross3(xba, xia, tmp);
    const R w_baia = dot3(d, tmp);
    if (nn > R(1e-24f) && w_iaca >= R(0) && w_baia >= R(0) && nn - w_iaca - w_baia >= R(0)) {
        *bb = w_iaca / nn;
        *bc = w_baia / nn;
        *ba = R(1) - *bb - *bc;
    } else {
        R best = R(999999999), r, dd;
        if (nn - w_iaca - w_baia < R(0) && ((dd = vtx_edge_sq(xi, xb, xc, &r)) < best)) {
            best = dd; *bb = R(1) - r; *bc = r; *ba = R(0);
        }
        if (w_iaca < R(0) && ((dd = vtx_edge_sq(xi, xa, xc, &r)) < best)) {
            best = dd; *bb = R(0); *bc = r; *ba = R(1) - *bb - *bc;
        }
        if (w_baia < R(0) && ((dd = vtx_edge_sq(xi, xa, xb, &r)) < best)) {
            best = dd; *bb = r; *bc = R(0); *ba = R(1) - *bb - *bc;
        }
    }
    for (int k = 0; k < 3; ++k) d[k] = xi[k] - xa[k] * *ba - xb[k] * *bb - xc[k] * *bc;
    return dot3(d, d);
}

template <typename R>
__device__ __forceinline__ R mn3(R a, R b, R c) { return dmin(dmin(a, b), c); }
template <typename R>
__device__ __forceinline__ R mx3(R a, R b, R c) { return dmax(dmax(a, b), c); }

// point_triangle_ccd_broadphase (cu:2347-2403)
template <typename R>
__device__ __forceinline__ bool pt_ccd_broad(const R (*x)[3], const R (*dx)[3], R dist) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        R tmin = mn3(x[1][k], x[2][k], x[3][k]);
        tmin = mn3(tmin, x[1][k] + dx[1][k], x[2][k] + dx[2][k]);
        tmin = dmin(tmin, x[3][k] + dx[3][k]);
        R tmax = mx3(x[1][k], x[2][k], x[3][k]);
        tmax = mx3(tmax, x[1][k] + dx[1][k], x[2][k] + dx[2][k]);
        tmax = dmax(tmax, x[3][k] + dx[3][k]);
        const R pmin = dmin(x[0][k], x[0][k] + dx[0][k]), pmax = dmax(x[0][k], x[0][k] + dx[0][k]);
        if ((pmin - tmax) > dist || (tmin - pmax) > dist) return false;
    }
    return true;
}
// edge_edge_ccd_broadphase (cu:2426-2457)
template <typename R>
__device__ __forceinline__ bool ee_ccd_broad(const R (*x)[3], const R (*dx)[3], R dist) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        R mina = dmin(x[0][k], x[0][k] + dx[0][k]);
        mina = dmin(mina, x[1][k]);
        mina = dmin(mina, x[1][k] + dx[1][k]);
        R maxa = dmax(x[0][k], x[0][k] + dx[0][k]);
        maxa = dmax(maxa, x[1][k]);
        maxa = dmax(maxa, x[1][k] + dx[1][k]);
        R minb = dmin(x[2][k], x[2][k] + dx[2][k]);
        minb = dmin(minb, x[3][k]);
        minb = dmin(minb, x[3][k] + dx[3][k]);
        R maxb = dmax(x[2][k], x[2][k] + dx[2][k]);
        maxb = dmax(maxb, x[3][k]);
        maxb = dmax(maxb, x[3][k] + dx[3][k]);
        if ((mina - maxb) > dist || (minb - maxa) > dist) return false;
    }
    return true;
}

template <typename R>
__device__ __forceinline__ R sqn(const R* a) { return dot3(a, a); }

// Squared gap between the bounding boxes of points a[0..na) and b[0..nb): a
// lower bound of the squared distance between the primitives they span.
template <typename R, int NA, int NB>
__device__ __forceinline__ R box_gap2(const R (*a)[3], const R (*b)[3]) {
    R g2 = R(0);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        R amin = a[0][k], amax = a[0][k], bmin = b[0][k], bmax = b[0][k];
#pragma unroll
        for (int j = 1; j < NA; ++j) {
            amin = dmin(amin, a[j][k]);
            amax = dmax(amax, a[j][k]);
        }
#pragma unroll
        for (int j = 1; j < NB; ++j) {
            bmin = dmin(bmin, b[j][k]);
            bmax = dmax(bmax, b[j][k]);
        }
        const R sep = dmax(dmax(bmin - amax, amin - bmax), R(0));
        g2 += sep * sep;
    }
    return g2;
}

// True when ccd_pt / ccd_ee below return 1 before computing any distance (no
// relative motion, or the box-gap exit of their first step): the same
// arithmetic as their opening lines, on copies.
template <typename R>
__device__ __forceinline__ bool ccd_pt_trivial(const R (*x)[3], const R (*dx)[3]) {
    R mov[3], d[4][3];
    for (int k = 0; k < 3; ++k) mov[k] = (dx[0][k] + dx[1][k] + dx[2][k] + dx[3][k]) / R(4);
    for (int j = 0; j < 4; ++j)
        for (int k = 0; k < 3; ++k) d[j][k] = dx[j][k] - mov[k];
    R m2 = dmax(sqn(d[1]), sqn(d[2]));
    m2 = dmax(m2, sqn(d[3]));
    const R maxd = dsqrt(sqn(d[0])) + dsqrt(m2);
    return maxd == R(0) || R(0.81) * box_gap2<R, 1, 3>(x, x + 1) > R(4) * maxd * maxd;
}
template <typename R>
__device__ __forceinline__ bool ccd_ee_trivial(const R (*x)[3], const R (*dx)[3]) {
    R mov[3], d[4][3];
    for (int k = 0; k < 3; ++k) mov[k] = (dx[0][k] + dx[1][k] + dx[2][k] + dx[3][k]) / R(4);
    for (int j = 0; j < 4; ++j)
        for (int k = 0; k < 3; ++k) d[j][k] = dx[j][k] - mov[k];
    const R m0 = dmax(sqn(d[0]), sqn(d[1])), m1 = dmax(sqn(d[2]), sqn(d[3]));
    const R maxd = dsqrt(m0) + dsqrt(m1);
    return maxd == R(0) || R(0.81) * box_gap2<R, 2, 2>(x, x + 2) > R(4) * maxd * maxd;
}

// The same exit decided from approximate coordinates: x and dx within eps of
// the exact ones per component.  The motion bound is taken eps_m larger and the
// box gap eps_g smaller (eps_m >= 8 eps, eps_g >= 4 eps cover the mean
// subtraction, the norms and the box corners), so a true result implies the
// exact test's.
template <typename R, bool kPT>
__device__ __forceinline__ bool ccd_trivial_approx(const R (*x)[3], const R (*dx)[3], R eps_g, R eps_m) {
    R mov[3], d[4][3];
    for (int k = 0; k < 3; ++k) mov[k] = (dx[0][k] + dx[1][k] + dx[2][k] + dx[3][k]) / R(4);
    for (int j = 0; j < 4; ++j)
        for (int k = 0; k < 3; ++k) d[j][k] = dx[j][k] - mov[k];
    R maxd;
    if (kPT) {
        R m2 = dmax(sqn(d[1]), sqn(d[2]));
        m2 = dmax(m2, sqn(d[3]));
        maxd = dsqrt(sqn(d[0])) + dsqrt(m2);
    } else {
        maxd = dsqrt(dmax(sqn(d[0]), sqn(d[1]))) + dsqrt(dmax(sqn(d[2]), sqn(d[3])));
    }
    maxd += eps_m;
    const R gap = dsqrt(kPT ? box_gap2<R, 1, 3>(x, x + 1) : box_gap2<R, 2, 2>(x, x + 2)) - eps_g;
    return gap > R(0) && R(0.81) * gap * gap > R(4) * maxd * maxd;
}

// ccdVertexTriangleToi (cu:2460-2529): additive CCD, at most max_iter conservative steps
template <typename R>
__device__ R ccd_pt(R (*x)[3], R (*dx)[3], R eta, int max_iter) {
    R mov[3];
    for (int k = 0; k < 3; ++k) mov[k] = (dx[0][k] + dx[1][k] + dx[2][k] + dx[3][k]) / R(4);
    for (int j = 0; j < 4; ++j)
        for (int k = 0; k < 3; ++k) dx[j][k] -= mov[k];
    R m2 = dmax(sqn(dx[1]), sqn(dx[2]));
    m2 = dmax(m2, sqn(dx[3]));
    const R maxd = dsqrt(sqn(dx[0])) + dsqrt(m2);
    if (maxd == R(0)) return R(1);
    // The first conservative step below returns 1 when 0.9 d > maxd.  The box
    // gap bounds d from below: when even half of it clears maxd, return that 1
    // without the distance (the factor 2 is far above the distance's rounding).
    if (R(0.81) * box_gap2<R, 1, 3>(x, x + 1) > R(4) * maxd * maxd) return R(1);
    R a, b, c, dd[3];
    R d2 = vtx_tri(x[0], x[1], x[2], x[3], &a, &b, &c, dd);
    R dc = dsqrt(d2);
    const R gap = eta * dc;
    R toc = R(0);
    for (int it = 0; it < max_iter; ++it) {
        const R lb = R(0.9) * d2 / (dc * maxd);
        // at it == 0 toc is 0, so the gap test below cannot fire and a first
        // bound above 1 returns 1 whatever the distance after the advance
        if (it == 0 && lb > R(1)) return R(1);
        for (int j = 0; j < 4; ++j)
            for (int k = 0; k < 3; ++k) x[j][k] += lb * dx[j][k];
        d2 = vtx_tri(x[0], x[1], x[2], x[3], &a, &b, &c, dd);
        dc = dsqrt(d2);
        if (toc != R(0) && dc < gap) break;
        toc += lb;
        if (toc > R(1)) {
            toc = R(1);
            break;
        }
    }
    return toc;
}

template <typename R>
__device__ __forceinline__ R pp_min(const R (*x)[3]) {
    auto d2 = [](const R* a, const R* b) {
        return (a[0] - b[0]) * (a[0] - b[0]) + (a[1] - b[1]) * (a[1] - b[1]) + (a[2] - b[2]) * (a[2] - b[2]);
    };
    R r = d2(x[0], x[2]);
    r = dmin(d2(x[0], x[3]), r);
    r = dmin(d2(x[1], x[2]), r);
    r = dmin(d2(x[1], x[3]), r);
    return r;
}

// ccdEdgeEdgeToi (cu:2531-2607): parallel edges fall back to point-point distances
template <typename R>
__device__ R ccd_ee(R (*x)[3], R (*dx)[3], R eta, int max_iter) {
    R mov[3];
    for (int k = 0; k < 3; ++k) mov[k] = (dx[0][k] + dx[1][k] + dx[2][k] + dx[3][k]) / R(4);
    for (int j = 0; j < 4; ++j)
        for (int k = 0; k < 3; ++k) dx[j][k] -= mov[k];
    const R m0 = dmax(sqn(dx[0]), sqn(dx[1])), m1 = dmax(sqn(dx[2]), sqn(dx[3]));
    const R maxd = dsqrt(m0) + dsqrt(m1);
    if (maxd == R(0)) return R(1);
    if (R(0.81) * box_gap2<R, 2, 2>(x, x + 2) > R(4) * maxd * maxd) return R(1);  // as in ccd_pt
    R r, s, dd[3];
    R d2 = edge_edge_sq(x[0], x[1], x[2], x[3], &r, &s, dd);
    R f = d2;
    if (f <= R(0)) {
        d2 = pp_min(x);
        f = d2;
    }
    R dc = dsqrt(d2);
    const R gap = eta * f / dc;
    R toc = R(0);
    for (int it = 0; it < max_iter; ++it) {
        const R lb = R(0.9) * f / (dc * maxd);
        if (it == 0 && lb > R(1)) return R(1);  // as in ccd_pt
        for (int j = 0; j < 4; ++j)
            for (int k = 0; k < 3; ++k) x[j][k] += lb * dx[j][k];
        d2 = edge_edge_sq(x[0], x[1], x[2], x[3], &r, &s, dd);
        f = d2;
        if (f <= R(0)) {
            d2 = pp_min(x);
            f = d2;
        }
        dc = dsqrt(d2);
        if (toc != R(0) && (f / dc) < gap) break;
        toc += lb;
        if (toc > R(1)) {
            toc = R(1);
            break;
        }
    }
    return toc;
}

}  // namespace geo
}  // namespace pdipc
