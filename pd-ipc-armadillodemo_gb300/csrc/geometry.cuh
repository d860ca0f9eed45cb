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

// ---------------- FP64 coplanarity-cubic CCD (optional, ccd_mode 1) ----------------
// Four points moving linearly over the step are coplanar where
// f(t) = u1(t) . (u2(t) x u3(t)) = 0, u_k(t) = (x_k - x_0) + t (d_k - d_0): a
// cubic in t (Provot's vertex-face / edge-edge coplanarity test).  Its roots
// in [0, 1] are found by splitting [0, 1] at the roots of f' (monotone pieces)
// and bisecting every piece that changes sign to full precision; at each root,
// in increasing order, the primitives are tested for actual contact (the
// point inside the triangle, the two edges crossing), with a relative
// tolerance that errs toward contact.  The first root that passes is the time
// of impact, else 1.  It can only lower the additive CCD's result, which
// stops after a fixed number of iterations.  x: positions relative to x_0,
// d: displacements; PT: x_0 the point, x_1..3 the triangle; EE: edges
// (x_0, x_1) and (x_2, x_3).
__device__ __forceinline__ double cubic_eval(const double (&c)[4], double t) {
    return ((c[3] * t + c[2]) * t + c[1]) * t + c[0];
}

template <bool kPT>
__device__ __forceinline__ bool touching_at(const double (*x)[3], const double (*d)[3], double t, double tol) {
    double p[4][3];
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int k = 0; k < 3; ++k) p[j][k] = x[j][k] + t * d[j][k];
    if (kPT) {
        double e1[3], e2[3], n[3];
        sub3(p[2], p[1], e1);
        sub3(p[3], p[1], e2);
        cross3(e1, e2, n);
        const double nn = dot3(n, n);
        if (!(nn > 0.0)) return false;
        double a[3], b[3], c[3], q[3];
        sub3(p[1], p[0], a);
        sub3(p[2], p[0], b);
        sub3(p[3], p[0], c);
        cross3(b, c, q);
        const double wa = dot3(q, n) / nn;
        cross3(c, a, q);
        const double wb = dot3(q, n) / nn;
        cross3(a, b, q);
        const double wc = dot3(q, n) / nn;
        return wa >= -tol && wb >= -tol && wc >= -tol;
    } else {
        double ea[3], eb[3], w[3];
        sub3(p[1], p[0], ea);
        sub3(p[3], p[2], eb);
        sub3(p[0], p[2], w);
        const double aa = dot3(ea, ea), bb = dot3(eb, eb), ab = dot3(ea, eb);
        const double den = aa * bb - ab * ab;
        if (!(den > 1e-24 * aa * bb)) return false;  // parallel edges: left to the additive CCD
        const double wa = dot3(w, ea), wb = dot3(w, eb);
        const double s = (ab * wb - bb * wa) / den, u = (aa * wb - ab * wa) / den;
        return s >= -tol && s <= 1.0 + tol && u >= -tol && u <= 1.0 + tol;
    }
}

template <bool kPT>
__device__ double ccd_cubic(const double (*x)[3], const double (*d)[3]) {
    double u0[3][3], u1[3][3];
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            u0[k][a] = x[k + 1][a] - x[0][a];
            u1[k][a] = d[k + 1][a] - d[0][a];
        }
    double c[4];
    {
        double bc[3], t1[3], t2[3], t3[3];
        cross3(u0[1], u0[2], bc);
        c[0] = dot3(u0[0], bc);
        cross3(u1[1], u0[2], t1);
        cross3(u0[1], u1[2], t2);
        c[1] = dot3(u1[0], bc) + dot3(u0[0], t1) + dot3(u0[0], t2);
        cross3(u1[1], u1[2], t3);
        c[2] = dot3(u1[0], t1) + dot3(u1[0], t2) + dot3(u0[0], t3);
        c[3] = dot3(u1[0], t3);
    }
    double scale = 0.0;
#pragma unroll
    for (int k = 0; k < 3; ++k)
        scale = fmax(scale, fmax(sqrt(dot3(u0[k], u0[k])), sqrt(dot3(u1[k], u1[k]))));
    const double s3 = scale * scale * scale;
    if (!(s3 > 0.0) || !(fabs(c[0]) + fabs(c[1]) + fabs(c[2]) + fabs(c[3]) > 1e-14 * s3))
        return 1.0;  // no motion, or coplanar throughout: left to the additive CCD
    // split points: 0, the roots of f' = 3 c3 t^2 + 2 c2 t + c1 inside (0, 1), 1
    double br[4] = {0.0, 1.0, 1.0, 1.0};
    int nb = 1;
    {
        const double A = 3.0 * c[3], B = 2.0 * c[2], C = c[1];
        double r0 = 2.0, r1 = 2.0;
        if (fabs(A) > 1e-300) {
            const double disc = B * B - 4.0 * A * C;
            if (disc >= 0.0) {
                const double q = -0.5 * (B + copysign(sqrt(disc), B));
                r0 = q / A;
                r1 = q != 0.0 ? C / q : r0;
            }
        } else if (fabs(B) > 1e-300) {
            r0 = -C / B;
        }
        if (r0 > r1) {
            const double tt = r0;
            r0 = r1;
            r1 = tt;
        }
        if (r0 > 0.0 && r0 < 1.0) br[nb++] = r0;
        if (r1 > 0.0 && r1 < 1.0 && r1 != r0) br[nb++] = r1;
        br[nb] = 1.0;
    }
    const double tol = 1e-6;
    for (int s = 0; s < nb; ++s) {
        double lo = br[s], hi = br[s + 1];
        double flo = cubic_eval(c, lo), fhi = cubic_eval(c, hi);
        double root;
        if (flo == 0.0) {
            root = lo;
        } else if ((flo < 0.0) != (fhi < 0.0) || fhi == 0.0) {
            for (int it = 0; it < 64 && hi - lo > 0.0; ++it) {  // to the last bit of [lo, hi]
                const double mid = 0.5 * (lo + hi);
                if (mid <= lo || mid >= hi) break;
                const double fm = cubic_eval(c, mid);
                if ((fm < 0.0) == (flo < 0.0) && fm != 0.0) {
                    lo = mid;
                    flo = fm;
                } else {
                    hi = mid;
                }
            }
            root = lo;  // the side before the crossing
        } else {
            continue;
        }
        if (touching_at<kPT>(x, d, root, tol) || touching_at<kPT>(x, d, hi, tol)) return root;
    }
    return 1.0;
}

}  // namespace geo
}  // namespace pdipc
