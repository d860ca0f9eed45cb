// adjoint_kernels.cu — discrete adjoint of the contact-free projective-dynamics
// step in the plain FP64 form (the reference has no adjoint; the forward kernels
// differentiated here are those of pd_kernels.cu, which replace
// PdIpcGpuFunc.cu:88-147, 627-790 and 1041-1346).
//
// Forward, per local-global iteration from x (positions at its start):
//   q_i = sum_s lbo_s x_nbr(s);  a_i = q_i c_i / |q_i|  (|q_i| >= 1e-10)
//   r_i = rhs0_i + sum_{s>b} k_i rest_s d_s / |d_s| + bend_b a_i + sum_{s>b} bendT_s a_nbr(s) + pin_i
//   S(z) = (1-w) z + w D^-1 (N z + r)
//   X1 = S(S(x));  X_{t+1} = om_t S(S(X_t)) + (1 - om_t) X_{t-1}
// with d_s = x_i - x_nbr(s), N_ij = k_i (spring neighbours) + bending terms,
// D_i = deg_i k_i + (bending + pin) + m_i/dt^2.  The reverse pass runs the same
// recurrence backwards: each sweep's adjoint is J^T u = (1-w) u + N^T (w D^-1 u)
// on the transposed matrix values, the right-hand side collects w D^-1 of the
// sum of every sweep's output adjoint, and the local step's adjoint is a
// gather over each vertex's own stencil (springs, the curvature normalisation
// and the transposed LBO weights).  The stretch-stiffness gradient is per
// vertex (the Strain table): k_i enters r_i, row i of N and D_i.
//
// One thread per vertex everywhere; nothing accumulates across threads, so the
// results do not depend on scheduling.
#include <type_traits>

#include "kernels.cuh"
#include "svd3.cuh"

namespace pdipc {

namespace {

constexpr int kBlock = 256;

inline int blocks_for(int n, int b = kBlock) { return std::max(1, (n + b - 1) / b); }

template <typename T>
__device__ __forceinline__ T dot3(const V4<T>& a, const V4<T>& b) {
    return a.x * b.x + a.y * b.y + a.z * b.z;
}

// lLboT[s] for slot s of row m pointing at j: the LBO weight of row j at m (the
// self slot keeps its own weight); NTval[e] for SELL entry e = (row i, column j):
// N_ji, found in row j (0 for padding and for entries whose mirror is absent).
template <typename T>
__global__ void k_adj_tables(int nsim, int nslice, const int* __restrict__ lPtr, const int* __restrict__ lNbr,
                             const T* __restrict__ lLbo, const int* __restrict__ sOff, const int* __restrict__ sLen,
                             const int* __restrict__ sCol, const T* __restrict__ sVal, T* __restrict__ lLboT,
                             T* __restrict__ NTval) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nsim) {
        const int b = lPtr[i], e = lPtr[i + 1];
        lLboT[b] = lLbo[b];
        for (int s = b + 1; s < e; ++s) {
            const int j = lNbr[s];
            T v = T(0);
            for (int t = lPtr[j] + 1; t < lPtr[j + 1]; ++t)
                if (lNbr[t] == i) {
                    v = lLbo[t];
                    break;
                }
            lLboT[s] = v;
        }
    }
    if (i >= nslice * 32) return;
    const int sl = i >> 5, lane = i & 31;
    const int base = sOff[sl] + lane, len = sLen[sl];
    for (int k = 0; k < len; ++k) {
        const int at = base + 32 * k;
        const int j = sCol[at];
        T v = T(0);
        if (i < nsim && j != i && sVal[at] != T(0)) {
            const int bj = sOff[j >> 5] + (j & 31), lj = sLen[j >> 5];
            for (int t = 0; t < lj; ++t)
                if (sCol[bj + 32 * t] == i) {
                    v = sVal[bj + 32 * t];
                    break;
                }
        }
        NTval[at] = v;
    }
}

// Adjoint of one sweep S at input z, output adjoint u = scale * in:
//   out (= or +=) J^T u;  rho += u;  kbar_i += u_i . dS_i/dk_i;
// other (if set) += (1 - scale) in: the Chebyshev step's term on X_{t-1}.
template <typename T>
__global__ void __launch_bounds__(kBlock) k_adj_sweep(
    int nsim, T relax, T scale, const V4<T>* __restrict__ in, V4<T>* __restrict__ other,
    const V4<T>* __restrict__ z, V4<T>* __restrict__ out, int accumulate, V4<T>* __restrict__ rho,
    T* __restrict__ kbar, const V4<T>* __restrict__ Rhs, const T* __restrict__ InvD, const int* __restrict__ sOff,
    const int* __restrict__ sLen, const int* __restrict__ sCol, const T* __restrict__ sVal,
    const T* __restrict__ NTval, const int* __restrict__ lPtr, const int* __restrict__ lNbr) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nsim) return;
    const V4<T> a = in[i];
    const V4<T> u{scale * a.x, scale * a.y, scale * a.z, T(0)};
    const T idi = InvD[i];
    const int sl = i >> 5, base = sOff[sl] + (i & 31), len = sLen[sl];
    T j0 = T(0), j1 = T(0), j2 = T(0);  // sum_j N_ji w D_j^-1 u_j
    T n0 = T(0), n1 = T(0), n2 = T(0);  // (N z)_i
    for (int k = 0; k < len; ++k) {
        const int at = base + 32 * k;
        const int j = sCol[at];
        const T c = NTval[at] * (relax * InvD[j] * scale);
        const V4<T> aj = in[j];
        j0 += c * aj.x;
        j1 += c * aj.y;
        j2 += c * aj.z;
        const T v = sVal[at];
        const V4<T> zj = z[j];
        n0 += v * zj.x;
        n1 += v * zj.y;
        n2 += v * zj.z;
    }
    const int b = lPtr[i], e = lPtr[i + 1];
    T s0 = T(0), s1 = T(0), s2 = T(0);  // sum of the spring neighbours' z
    for (int s = b + 1; s < e; ++s) {
        const V4<T> zj = z[lNbr[s]];
        s0 += zj.x;
        s1 += zj.y;
        s2 += zj.z;
    }
    const V4<T> r = Rhs[i];
    const T dg = T(e - b - 1) * idi;
    const V4<T> g{s0 - dg * (n0 + r.x), s1 - dg * (n1 + r.y), s2 - dg * (n2 + r.z), T(0)};
    kbar[i] += relax * idi * dot3(u, g);
    V4<T> p = rho[i];
    rho[i] = V4<T>{p.x + u.x, p.y + u.y, p.z + u.z, T(0)};
    if (other) {
        const T f = T(1) - scale;
        const V4<T> o = other[i];
        other[i] = V4<T>{o.x + f * a.x, o.y + f * a.y, o.z + f * a.z, T(0)};
    }
    const T om = T(1) - relax;
    V4<T> y{om * u.x + j0, om * u.y + j1, om * u.z + j2, T(0)};
    if (accumulate) {
        const V4<T> q = out[i];
        y = V4<T>{q.x + y.x, q.y + y.y, q.z + y.z, T(0)};
    }
    out[i] = y;
}

// adjoint of the right-hand side: rb = w D^-1 rho; rhs0's adjoint collects it
template <typename T>
__global__ void k_adj_rhs(int nsim, T relax, const V4<T>* __restrict__ rho, const T* __restrict__ InvD,
                          V4<T>* __restrict__ rb, V4<T>* __restrict__ r0b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nsim) return;
    const T f = relax * InvD[i];
    const V4<T> p = rho[i];
    const V4<T> v{f * p.x, f * p.y, f * p.z, T(0)};
    rb[i] = v;
    const V4<T> o = r0b[i];
    r0b[i] = V4<T>{o.x + v.x, o.y + v.y, o.z + v.z, T(0)};
}

// adjoint of the curvature vectors: abar_k = sum_{s in row k} bend_s rb_nbr(s),
// then through the rescaling a = q c / |q|
template <typename T>
__global__ void k_adj_curv(int nsim, const V4<T>* __restrict__ x, const V4<T>* __restrict__ rb,
                           const int* __restrict__ lPtr, const int* __restrict__ lNbr, const T* __restrict__ lLbo,
                           const T* __restrict__ lBend, const T* __restrict__ CurvNorm, V4<T>* __restrict__ qb) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nsim) return;
    T q0 = T(0), q1 = T(0), q2 = T(0), a0 = T(0), a1 = T(0), a2 = T(0);
    for (int s = lPtr[k]; s < lPtr[k + 1]; ++s) {
        const int j = lNbr[s];
        const V4<T> xj = x[j];
        const T l = lLbo[s];
        q0 += l * xj.x;
        q1 += l * xj.y;
        q2 += l * xj.z;
        const V4<T> r = rb[j];
        const T bs = lBend[s];
        a0 += bs * r.x;
        a1 += bs * r.y;
        a2 += bs * r.z;
    }
    const T nrm = dsqrt(q0 * q0 + q1 * q1 + q2 * q2);
    if (nrm >= T(1e-10)) {
        const T h0 = q0 / nrm, h1 = q1 / nrm, h2 = q2 / nrm;
        const T pr = h0 * a0 + h1 * a1 + h2 * a2;
        const T c = CurvNorm[k] / nrm;
        a0 = c * (a0 - h0 * pr);
        a1 = c * (a1 - h1 * pr);
        a2 = c * (a2 - h2 * pr);
    }
    qb[k] = V4<T>{a0, a1, a2, T(0)};
}

// adjoint of the local step at x: xb_m (holding the solve's adjoint of x) +=
// transposed LBO gather of qb + spring terms; kbar_m += rb_m . sum_s rest_s d_s/|d_s|
template <typename T>
__global__ void k_adj_local(int nsim, const V4<T>* __restrict__ x, const V4<T>* __restrict__ rb,
                            const V4<T>* __restrict__ qb, const int* __restrict__ lPtr, const int* __restrict__ lNbr,
                            const T* __restrict__ lLboT, const T* __restrict__ lRest, const T* __restrict__ Strain,
                            V4<T>* __restrict__ xb, T* __restrict__ kbar) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nsim) return;
    const int b = lPtr[m], e = lPtr[m + 1];
    const V4<T> xm = x[m], rm = rb[m];
    const T km = Strain[m];
    V4<T> acc = xb[m];
    T kb = T(0);
    for (int s = b; s < e; ++s) {
        const int j = lNbr[s];
        const V4<T> q = qb[j];
        const T l = lLboT[s];
        acc.x += l * q.x;
        acc.y += l * q.y;
        acc.z += l * q.z;
        if (s == b) continue;
        const V4<T> xj = x[j], rj = rb[j];
        const T d0 = xm.x - xj.x, d1 = xm.y - xj.y, d2 = xm.z - xj.z;
        const T len = dsqrt(d0 * d0 + d1 * d1 + d2 * d2);
        const T h0 = d0 / len, h1 = d1 / len, h2 = d2 / len;
        const T rest = lRest[s];
        const T cm = km * rest, cj = Strain[j] * rest;
        const T u0 = cm * rm.x - cj * rj.x, u1 = cm * rm.y - cj * rj.y, u2 = cm * rm.z - cj * rj.z;
        const T pr = h0 * u0 + h1 * u1 + h2 * u2;
        acc.x += (u0 - h0 * pr) / len;
        acc.y += (u1 - h1 * pr) / len;
        acc.z += (u2 - h2 * pr) / len;
        kb += rest * (rm.x * h0 + rm.y * h1 + rm.z * h2);
    }
    xb[m] = V4<T>{acc.x, acc.y, acc.z, T(0)};
    kbar[m] += kb;
}

// Adjoint of the strain-limit projection R(F) = U C V^T (svd3.cuh: F = U
// diag(s) V^T, C the clamped singular values) at F: given Rb = dL/dR, returns
// Fb = dL/dF = U Pb V^T, where in the singular frame (Rb' = U^T Rb V) the
// differential of R is dR'_kk = c'_k dP_kk and, for k != m,
// dR'_km = alpha dP_km + beta dP_mk, dR'_mk = beta dP_km + alpha dP_mk with
// alpha = (c_m s_m - c_k s_k) / (s_m^2 - s_k^2), beta = (c_m s_k - c_k s_m) /
// (s_m^2 - s_k^2) (from U^T dU and V^T dV, the SVD's skew differentials).
// Unclamped pairs give alpha = 1, beta = 0 (R = F there); two values clamped to
// one bound give alpha = -beta = c / (s_k + s_m).  dc[k] = dc_k / ds_k.
template <typename T>
__device__ void clamp_svd_adjoint(const T (&U)[3][3], const T (&s)[3], const T (&V)[3][3], const T (&c)[3],
                                  const T (&dc)[3], const T (&Rb)[3][3], T (&Fb)[3][3]) {
    T A[3][3], Pb[3][3];  // A = Rb V, then Rb' = U^T A
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) A[i][j] = Rb[i][0] * V[0][j] + Rb[i][1] * V[1][j] + Rb[i][2] * V[2][j];
    T Rp[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) Rp[i][j] = U[0][i] * A[0][j] + U[1][i] * A[1][j] + U[2][i] * A[2][j];
    for (int k = 0; k < 3; ++k) Pb[k][k] = dc[k] * Rp[k][k];
    for (int k = 0; k < 3; ++k)
        for (int m = k + 1; m < 3; ++m) {
            T al, be;
            const T sk = s[k], sm = s[m];
            if (c[k] == sk && c[m] == sm) {
                al = T(1);
                be = T(0);
            } else {
                T den = sm * sm - sk * sk;
                if (den * den < T(1e-28) * (sk * sk + sm * sm) * (sk * sk + sm * sm)) {
                    // equal singular values: the limit for values clamped to one bound
                    const T ss = sk + sm;
                    al = (ss != T(0)) ? c[k] / ss : T(0);
                    be = -al;
                } else {
                    al = (c[m] * sm - c[k] * sk) / den;
                    be = (c[m] * sk - c[k] * sm) / den;
                }
            }
            Pb[k][m] = al * Rp[k][m] + be * Rp[m][k];
            Pb[m][k] = be * Rp[k][m] + al * Rp[m][k];
        }
    for (int i = 0; i < 3; ++i)  // Fb = U Pb V^T
        for (int j = 0; j < 3; ++j) {
            T a = T(0);
            for (int k = 0; k < 3; ++k) {
                const T w = U[i][k];
                a += w * (Pb[k][0] * V[j][0] + Pb[k][1] * V[j][1] + Pb[k][2] * V[j][2]);
            }
            Fb[i][j] = a;
        }
}

// Adjoint of the strain-limit projections (tets; cloth triangles, whose
// fourth vertex is -1) at the positions x the forward projected: element e
// added out[c] = w R G[:, c] to its vertex c's right-hand side (svd3.cuh:
// tet_project, tri_project), so with rb the right-hand sides' adjoint,
// Rb = w sum_c rb_c G[:, c]^T; through the SVD (and, for a triangle, its unit
// normal column) to Fb, then Dsb = Fb Dm^-T and the vertices' adjoints into
// Eb[4 e + c] (gathered per vertex in ascending element order).
template <typename T>
__global__ void k_adj_elem(int ntet, const int4* __restrict__ Tets, const T* __restrict__ Idm,
                           const T* __restrict__ W, const V4<T>* __restrict__ x, const V4<T>* __restrict__ rb,
                           V4<T>* __restrict__ Eb) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ntet) return;
    const int4 q = Tets[e];
    const bool tri = q.w < 0;
    const int id[4] = {q.x, q.y, q.z, tri ? q.x : q.w};
    const V4<T> x0 = x[id[0]];
    T Ds[3][3];
    for (int c = 0; c < 3; ++c) {
        const V4<T> xc = x[id[c + 1]];
        Ds[0][c] = xc.x - x0.x;
        Ds[1][c] = xc.y - x0.y;
        Ds[2][c] = xc.z - x0.z;
    }
    T idm[9];
    for (int k = 0; k < 9; ++k) idm[k] = Idm[9 * (size_t)e + k];
    const T w = W[e];
    T F[3][3], U[3][3], sv[3], V[3][3], c[3], dc[3], Rb[3][3], Fb[3][3];
    auto clamp_ = [](T a, T& d) {
        d = (a > T(0.999) && a < T(1.001)) ? T(1) : T(0);
        return a < T(1.001) ? (a < T(0.999) ? T(0.999) : a) : T(1.001);
    };
    auto rbv = [&](int c) -> V4<T> { return rb[id[c]]; };
    if (tri) {
        for (int i = 0; i < 3; ++i) {
            F[i][0] = Ds[i][0] * idm[0] + Ds[i][1] * idm[2];
            F[i][1] = Ds[i][0] * idm[1] + Ds[i][1] * idm[3];
        }
        const T n[3] = {F[1][0] * F[2][1] - F[2][0] * F[1][1], F[2][0] * F[0][1] - F[0][0] * F[2][1],
                        F[0][0] * F[1][1] - F[1][0] * F[0][1]};
        const T nn = n[0] * n[0] + n[1] * n[1] + n[2] * n[2];
        const T nl = nn > T(0) ? dsqrt(nn) : T(0);
        const T inv = nl > T(0) ? T(1) / nl : T(0);
        for (int i = 0; i < 3; ++i) F[i][2] = n[i] * inv;
        svd::svd3(F, U, sv, V);
        for (int k = 0; k < 3; ++k) {  // sc_k = sign(s_k) clamp(|s_k|): dc_k / ds_k = clamp'(|s_k|)
            const T a = sv[k] < T(0) ? -sv[k] : sv[k];
            c[k] = clamp_(a, dc[k]);
            if (sv[k] < T(0)) c[k] = -c[k];
        }
        const T G[3][2] = {{-(idm[0] + idm[2]), -(idm[1] + idm[3])}, {idm[0], idm[1]}, {idm[2], idm[3]}};
        for (int r = 0; r < 3; ++r) {
            Rb[r][2] = T(0);
            for (int j = 0; j < 2; ++j) {
                T a = T(0);
                for (int cc = 0; cc < 3; ++cc) {
                    const V4<T> v = rbv(cc);
                    a += (r == 0 ? v.x : r == 1 ? v.y : v.z) * G[cc][j];
                }
                Rb[r][j] = w * a;
            }
        }
        clamp_svd_adjoint(U, sv, V, c, dc, Rb, Fb);
        // the normal column: F[:, 2] = n / |n| with n = a x b (a, b the first two columns)
        T nb[3] = {Fb[0][2], Fb[1][2], Fb[2][2]};
        if (nl > T(0)) {
            const T h[3] = {n[0] * inv, n[1] * inv, n[2] * inv};
            const T pr = h[0] * nb[0] + h[1] * nb[1] + h[2] * nb[2];
            for (int i = 0; i < 3; ++i) nb[i] = (nb[i] - h[i] * pr) * inv;
            const T a[3] = {F[0][0], F[1][0], F[2][0]}, b[3] = {F[0][1], F[1][1], F[2][1]};
            // d(a x b) = da x b + a x db: ab += b x nb, bb += nb x a
            Fb[0][0] += b[1] * nb[2] - b[2] * nb[1];
            Fb[1][0] += b[2] * nb[0] - b[0] * nb[2];
            Fb[2][0] += b[0] * nb[1] - b[1] * nb[0];
            Fb[0][1] += nb[1] * a[2] - nb[2] * a[1];
            Fb[1][1] += nb[2] * a[0] - nb[0] * a[2];
            Fb[2][1] += nb[0] * a[1] - nb[1] * a[0];
        }
        T d0[3], d1[3];
        for (int i = 0; i < 3; ++i) {
            d0[i] = Fb[i][0] * idm[0] + Fb[i][1] * idm[1];
            d1[i] = Fb[i][0] * idm[2] + Fb[i][1] * idm[3];
        }
        Eb[4 * (size_t)e + 0] = V4<T>{-(d0[0] + d1[0]), -(d0[1] + d1[1]), -(d0[2] + d1[2]), T(0)};
        Eb[4 * (size_t)e + 1] = V4<T>{d0[0], d0[1], d0[2], T(0)};
        Eb[4 * (size_t)e + 2] = V4<T>{d1[0], d1[1], d1[2], T(0)};
        Eb[4 * (size_t)e + 3] = V4<T>{T(0), T(0), T(0), T(0)};
        return;
    }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) F[i][j] = Ds[i][0] * idm[j] + Ds[i][1] * idm[3 + j] + Ds[i][2] * idm[6 + j];
    svd::svd3(F, U, sv, V);
    // sc_k = clamp(|s_k|) (a negative determinant's s_2 flipped, |s| already
    // descending): dc_k / ds_k = clamp'(|s_k|) sign(s_k)
    for (int k = 0; k < 3; ++k) {
        const T a = sv[k] < T(0) ? -sv[k] : sv[k];
        c[k] = clamp_(a, dc[k]);
        if (sv[k] < T(0)) dc[k] = -dc[k];
    }
    T G[3][4];
    for (int i = 0; i < 3; ++i) {
        G[i][1] = idm[i];
        G[i][2] = idm[3 + i];
        G[i][3] = idm[6 + i];
        G[i][0] = -(G[i][1] + G[i][2] + G[i][3]);
    }
    for (int r = 0; r < 3; ++r)
        for (int j = 0; j < 3; ++j) {
            T a = T(0);
            for (int cc = 0; cc < 4; ++cc) {
                const V4<T> v = rbv(cc);
                a += (r == 0 ? v.x : r == 1 ? v.y : v.z) * G[j][cc];
            }
            Rb[r][j] = w * a;
        }
    clamp_svd_adjoint(U, sv, V, c, dc, Rb, Fb);
    T db[3][3];  // Dsb = Fb Dm^-T
    for (int i = 0; i < 3; ++i)
        for (int k = 0; k < 3; ++k) db[i][k] = Fb[i][0] * idm[3 * k] + Fb[i][1] * idm[3 * k + 1] + Fb[i][2] * idm[3 * k + 2];
    Eb[4 * (size_t)e + 0] =
        V4<T>{-(db[0][0] + db[0][1] + db[0][2]), -(db[1][0] + db[1][1] + db[1][2]), -(db[2][0] + db[2][1] + db[2][2]), T(0)};
    for (int k = 0; k < 3; ++k) Eb[4 * (size_t)e + 1 + k] = V4<T>{db[0][k], db[1][k], db[2][k], T(0)};
}

// xb_i += the element adjoints of vertex i, in ascending element order
template <typename T>
__global__ void k_adj_elem_gather(int nsim, const int* __restrict__ vtPtr, const int* __restrict__ vtIdx,
                                  const V4<T>* __restrict__ Eb, V4<T>* __restrict__ xb) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nsim) return;
    V4<T> a = xb[i];
    for (int q = vtPtr[i]; q < vtPtr[i + 1]; ++q) {
        const V4<T> v = Eb[vtIdx[q]];
        a.x += v.x;
        a.y += v.y;
        a.z += v.z;
    }
    xb[i] = a;
}

// step output adjoints (pb of P, vb of V = (P - X0) invt) -> pb of the solved
// positions, vb := adjoint of X0; r0b := 0
template <typename T>
__global__ void k_adj_step_begin(int nsim, T invt, V4<T>* __restrict__ pb, V4<T>* __restrict__ vb,
                                 V4<T>* __restrict__ r0b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nsim) return;
    const V4<T> p = pb[i], v = vb[i];
    pb[i] = V4<T>{p.x + invt * v.x, p.y + invt * v.y, p.z + invt * v.z, T(0)};
    vb[i] = V4<T>{-invt * v.x, -invt * v.y, -invt * v.z, T(0)};
    r0b[i] = V4<T>{T(0), T(0), T(0), T(0)};
}

// through the prediction: free vertices y = (v + m g) dt + x, rhs0 = y / (dt m),
// start positions y; pinned vertices start at x and keep rhs0 = 0 and v = 0.
// pb := adjoint of the step's input positions, vb := of its input velocities.
template <typename T>
__global__ void k_adj_step_end(int nsim, T dt, const T* __restrict__ InvMass, const int* __restrict__ PinFlag,
                               V4<T>* __restrict__ pb, V4<T>* __restrict__ vb, const V4<T>* __restrict__ r0b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nsim) return;
    const V4<T> p = pb[i], x0 = vb[i];
    if (PinFlag[i] != -1) {
        pb[i] = V4<T>{x0.x + p.x, x0.y + p.y, x0.z + p.z, T(0)};
        vb[i] = V4<T>{T(0), T(0), T(0), T(0)};
        return;
    }
    const T m = InvMass[i] * dt;
    const T mm = T(1) / (dt * m);
    const V4<T> r = r0b[i];
    const T y0 = p.x + mm * r.x, y1 = p.y + mm * r.y, y2 = p.z + mm * r.z;
    pb[i] = V4<T>{x0.x + y0, x0.y + y1, x0.z + y2, T(0)};
    vb[i] = V4<T>{dt * y0, dt * y1, dt * y2, T(0)};
}

}  // namespace

template <typename T, typename TC>
void launch_adj_tables(const Dev<T, TC>& d, T* lLboT, T* NTval, cudaStream_t s) {
    const int n = std::max(d.nsim, d.nslice * 32);
    k_adj_tables<T><<<blocks_for(n), kBlock, 0, s>>>(d.nsim, d.nslice, d.lPtr, d.lNbr, d.lLbo, d.sOff, d.sLen,
                                                     d.sCol, d.sVal, lLboT, NTval);
}
template <typename T, typename TC>
void launch_adj_sweep(const Dev<T, TC>& d, const T* NTval, T relax, T scale, const V4<T>* in, V4<T>* other,
                      const V4<T>* z, V4<T>* out, bool accumulate, V4<T>* rho, T* kbar, cudaStream_t s) {
    k_adj_sweep<T><<<blocks_for(d.nsim), kBlock, 0, s>>>(d.nsim, relax, scale, in, other, z, out, accumulate ? 1 : 0,
                                                         rho, kbar, d.Rhs, d.InvD, d.sOff, d.sLen, d.sCol, d.sVal,
                                                         NTval, d.lPtr, d.lNbr);
}
template <typename T, typename TC>
void launch_adj_local(const Dev<T, TC>& d, const T* lLboT, T relax, const V4<T>* x, const V4<T>* rho, V4<T>* rb,
                      V4<T>* qb, V4<T>* r0b, V4<T>* xb, T* kbar, V4<T>* eb, cudaStream_t s) {
    k_adj_rhs<T><<<blocks_for(d.nsim), kBlock, 0, s>>>(d.nsim, relax, rho, d.InvD, rb, r0b);
    k_adj_curv<T><<<blocks_for(d.nsim), kBlock, 0, s>>>(d.nsim, x, rb, d.lPtr, d.lNbr, d.lLbo, d.lBend, d.CurvNorm,
                                                        qb);
    k_adj_local<T><<<blocks_for(d.nsim), kBlock, 0, s>>>(d.nsim, x, rb, qb, d.lPtr, d.lNbr, lLboT, d.lRest,
                                                         d.Strain, xb, kbar);
    if (d.ntet > 0 && eb) {
        k_adj_elem<T><<<blocks_for(d.ntet, 128), 128, 0, s>>>(d.ntet, d.Tets, d.TetIdm, d.TetW, x, rb, eb);
        k_adj_elem_gather<T><<<blocks_for(d.nsim), kBlock, 0, s>>>(d.nsim, d.vtPtr, d.vtIdx, eb, xb);
    }
}
template <typename T, typename TC>
void launch_adj_step_begin(const Dev<T, TC>& d, T invt, V4<T>* pb, V4<T>* vb, V4<T>* r0b, cudaStream_t s) {
    k_adj_step_begin<T><<<blocks_for(d.nsim), kBlock, 0, s>>>(d.nsim, invt, pb, vb, r0b);
}
template <typename T, typename TC>
void launch_adj_step_end(const Dev<T, TC>& d, T dt, V4<T>* pb, V4<T>* vb, const V4<T>* r0b, cudaStream_t s) {
    k_adj_step_end<T><<<blocks_for(d.nsim), kBlock, 0, s>>>(d.nsim, dt, d.InvMass, d.PinFlag, pb, vb, r0b);
}

template void launch_adj_tables<double, double>(const Dev<double, double>&, double*, double*, cudaStream_t);
template void launch_adj_sweep<double, double>(const Dev<double, double>&, const double*, double, double,
                                               const V4<double>*, V4<double>*, const V4<double>*, V4<double>*,
                                               bool, V4<double>*, double*, cudaStream_t);
template void launch_adj_local<double, double>(const Dev<double, double>&, const double*, double,
                                               const V4<double>*, const V4<double>*, V4<double>*, V4<double>*,
                                               V4<double>*, V4<double>*, double*, V4<double>*, cudaStream_t);
template void launch_adj_step_begin<double, double>(const Dev<double, double>&, double, V4<double>*, V4<double>*,
                                                    V4<double>*, cudaStream_t);
template void launch_adj_step_end<double, double>(const Dev<double, double>&, double, V4<double>*, V4<double>*,
                                                  const V4<double>*, cudaStream_t);

}  // namespace pdipc
