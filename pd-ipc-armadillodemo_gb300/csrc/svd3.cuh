// svd3.cuh — 3x3 singular value decomposition for the tet strain projection.
//
// F = U diag(s) V^T with U and V proper rotations, |s0| >= |s1| >= |s2| and the
// sign of det F carried by s2: the convention of the reference's GPU SVD,
// whose output solveVolumetricStrainConstraintKernel (PdIpcGpuFunc.cu:487-525)
// post-processes.  Method: cyclic Jacobi on the symmetric F^T F gives V (a
// product of plane rotations, so det V = +1) and the squared singular values;
// the columns of F V are then reduced by three Givens rotations (a QR
// factorisation), whose product is U and whose diagonal is s, the last entry
// signed.  Every step is branch-light, register-resident arithmetic.
#pragma once

#include "common.cuh"

namespace pdipc {
namespace svd {

template <typename R>
__device__ __forceinline__ R rsqrt_(R v) {
    return R(1) / dsqrt(v);
}

// One Jacobi rotation zeroing S[p][q] of the symmetric S (Numerical Recipes
// form: theta = (S_qq - S_pp) / (2 S_pq), t = sgn(theta) / (|theta| + sqrt(theta^2 + 1))).
template <typename R>
__device__ __forceinline__ void jacobi(R (&S)[3][3], R (&V)[3][3], int p, int q) {
    const R apq = S[p][q];
    if (apq == R(0)) return;
    const R theta = (S[q][q] - S[p][p]) / (R(2) * apq);
    const R at = theta < R(0) ? -theta : theta;
    R t = R(1) / (at + dsqrt(at * at + R(1)));
    if (theta < R(0)) t = -t;
    const R c = rsqrt_(t * t + R(1)), s = t * c;
    const int r = 3 - p - q;
    const R srp = S[r][p], srq = S[r][q];
    S[p][p] -= t * apq;
    S[q][q] += t * apq;
    S[p][q] = S[q][p] = R(0);
    S[r][p] = S[p][r] = c * srp - s * srq;
    S[r][q] = S[q][r] = s * srp + c * srq;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const R vp = V[i][p], vq = V[i][q];
        V[i][p] = c * vp - s * vq;
        V[i][q] = s * vp + c * vq;
    }
}

// Givens rotation of rows a, b of B zeroing B[b][col]; U accumulates its transpose.
template <typename R>
__device__ __forceinline__ void givens(R (&B)[3][3], R (&U)[3][3], int a, int b, int col) {
    const R x = B[a][col], y = B[b][col];
    const R r2 = x * x + y * y;
    if (!(r2 > R(0))) return;
    const R ir = rsqrt_(r2);
    const R c = x * ir, s = y * ir;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        const R ba = B[a][j], bb = B[b][j];
        B[a][j] = c * ba + s * bb;
        B[b][j] = -s * ba + c * bb;
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const R ua = U[i][a], ub = U[i][b];
        U[i][a] = c * ua + s * ub;
        U[i][b] = -s * ua + c * ub;
    }
}

template <typename R>
__device__ __forceinline__ void swap_cols(R (&M)[3][3], int a, int b) {
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const R t = M[i][a];
        M[i][a] = M[i][b];
        M[i][b] = t;
    }
}

// F row-major; outputs U, V (row-major, proper rotations) and s.
template <typename R>
__device__ void svd3(const R (&F)[3][3], R (&U)[3][3], R (&s)[3], R (&V)[3][3]) {
    R S[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) S[i][j] = F[0][i] * F[0][j] + F[1][i] * F[1][j] + F[2][i] * F[2][j];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) V[i][j] = (i == j) ? R(1) : R(0);
    const R eps = sizeof(R) == 4 ? R(1e-7) : R(1e-16);
    for (int sweep = 0; sweep < (sizeof(R) == 4 ? 8 : 12); ++sweep) {
        const R off = S[0][1] * S[0][1] + S[0][2] * S[0][2] + S[1][2] * S[1][2];
        const R dia = S[0][0] * S[0][0] + S[1][1] * S[1][1] + S[2][2] * S[2][2];
        if (!(off > eps * eps * dia)) break;
        jacobi(S, V, 0, 1);
        jacobi(S, V, 0, 2);
        jacobi(S, V, 1, 2);
    }
    // eigenvalues descending; an odd permutation flips a column to keep det V = +1
    R l[3] = {S[0][0], S[1][1], S[2][2]};
    bool odd = false;
    auto order = [&](int a, int b) {
        if (l[a] < l[b]) {
            const R t = l[a];
            l[a] = l[b];
            l[b] = t;
            swap_cols(V, a, b);
            odd = !odd;
        }
    };
    order(0, 1);
    order(0, 2);
    order(1, 2);
    if (odd)
#pragma unroll
        for (int i = 0; i < 3; ++i) V[i][2] = -V[i][2];
    // B = F V; QR by Givens: B = U Rm, Rm upper triangular, diagonal = s
    R B[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) B[i][j] = F[i][0] * V[0][j] + F[i][1] * V[1][j] + F[i][2] * V[2][j];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) U[i][j] = (i == j) ? R(1) : R(0);
    givens(B, U, 0, 1, 0);
    givens(B, U, 0, 2, 0);
    givens(B, U, 1, 2, 1);
    s[0] = B[0][0];
    s[1] = B[1][1];
    s[2] = B[2][2];
}

// solveVolumetricStrainConstraintKernel (PdIpcGpuFunc.cu:439-599) for one tet:
// F = Ds Dm^-1 (Ds columns x_k - x_0), SVD, a negative determinant moved to a
// positive smallest singular value and the three re-sorted, each clamped to
// [0.999, 1.001] (clamp, cu:307-316), R = U S' V^T, out[c] = w R G[:, c] with
// G = [-sum_k Dm^-T(:, k) | Dm^-T].
template <typename R>
__device__ __forceinline__ void tet_project(const R (&Ds)[3][3], const R* idm, R w, R (&out)[4][3]) {
    R F[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) F[i][j] = Ds[i][0] * idm[j] + Ds[i][1] * idm[3 + j] + Ds[i][2] * idm[6 + j];
    R U[3][3], s[3], V[3][3];
    svd3(F, U, s, V);
    if (s[0] * s[1] * s[2] < R(0)) s[2] = -s[2];
    R hi = s[0], mid = s[1], lo = s[2];  // the reference's three-element sort
    if (mid < lo) { const R t = lo; lo = mid; mid = t; }
    if (hi < lo) { const R t = lo; lo = hi; hi = t; }
    if (hi < mid) { const R t = mid; mid = hi; hi = t; }
    R sc[3] = {hi, mid, lo};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        R v = sc[k] < R(1.001) ? sc[k] : R(1.001);
        sc[k] = v < R(0.999) ? R(0.999) : v;
    }
    R Rm[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
            Rm[i][j] = U[i][0] * sc[0] * V[j][0] + U[i][1] * sc[1] * V[j][1] + U[i][2] * sc[2] * V[j][2];
    R G[3][4];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        G[i][1] = idm[i];
        G[i][2] = idm[3 + i];
        G[i][3] = idm[6 + i];
        G[i][0] = -(G[i][1] + G[i][2] + G[i][3]);
    }
#pragma unroll
    for (int c = 0; c < 4; ++c)
#pragma unroll
        for (int r = 0; r < 3; ++r) out[c][r] = w * (Rm[r][0] * G[0][c] + Rm[r][1] * G[1][c] + Rm[r][2] * G[2][c]);
}

// The same strain limit for a cloth triangle (an element with three
// vertices): F = Ds Dm^-1 (3 x 2: the deformed edges x1 - x0, x2 - x0 over the
// rest edges in the rest triangle's own orthonormal frame, idm = Dm^-1
// row-major 2 x 2).  F takes the deformed unit normal as a third column, so the
// 3 x 3 F has singular values (s0, s1, 1) and det F > 0 (no flip); its SVD,
// clamped to [0.999, 1.001] as above, gives R = U S' V^T, whose first two
// columns P are the projection of F.  out[c] = w P G[c] with G = S Dm^-1, S
// the edge-selection rows (-1, -1), (1, 0), (0, 1).  A triangle folded flat
// (zero normal) keeps the third column zero and still projects its two
// in-plane directions.
template <typename R>
__device__ __forceinline__ void tri_project(const R (&Ds)[3][2], const R* idm, R w, R (&out)[3][3]) {
    R F[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        F[i][0] = Ds[i][0] * idm[0] + Ds[i][1] * idm[2];
        F[i][1] = Ds[i][0] * idm[1] + Ds[i][1] * idm[3];
    }
    R n[3] = {F[1][0] * F[2][1] - F[2][0] * F[1][1], F[2][0] * F[0][1] - F[0][0] * F[2][1],
              F[0][0] * F[1][1] - F[1][0] * F[0][1]};
    const R nn = n[0] * n[0] + n[1] * n[1] + n[2] * n[2];
    const R inv = nn > R(0) ? R(1) / dsqrt(nn) : R(0);
#pragma unroll
    for (int i = 0; i < 3; ++i) F[i][2] = n[i] * inv;
    R U[3][3], s[3], V[3][3];
    svd3(F, U, s, V);
    R sc[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const R a = s[k] < R(0) ? -s[k] : s[k];
        R v = a < R(1.001) ? a : R(1.001);
        sc[k] = v < R(0.999) ? R(0.999) : v;
        if (s[k] < R(0)) sc[k] = -sc[k];  // rank-deficient F only: keep U S V^T's orientation
    }
    R P[3][2];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j)
            P[i][j] = U[i][0] * sc[0] * V[j][0] + U[i][1] * sc[1] * V[j][1] + U[i][2] * sc[2] * V[j][2];
    const R G[3][2] = {{-(idm[0] + idm[2]), -(idm[1] + idm[3])}, {idm[0], idm[1]}, {idm[2], idm[3]}};
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int r = 0; r < 3; ++r) out[c][r] = w * (P[r][0] * G[c][0] + P[r][1] * G[c][1]);
}

}  // namespace svd
}  // namespace pdipc
