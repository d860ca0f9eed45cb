"""The discrete adjoint of the contact-free projective-dynamics step, restated
in numpy on random tables and checked against central differences on the CPU.

The forward restates the plain FP64 form of pd_kernels.cu on a 4x4 grid with
random stencil weights (LBO weights, bending coefficients and their
transposes, rest lengths, per-vertex strain weights, a symmetric bending
part of the matrix plus the strain weights on the spring neighbours, two
pinned vertices): prediction, local steps (spring projections, rescaled
curvature vectors, bending terms), the two-sweep Chebyshev-Jacobi global step,
and the velocity update.  The adjoint follows the same recurrences as
adjoint_kernels.cu and the reverse pass of solver.cu (adjoint_step): transposed
sweeps, the right-hand side's adjoint w D^-1 sum(u), the local step's gathers,
and the per-vertex stretch-stiffness terms of the rhs, N and D.  It pins the
method.  The oracle's C++ restatement of the same reverse pass on real scene
tables is checked here against central differences of the oracle's own
forward; test_adjoint_gpu.py checks the kernels against differences of the GPU
forward and against the oracle's adjoint."""
import os

import numpy as np
import pytest

rng = np.random.default_rng(1)  # the random tables
G = 4
n = G * G
def vid(r, c): return r * G + c
nbrs = []
for r in range(G):
    for c in range(G):
        s = []
        for dr in (-1, 0, 1):
            for dc in (-1, 0, 1):
                if (dr or dc) and 0 <= r + dr < G and 0 <= c + dc < G:
                    s.append(vid(r + dr, c + dc))
        nbrs.append(sorted(s))
lPtr = [0]
lNbr = []
for i in range(n):
    lNbr += [i] + nbrs[i]
    lPtr.append(len(lNbr))
lPtr = np.array(lPtr); lNbr = np.array(lNbr)
ns = len(lNbr)
rev = np.zeros(ns, int)
for i in range(n):
    for s in range(lPtr[i], lPtr[i + 1]):
        j = lNbr[s]
        rev[s] = next(t for t in range(lPtr[j], lPtr[j + 1]) if lNbr[t] == i)
X = np.array([[vid(r, c) % G * 0.1, 0.0, vid(r, c) // G * 0.1] for r in range(G) for c in range(G)]) + rng.uniform(-0.01, 0.01, (n, 3))
lRest = np.zeros(ns)
for i in range(n):
    for s in range(lPtr[i] + 1, lPtr[i + 1]):
        lRest[s] = np.linalg.norm(X[i] - X[lNbr[s]]) * (1 + 0.05 * ((i + lNbr[s]) % 3))
lLbo = rng.uniform(-1, 1, ns)
lBend = rng.uniform(-0.1, 0.1, ns) * 1e-2
lBendT = lBend[rev]
strain = rng.uniform(50, 150, n)
curv = rng.uniform(0.5, 2.0, n)
invm = rng.uniform(50, 100, n)
grav = np.tile([0.0, -9.8, 0.0], (n, 1)) / invm[:, None]
pinned = np.zeros(n, bool); pinned[[0, G - 1]] = True
pinK = 1e3
pinRhs = np.where(pinned[:, None], pinK * X, 0.0)
Bsym = np.zeros((n, n))
for i in range(n):
    for j in nbrs[i]:
        if j > i:
            Bsym[i, j] = Bsym[j, i] = rng.uniform(-0.2, 0.2)
dt = 1 / 240.0
w, rho = 2 / 3, 0.9992
LG, CHEBY, K = 3, 4, 2

def tables(k):
    N = Bsym.copy()
    De = np.zeros(n)
    for i in range(n):
        for j in nbrs[i]:
            N[i, j] += k[i]
        De[i] = len(nbrs[i]) * k[i] + 3.0 + (pinK if pinned[i] else 0.0)
    return N, De

def omegas():
    r2 = rho * rho
    om = 2 / (2 - r2)
    out = []
    for it in range(1, CHEBY):
        out.append(om)
        om = 4 / (4 - r2 * om)
    return out

def local(x, k, Rhs0):
    q = np.zeros((n, 3))
    for i in range(n):
        for s in range(lPtr[i], lPtr[i + 1]):
            q[i] += lLbo[s] * x[lNbr[s]]
    a = q.copy()
    for i in range(n):
        nr = np.linalg.norm(q[i])
        if nr >= 1e-10: a[i] = q[i] * (curv[i] / nr)
    r = np.zeros((n, 3))
    for i in range(n):
        t = np.zeros(3)
        for s in range(lPtr[i] + 1, lPtr[i + 1]):
            d = x[i] - x[lNbr[s]]
            t += k[i] * (lRest[s] / np.linalg.norm(d)) * d
        t += lBend[lPtr[i]] * a[i]
        ri = Rhs0[i] + t
        for s in range(lPtr[i] + 1, lPtr[i + 1]):
            ri = ri + lBendT[s] * a[lNbr[s]]
        r[i] = ri + pinRhs[i]
    return r, q

def sweep(z, r, N, invD):
    return (1 - w) * z + w * (invD[:, None] * (N @ z + r))

def lg_forward(x, k, Rhs0, N, invD, tape=False):
    r, q = local(x, k, Rhs0)
    Xs = [x]
    Ys = []
    Y = sweep(x, r, N, invD); Ys.append(Y)
    Xs.append(sweep(Y, r, N, invD))
    for it, om in enumerate(omegas(), start=1):
        Y = sweep(Xs[it], r, N, invD); Ys.append(Y)
        Xs.append(om * (sweep(Y, r, N, invD) - Xs[it - 1]) + Xs[it - 1])
    return (Xs[-1], Xs, Ys, r) if tape else Xs[-1]

def step(x, v, k):
    N, De = tables(k)
    im = invm
    m = im * dt
    Di = np.where(pinned, 0.0, 1 / (im * dt * dt))
    invD = 1 / (De + Di)
    y = (v + m[:, None] * grav) * dt + x
    Rhs0 = np.where(pinned[:, None], 0.0, (1 / (dt * m))[:, None] * y)
    P = np.where(pinned[:, None], x, y)
    for o in range(K):
        for l in range(LG):
            P = lg_forward(P, k, Rhs0, N, invD)
    invt = (1 / dt) * (1 - dt)
    V = (P - x) * invt
    return P, V

def step_adj(x, v, k, Pb_T, Vb_T):
    N, De = tables(k)
    im = invm; m = im * dt
    Di = np.where(pinned, 0.0, 1 / (im * dt * dt))
    invD = 1 / (De + Di)
    deg = np.array([len(nbrs[i]) for i in range(n)])
    y = (v + m[:, None] * grav) * dt + x
    Rhs0 = np.where(pinned[:, None], 0.0, (1 / (dt * m))[:, None] * y)
    P = np.where(pinned[:, None], x, y)
    tapeX = []
    for o in range(K):
        for l in range(LG):
            tapeX.append(P)
            P = lg_forward(P, k, Rhs0, N, invD)
    invt = (1 / dt) * (1 - dt)
    Pb = Pb_T + invt * Vb_T
    X0b = -invt * Vb_T
    r0b = np.zeros((n, 3))
    kb = np.zeros(n)
    NT = N.T
    oms = omegas()
    def stiff(ub, z, r):
        nz = N @ z + r
        sz = np.array([z[nbrs[i]].sum(0) for i in range(n)])
        return w * invD * np.sum(ub * (sz - (deg * invD)[:, None] * nz), axis=1)
    def JT(ub):
        return (1 - w) * ub + NT @ (w * invD[:, None] * ub)
    for xl in reversed(tapeX):
        _, Xs, Ys, r = lg_forward(xl, k, Rhs0, N, invD, tape=True)
        Xb = [np.zeros((n, 3)) for _ in range(CHEBY + 1)]
        Xb[CHEBY] = Pb.copy()
        rhob = np.zeros((n, 3))
        for it in range(CHEBY - 1, 0, -1):
            om = oms[it - 1]
            u2 = om * Xb[it + 1]
            Xb[it - 1] += (1 - om) * Xb[it + 1]
            rhob += u2; kb += stiff(u2, Ys[it], r)
            u1 = JT(u2)
            rhob += u1; kb += stiff(u1, Xs[it], r)
            Xb[it] += JT(u1)
        u2 = Xb[1]
        rhob += u2; kb += stiff(u2, Ys[0], r)
        u1 = JT(u2)
        rhob += u1; kb += stiff(u1, Xs[0], r)
        Xb[0] += JT(u1)
        rb = w * invD[:, None] * rhob
        r0b += rb
        # local step adjoint at xl
        q = np.zeros((n, 3))
        for i in range(n):
            for s in range(lPtr[i], lPtr[i + 1]):
                q[i] += lLbo[s] * xl[lNbr[s]]
        ab = np.zeros((n, 3))
        for kk in range(n):
            for s in range(lPtr[kk], lPtr[kk + 1]):
                ab[kk] += lBend[s] * rb[lNbr[s]]
        qb = ab.copy()
        for i in range(n):
            nr = np.linalg.norm(q[i])
            if nr >= 1e-10:
                qh = q[i] / nr
                qb[i] = (curv[i] / nr) * (ab[i] - qh * (qh @ ab[i]))
        xb = Xb[0].copy()
        for mm in range(n):
            for s in range(lPtr[mm], lPtr[mm + 1]):
                xb[mm] += lLbo[rev[s]] * qb[lNbr[s]]
            for s in range(lPtr[mm] + 1, lPtr[mm + 1]):
                j = lNbr[s]
                d = xl[mm] - xl[j]
                L = np.linalg.norm(d); dh = d / L
                u = k[mm] * lRest[s] * rb[mm] - k[j] * lRest[s] * rb[j]
                xb[mm] += (u - dh * (dh @ u)) / L
                kb[mm] += lRest[s] * (rb[mm] @ dh)
        Pb = xb
    mm_ = 1 / (dt * m)
    yb = np.where(pinned[:, None], 0.0, Pb + mm_[:, None] * r0b)
    xb0 = X0b + np.where(pinned[:, None], Pb, yb)
    vb0 = dt * yb
    return xb0, vb0, kb

def rollout(x, v, k, T):
    for _ in range(T):
        x, v = step(x, v, k)
    return x, v


def test_adjoint_recurrences_match_central_differences():
    T = 3
    x0 = X.copy()
    v0 = rng.uniform(-0.1, 0.1, (n, 3))
    v0[pinned] = 0
    k0 = strain.copy()
    cx, cv = rng.normal(size=(n, 3)), rng.normal(size=(n, 3))

    def loss(x, v, k):
        P, V = rollout(x, v, k, T)
        return np.sum(cx * P) + np.sum(cv * V) + 0.5 * np.sum(P * P)

    states = [(x0, v0)]
    x, v = x0, v0
    for _ in range(T):
        x, v = step(x, v, k0)
        states.append((x, v))
    Pb, Vb = cx + states[-1][0], cv.copy()
    kb = np.zeros(n)
    for t in range(T - 1, -1, -1):
        Pb, Vb, kbt = step_adj(*states[t], k0, Pb, Vb)
        kb += kbt
    eps = 1e-6
    cases = (("v", Vb, lambda d, e: (x0, v0 + e * d, k0)), ("x", Pb, lambda d, e: (x0 + e * d, v0, k0)),
             ("k", kb, lambda d, e: (x0, v0, k0 + e * d)))
    for name, g, pert in cases:
        for trial in range(3):
            d = rng.normal(size=g.shape)
            fd = (loss(*pert(d, eps)) - loss(*pert(d, -eps))) / (2 * eps)
            ad = float(np.sum(g * d))
            assert abs(fd - ad) <= 1e-4 * max(abs(fd), abs(ad)), (name, trial, fd, ad)


def test_oracle_adjoint_matches_its_own_central_differences():
    """The oracle's restatement of the adjoint (FP64, two-sweep form) on a real
    scene's tables: a 10x10 cloth with two pinned corners, three steps, against
    central differences of the oracle's forward (stiffness: Richardson
    extrapolation of two central differences of rebuilt contexts)."""
    from oracle.oracle import FORM_JJ, Oracle
    from pdipc import scenes

    for lg, cheby, outer in ((1, 1, 1), (2, 4, 1), (10, 15, 2)):
        def scene(k=1e4):
            return scenes.cloth_drop(10, 1, with_sphere=False, lg=lg, k_stretch=k)

        kw = dict(cheby_iterations=cheby, fixed_outer=outer)
        sc = scene()
        orc = Oracle(sc, "fp64", FORM_JJ, threads=2, **kw)
        r = np.random.default_rng(7 + lg)
        nv, T = sc.n_sim, 3
        x0 = sc.initial_positions()
        v0 = r.uniform(-0.1, 0.1, (nv, 3))
        cx, cv = r.normal(size=(nv, 3)), r.normal(size=(nv, 3))
        tgt = x0 + r.uniform(-0.05, 0.05, x0.shape)

        def run(o, x, v):
            o.set_state(x, v)
            o.step(T)
            return o.positions()[:nv].copy(), o.velocities().copy()

        def loss(x, v):
            return float(np.sum(cx * x) + np.sum(cv * v) + 0.5 * np.sum((x - tgt) ** 2))

        x, v = run(orc, x0, v0)
        gx0, gv0, gk = orc.adjoint_rollout(T, x0, v0, cx + (x - tgt), cv)
        for trial in range(2):
            d = r.normal(size=(nv, 3))
            fd = (loss(*run(orc, x0, v0 + 1e-5 * d)) - loss(*run(orc, x0, v0 - 1e-5 * d))) / 2e-5
            ad = float(np.sum(gv0 * d))
            assert abs(fd - ad) <= 1e-5 * abs(fd), ("v", lg, cheby, outer, fd, ad)
            fd = (loss(*run(orc, x0 + 1e-7 * d, v0)) - loss(*run(orc, x0 - 1e-7 * d, v0))) / 2e-7
            ad = float(np.sum(gx0 * d))
            assert abs(fd - ad) <= 1e-5 * abs(fd), ("x", lg, cheby, outer, fd, ad)

        def cd(h):
            lp = loss(*run(Oracle(scene(1e4 + h), "fp64", FORM_JJ, threads=2, **kw), x0, v0))
            lm = loss(*run(Oracle(scene(1e4 - h), "fp64", FORM_JJ, threads=2, **kw), x0, v0))
            return (lp - lm) / (2 * h)

        fd = (4.0 * cd(1.0) - cd(2.0)) / 3.0
        assert abs(fd - gk.sum()) <= 1e-4 * abs(fd), ("k", lg, cheby, outer, fd, gk.sum())


def _oracle_identity(n, T, lg, cheby, outer, threads=8, seed=7):
    """<dL/dout, tangent of out> against <dL/din, tangent of in> for separate
    position, velocity and stiffness directions, with the summed magnitude of
    the first product's terms (its round-off scale)."""
    from oracle.oracle import FORM_JJ, Oracle
    from pdipc import scenes

    sc = scenes.cloth_drop(n, 1, with_sphere=False, lg=lg)
    orc = Oracle(sc, "fp64", FORM_JJ, threads=threads, cheby_iterations=cheby, fixed_outer=outer)
    r = np.random.default_rng(seed)
    nv = sc.n_sim
    x0 = sc.initial_positions()
    v0 = r.uniform(-0.1, 0.1, (nv, 3))
    gx, gv = r.normal(size=(nv, 3)), r.normal(size=(nv, 3))
    gx0, gv0, gk = orc.adjoint_rollout(T, x0, v0, gx, gv)
    zero3, zero1 = np.zeros((nv, 3)), np.zeros(nv)
    out = []
    for name, dX, dV, dk, g, d in (("x", r.normal(size=(nv, 3)), zero3, zero1, gx0, 0),
                                   ("v", zero3, r.normal(size=(nv, 3)), zero1, gv0, 1),
                                   ("k", zero3, zero3, r.normal(size=nv), gk, 2)):
        tx, tv = orc.tangent_rollout(T, x0, v0, dX, dV, dk)
        lhs = float(np.sum(gx * tx) + np.sum(gv * tv))
        rhs = float(np.sum(g * (dX, dV, dk)[d]))
        out.append((name, lhs, rhs, float(np.sum(np.abs(gx * tx)) + np.sum(np.abs(gv * tv)))))
    return out


def test_oracle_adjoint_is_the_transpose_of_its_forward_tangent():
    """The oracle's adjoint against its forward-mode tangent of the same
    iteration: exact to round-off at any rollout length, where central
    differences of this strongly curved forward stop converging."""
    for case in ((10, 3, 1, 1, 1), (10, 3, 10, 15, 2), (32, 10, 10, 15, 3)):
        for name, lhs, rhs, scale in _oracle_identity(*case):
            assert abs(lhs - rhs) <= 1e-10 * scale, (case, name, lhs, rhs, scale)


@pytest.mark.skipif(not os.environ.get("PDIPC_LONG_TESTS"), reason="set PDIPC_LONG_TESTS=1 (minutes on the CPU)")
def test_oracle_adjoint_tangent_identity_128_cloth_50_steps():
    """The differentiable-rollout workload's shape on the oracle: 128x128 cloth,
    50 steps, 3 outer iterations of 10 local-global iterations per step."""
    for name, lhs, rhs, scale in _oracle_identity(128, 50, 10, 15, 3):
        assert abs(lhs - rhs) <= 1e-10 * scale, (name, lhs, rhs, scale)


def test_oracle_adjoint_through_strain_limits_matches_its_central_differences():
    """The oracle's adjoint of the strain-limit projections (the derivative of
    the clamped 3x3 SVD, and for a cloth triangle of its unit-normal column)
    against central differences of the oracle's own forward: an 8x8 cloth with
    the triangle strain limit, and a 2x2x2 tet block, with initial velocities
    that stretch most elements past the clamp."""
    from oracle.oracle import FORM_JJ, Oracle
    from pdipc import scenes

    cloth = scenes.cloth_drop(8, 1, with_sphere=False, lg=3)
    cloth.cloths[0].k_tri_strain = 2e3
    X, Tt = scenes.tet_block(2, 2, 2, size=(0.1, 0.1, 0.1))
    block = scenes.Scene("tet_adjoint", [], [], lg_iterations=3, steps=10, solids=[
        scenes.SolidSpec(X, Tt, np.array([0], np.int32), density=500.0, k_strain=2e3, patch_dim=2)])
    for sc, seed in ((cloth, 11), (block, 12)):
        orc = Oracle(sc, "fp64", FORM_JJ, threads=2, cheby_iterations=5, fixed_outer=2)
        r = np.random.default_rng(seed)
        nv, T = sc.n_sim, 3
        x0 = sc.initial_positions()
        v0 = r.uniform(-0.3, 0.3, (nv, 3))
        cx, cv = r.normal(size=(nv, 3)), r.normal(size=(nv, 3))

        def run(x, v):
            orc.set_state(x, v)
            orc.step(T)
            return orc.positions()[:nv].copy(), orc.velocities().copy()

        def loss(x, v):
            return float(np.sum(cx * x) + np.sum(cv * v))

        gx0, gv0, _ = orc.adjoint_rollout(T, x0, v0, cx, cv)
        for trial in range(3):
            d = r.normal(size=(nv, 3))
            fd = (loss(*run(x0, v0 + 1e-6 * d)) - loss(*run(x0, v0 - 1e-6 * d))) / 2e-6
            ad = float(np.sum(gv0 * d))
            assert abs(fd - ad) <= 1e-5 * abs(fd), ("v", sc.name, trial, fd, ad)
            fd = (loss(*run(x0 + 1e-8 * d, v0)) - loss(*run(x0 - 1e-8 * d, v0))) / 2e-8
            ad = float(np.sum(gx0 * d))
            assert abs(fd - ad) <= 1e-5 * abs(fd), ("x", sc.name, trial, fd, ad)
