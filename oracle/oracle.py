"""ctypes wrapper of the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module; the shipped library never loads it.
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(ROOT, "pd-ipc-armadillodemo_gb300"))

from pdipc.abi import Params, Stats, STATUS_NAMES, params_for_scene  # noqa: E402

from . import build as _build  # noqa: E402

_lib = None

FORM_R2 = 0   # the reference's R2 operator with path tables
FORM_JJ = 1   # R2 applied as two weighted-Jacobi sweeps (the library's form)

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_i64p = C.POINTER(C.c_longlong)


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.POINTER(Params), C.c_int, C.c_int]
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_add_cloth.argtypes = [C.c_void_p, _dp, C.c_int, _ip, C.c_int, C.c_double, C.c_double,
                                    C.c_double, _ip, C.c_int, C.c_double, C.c_int]
        L.orc_add_cloth_ex.argtypes = [C.c_void_p, _dp, C.c_int, _ip, C.c_int, C.c_double, C.c_double,
                                       C.c_double, _ip, C.c_int, C.c_double, C.c_int, _dp, C.c_double, _dp]
        L.orc_add_static.argtypes = [C.c_void_p, _dp, C.c_int, _ip, C.c_int, C.c_int]
        L.orc_add_volumetric.argtypes = [C.c_void_p, _dp, C.c_int, _ip, C.c_int, C.c_double, C.c_double, _ip,
                                         C.c_int, C.c_double, C.c_int]
        L.orc_tet_project.argtypes = [C.c_int, _dp, _dp, _dp, _dp]
        L.orc_tri_project.argtypes = [C.c_int, _dp, _dp, _dp, _dp]
        L.orc_svd3.argtypes = [_dp, _dp, _dp, _dp]
        L.orc_tet_surface.argtypes = [_dp, C.c_int, _ip, C.c_int, _ip, C.c_int, _ip]
        L.orc_initialize.argtypes = [C.c_void_p]
        L.orc_step.argtypes = [C.c_void_p, C.c_int]
        L.orc_get_positions.argtypes = [C.c_void_p, _dp]
        L.orc_get_velocities.argtypes = [C.c_void_p, _dp]
        L.orc_set_state.argtypes = [C.c_void_p, _dp, _dp]
        L.orc_get_stats.argtypes = [C.c_void_p, C.POINTER(Stats)]
        L.orc_broadphase.argtypes = [C.c_void_p, _dp, _dp, _ip, C.c_longlong, _i64p, _ip, C.c_longlong,
                                     _i64p, _ip, C.c_longlong, _i64p]
        L.orc_morton.argtypes = [C.c_void_p, C.POINTER(C.c_ulonglong), _ip, C.c_int]
        L.orc_toi.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp, _dp]
        L.orc_contact.argtypes = [C.c_void_p, _dp, _dp, _dp, _i64p]
        L.orc_table.restype = C.c_longlong
        L.orc_table.argtypes = [C.c_void_p, C.c_char_p, _dp, _ip, C.c_longlong]
        L.orc_stage_pd.argtypes = [C.c_void_p, _dp, _dp, _dp]
        L.orc_adjoint_rollout.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _dp, _dp, _dp, _dp, _dp]
        L.orc_tangent_rollout.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _dp, _dp, _dp, _dp, _dp]
        L.orc_penalty_predict.argtypes = [C.c_void_p, _dp, _dp, _dp]
        L.orc_penalty.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _ip, C.c_longlong, C.c_double, C.c_double,
                                  C.c_double, _dp, _dp, _ip]
        L.orc_mesh_topology.argtypes = [_dp, C.c_int, _ip, C.c_int, C.c_int, _ip, C.c_int, _ip, _ip, C.c_int,
                                        _ip, C.c_int, _ip, _ip, _ip, _ip, _ip]
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


class OracleError(RuntimeError):
    pass


def _check(rc, what):
    if rc != 0:
        raise OracleError(f"{what}: {STATUS_NAMES.get(rc, rc)}")


class Oracle:
    """CPU restatement of PdIpcSimulator for one scene."""

    def __init__(self, scene, precision="fp64", form=FORM_JJ, threads=None, **overrides):
        L = lib()
        self.params = params_for_scene(scene, precision, **overrides)
        if threads is None:
            threads = os.cpu_count() or 1
        self.threads = threads
        self.h = L.orc_create(C.byref(self.params), form, threads)
        if not self.h:
            raise OracleError("orc_create failed")
        self._keep = []
        for c in scene.cloths:
            X = np.ascontiguousarray(c.X, dtype=np.float64)
            F = np.ascontiguousarray(c.F, dtype=np.int32)
            P = np.ascontiguousarray(c.pins, dtype=np.int32)
            ts, tk = getattr(c, "tri_stretch", None), getattr(c, "tri_strain", None)
            ts = None if ts is None else np.ascontiguousarray(ts, dtype=np.float64)
            tk = None if tk is None else np.ascontiguousarray(tk, dtype=np.float64)
            self._keep += [a for a in (ts, tk) if a is not None]
            _check(L.orc_add_cloth_ex(self.h, _d(X), X.shape[0], _i(F), F.shape[0], c.density, c.k_stretch,
                                      c.k_bend, _i(P), P.shape[0], c.k_pin, c.patch_dim,
                                      None if ts is None else _d(ts), float(getattr(c, "k_tri_strain", 0.0)),
                                      None if tk is None else _d(tk)), "add_cloth")
        for v in getattr(scene, "solids", []):
            X = np.ascontiguousarray(v.X, dtype=np.float64)
            T = np.ascontiguousarray(v.T, dtype=np.int32)
            P = np.ascontiguousarray(v.pins, dtype=np.int32)
            _check(L.orc_add_volumetric(self.h, _d(X), X.shape[0], _i(T), T.shape[0], v.density, v.k_strain,
                                        _i(P), P.shape[0], v.k_pin, v.patch_dim), "add_volumetric")
        for s in scene.statics:
            X = np.ascontiguousarray(s.X, dtype=np.float64)
            F = np.ascontiguousarray(s.F, dtype=np.int32)
            _check(L.orc_add_static(self.h, _d(X), X.shape[0], _i(F), F.shape[0], s.patch_dim), "add_static")
        _check(L.orc_initialize(self.h), "initialize")
        self.n_sim = scene.n_sim
        self.n_total = scene.n_total

    def close(self):
        if self.h:
            lib().orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, n=1):
        _check(lib().orc_step(self.h, n), "step")

    def positions(self):
        out = np.empty((self.n_total, 3), dtype=np.float64)
        _check(lib().orc_get_positions(self.h, _d(out)), "get_positions")
        return out

    def velocities(self):
        out = np.empty((self.n_sim, 3), dtype=np.float64)
        _check(lib().orc_get_velocities(self.h, _d(out)), "get_velocities")
        return out

    def set_state(self, X, V=None):
        X = np.ascontiguousarray(X, dtype=np.float64)
        Vp = None
        if V is not None:
            V = np.ascontiguousarray(V, dtype=np.float64)
            Vp = _d(V)
        _check(lib().orc_set_state(self.h, _d(X), Vp), "set_state")

    def stats(self):
        s = Stats()
        _check(lib().orc_get_stats(self.h, C.byref(s)), "get_stats")
        return s.as_dict()

    def broadphase(self, x_old, dx, cap=None):
        x_old = np.ascontiguousarray(x_old, dtype=np.float64)
        dx = np.ascontiguousarray(dx, dtype=np.float64)
        npair, npt, nee = C.c_longlong(), C.c_longlong(), C.c_longlong()
        cap = cap or 1 << 16
        while True:
            pairs = np.empty((cap, 2), np.int32)
            pt = np.empty((cap, 4), np.int32)
            ee = np.empty((cap, 4), np.int32)
            rc = lib().orc_broadphase(self.h, _d(x_old), _d(dx), _i(pairs), cap, C.byref(npair), _i(pt), cap,
                                      C.byref(npt), _i(ee), cap, C.byref(nee))
            if rc == 3:
                cap = max(npair.value, npt.value, nee.value)
                continue
            _check(rc, "broadphase")
            return pairs[:npair.value].copy(), pt[:npt.value].copy(), ee[:nee.value].copy()

    def morton(self, npatch):
        codes = np.empty(npatch, np.uint64)
        order = np.empty(npatch, np.int32)
        _check(lib().orc_morton(self.h, codes.ctypes.data_as(C.POINTER(C.c_ulonglong)), _i(order), npatch),
               "morton")
        return codes, order

    _INT_TABLES = {"lOff", "lNum", "lNbr", "pinFlag", "nPtr", "nCol", "r2Ptr", "r2Col", "r2Const", "r2First",
                   "pathPtr", "pathK"}

    def table(self, name):
        """One initialised table (orc_table): int32 for index tables, float64 otherwise."""
        n = lib().orc_table(self.h, name.encode(), None, None, 0)
        if n < 0:
            raise OracleError(f"unknown table {name}")
        if name in self._INT_TABLES:
            out = np.empty(max(n, 1), np.int32)
            lib().orc_table(self.h, name.encode(), None, _i(out), n)
        else:
            out = np.empty(max(n, 1), np.float64)
            lib().orc_table(self.h, name.encode(), _d(out), None, n)
        return out[:n]

    def toi(self, x0, x1, npt, nee):
        x0 = np.ascontiguousarray(x0, dtype=np.float64)
        x1 = np.ascontiguousarray(x1, dtype=np.float64)
        tp = np.empty(max(npt, 1), np.float64)
        te = np.empty(max(nee, 1), np.float64)
        g = C.c_double()
        _check(lib().orc_toi(self.h, _d(x0), _d(x1), _d(tp), _d(te), C.byref(g)), "toi")
        return tp[:npt], te[:nee], g.value

    # -- the reference's penalty / discrete-collision path (PdIpcGpuFunc.cu:2933-3740) --------
    def penalty_predict(self, X, V):
        X = np.ascontiguousarray(X, dtype=np.float64)
        V = np.array(V, dtype=np.float64, order="C")
        sn = np.empty((self.n_sim, 3), np.float64)
        _check(lib().orc_penalty_predict(self.h, _d(X), _d(V), _d(sn)), "penalty_predict")
        return sn, V

    def _penalty(self, kind, x, d, fp, k, kself, damping, V):
        x = np.ascontiguousarray(x, dtype=np.float64)
        d = np.ascontiguousarray(d if d is not None else x, dtype=np.float64)
        fp = np.ascontiguousarray(fp if fp is not None else np.zeros((0, 2)), dtype=np.int32).reshape(-1, 2)
        V = np.array(V, dtype=np.float64, order="C")
        F = np.empty((self.n_total, 3), np.float64)
        t = np.empty(self.n_total, np.int32)
        _check(lib().orc_penalty(self.h, kind, _d(x), _d(d), _i(fp) if fp.size else None, fp.shape[0], k, kself,
                                 damping, _d(V), _d(F), _i(t)), "penalty")
        return F, t, V

    def penalty_ccd(self, x0, d, stiffness, damping, V):
        return self._penalty(0, x0, d, None, stiffness, 0.0, damping, V)

    def penalty_floor(self, x, stiffness, damping, V):
        return self._penalty(1, x, None, None, stiffness, 0.0, damping, V)

    def penalty_dcd(self, x, face_pairs, stiffness, self_stiffness, damping, V):
        return self._penalty(2, x, None, face_pairs, stiffness, self_stiffness, damping, V)

    def stage_pd(self, X, V):
        X = np.ascontiguousarray(X, dtype=np.float64)
        V = np.ascontiguousarray(V, dtype=np.float64)
        out = np.empty((self.n_total, 3), np.float64)
        _check(lib().orc_stage_pd(self.h, _d(X), _d(V), _d(out)), "stage_pd")
        return out

    def adjoint_rollout(self, steps, X, V, dl_dx, dl_dv=None):
        """A contact-free rollout of `steps` from (X, V) and its discrete
        adjoint (FP64, two-sweep form): (dL/dX0, dL/dV0, dL/dk per simulated
        vertex) for dL/d(final positions, velocities) = (dl_dx, dl_dv)."""
        X = np.ascontiguousarray(X, dtype=np.float64)
        V = np.ascontiguousarray(V, dtype=np.float64)
        gx = np.ascontiguousarray(dl_dx, dtype=np.float64)
        gv = None if dl_dv is None else np.ascontiguousarray(dl_dv, dtype=np.float64)
        gx0 = np.empty((self.n_sim, 3), np.float64)
        gv0 = np.empty((self.n_sim, 3), np.float64)
        gk = np.empty(self.n_sim, np.float64)
        _check(lib().orc_adjoint_rollout(self.h, int(steps), _d(X), _d(V), _d(gx), _d(gv) if gv is not None else None,
                                         _d(gx0), _d(gv0), _d(gk)), "adjoint_rollout")
        return gx0, gv0, gk

    def tangent_rollout(self, steps, X, V, dX, dV, dk):
        """A contact-free rollout of `steps` from (X, V) with the forward-mode
        tangent (dX, dV, dk per simulated vertex) carried along (FP64,
        two-sweep form): the tangents of the final positions and velocities."""
        X = np.ascontiguousarray(X, dtype=np.float64)
        V = np.ascontiguousarray(V, dtype=np.float64)
        dX = np.ascontiguousarray(dX, dtype=np.float64)
        dV = np.ascontiguousarray(dV, dtype=np.float64)
        dk = np.ascontiguousarray(dk, dtype=np.float64)
        ox = np.empty((self.n_sim, 3), np.float64)
        ov = np.empty((self.n_sim, 3), np.float64)
        _check(lib().orc_tangent_rollout(self.h, int(steps), _d(X), _d(V), _d(dX), _d(dV), _d(dk), _d(ox), _d(ov)),
               "tangent_rollout")
        return ox, ov

    def contact(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        diag = np.empty(self.n_total, np.float64)
        rhs = np.empty((self.n_total, 3), np.float64)
        na = C.c_longlong()
        _check(lib().orc_contact(self.h, _d(x), _d(diag), _d(rhs), C.byref(na)), "contact")
        return diag, rhs, na.value


def mesh_topology(X, F, patch_dim):
    """Edges, grid patches and face ownership lists of one standalone mesh."""
    X = np.ascontiguousarray(X, dtype=np.float64)
    F = np.ascontiguousarray(F, dtype=np.int32)
    nv, nf = X.shape[0], F.shape[0]
    cap_e = 3 * nf
    edges = np.empty((cap_e, 2), np.int32)
    ne, npch = C.c_int(), C.c_int()
    poff = np.empty(nf + 1, np.int32)
    pf = np.empty(nf, np.int32)
    opo = np.empty(nf + 1, np.int32)
    op = np.empty(nv, np.int32)
    oeo = np.empty(nf + 1, np.int32)
    oe = np.empty(cap_e, np.int32)
    _check(lib().orc_mesh_topology(_d(X), nv, _i(F), nf, patch_dim, _i(edges), cap_e, C.byref(ne), _i(poff), nf,
                                   _i(pf), nf, C.byref(npch), _i(opo), _i(op), _i(oeo), _i(oe)), "mesh_topology")
    n_e, n_p = ne.value, npch.value
    patches = [pf[poff[p]:poff[p + 1]].copy() for p in range(n_p)]
    owned_points = [op[opo[f]:opo[f + 1]].copy() for f in range(nf)]
    owned_edges = [oe[oeo[f]:oeo[f + 1]].copy() for f in range(nf)]
    return edges[:n_e].copy(), patches, owned_points, owned_edges


def tet_project(x, idm, w):
    """The oracle's tet strain projection on its own: x (n, 4, 3) positions,
    idm (n, 3, 3) row-major Dm^-1, w (n,) -> (n, 4, 3) = w R G per vertex."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    idm = np.ascontiguousarray(idm, dtype=np.float64)
    w = np.ascontiguousarray(w, dtype=np.float64)
    out = np.empty((x.shape[0], 4, 3), np.float64)
    _check(lib().orc_tet_project(x.shape[0], _d(x), _d(idm), _d(w), _d(out)), "tet_project")
    return out


def tri_project(x, idm, w):
    """The oracle's triangle strain projection on its own: x (n, 3, 3) vertex
    positions, idm (n, 2, 2) row-major Dm^-1, w (n,) -> (n, 3, 3) = w P G per vertex."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    idm = np.ascontiguousarray(idm, dtype=np.float64)
    w = np.ascontiguousarray(w, dtype=np.float64)
    out = np.empty((x.shape[0], 3, 3), np.float64)
    _check(lib().orc_tri_project(x.shape[0], _d(x), _d(idm), _d(w), _d(out)), "tri_project")
    return out


def svd3(F):
    """The oracle's SVD of one 3x3 matrix: (U, s, V), U and V proper rotations,
    the sign of det F on s[2]."""
    F = np.ascontiguousarray(F, dtype=np.float64)
    U, V, sv = np.empty((3, 3)), np.empty((3, 3)), np.empty(3)
    _check(lib().orc_svd3(_d(F), _d(U), _d(sv), _d(V)), "svd3")
    return U, sv, V


def tet_surface(X, T):
    """The oracle's boundary faces of a tet mesh (ascending sorted triple, outward)."""
    X = np.ascontiguousarray(X, dtype=np.float64)
    T = np.ascontiguousarray(T, dtype=np.int32)
    cap = 4 * T.shape[0]
    out = np.empty((cap, 3), np.int32)
    nf = C.c_int()
    _check(lib().orc_tet_surface(_d(X), X.shape[0], _i(T), T.shape[0], _i(out), cap, C.byref(nf)), "tet_surface")
    return out[:nf.value].copy()
