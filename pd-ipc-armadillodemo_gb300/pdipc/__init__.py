"""Python binding of libpdipc.so, the GB300 PD-IPC cloth step.

``Simulator`` mirrors the reference's PD_IPC::PdIpcSimulator lifecycle
(Simulator/PD-IPC/PdIpcSimulator.h): add models, ``initialization()``,
``run(frame)`` / ``animate(frame)``, ``postRun()`` positions,
``saveSimulator(frame)``.  Every call goes through the C ABI in
include/pdipc.h.  There is no fallback: if the CUDA library is missing or no
GB300 is present, construction raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .abi import (PDIPC_ERR_CUDA, PDIPC_ERR_OVERFLOW, PDIPC_OK, PRECISIONS, STATUS_NAMES, ClothOptions,  # noqa: F401
                  Params, SceneModel, Stats, Tuning, default_params, params_for_scene)
from . import scenes  # noqa: F401

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_DIR, "libpdipc.so")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_i64p = C.POINTER(C.c_int64)
_lib = None

# every entry point declared in include/pdipc.h
EXPORTS = [
    "pdipc_default_params", "pdipc_create", "pdipc_add_cloth", "pdipc_add_static", "pdipc_initialize",
    "pdipc_step", "pdipc_animate", "pdipc_get_positions", "pdipc_get_velocities", "pdipc_set_state",
    "pdipc_reset", "pdipc_get_stats", "pdipc_save", "pdipc_load", "pdipc_destroy", "pdipc_status_string",
    "pdipc_last_error", "pdipc_abi_version", "pdipc_stage_broadphase", "pdipc_stage_morton", "pdipc_stage_toi",
    "pdipc_stage_contact", "pdipc_stage_pd", "pdipc_mesh_topology",
    "pdipc_stage_sweep_timing", "pdipc_stage_toi_noalloc", "pdipc_add_volumetric", "pdipc_tet_surface",
    "pdipc_scene_load", "pdipc_scene_model_count", "pdipc_scene_get_model", "pdipc_scene_apply_params",
    "pdipc_scene_add_models", "pdipc_scene_free", "pdipc_stage_penalty_predict", "pdipc_stage_penalty_ccd",
    "pdipc_stage_penalty_floor", "pdipc_stage_penalty_dcd", "pdipc_adjoint_record", "pdipc_adjoint_backward",
    "pdipc_set_wait_limit", "pdipc_stage_local_timing", "pdipc_get_tuning", "pdipc_add_cloth_ex",
    "pdipc_stretch_gradient_per_triangle", "pdipc_partition_instances",
]


ABI_VERSION = 9  # PDIPC_ABI_VERSION of include/pdipc.h


class PdipcError(RuntimeError):
    def __init__(self, status: int, what: str, detail: str = ""):
        self.status = status
        msg = f"{what}: {STATUS_NAMES.get(status, status)}"
        if detail:
            msg += f" ({detail})"
        super().__init__(msg)


def load_library(path: str | None = None):
    """Load libpdipc.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise ImportError(f"{path} not built: run __graft_entry__.build() or pdipc/build.py")
    L = C.CDLL(path)
    vp = C.c_void_p
    L.pdipc_default_params.argtypes = [C.POINTER(Params)]
    L.pdipc_default_params.restype = None
    L.pdipc_create.argtypes = [C.POINTER(Params), C.POINTER(vp)]
    L.pdipc_add_cloth.argtypes = [vp, _dp, C.c_int, _ip, C.c_int, C.c_double, C.c_double, C.c_double, _ip,
                                  C.c_int, C.c_double, C.c_int]
    L.pdipc_add_cloth_ex.argtypes = [vp, _dp, C.c_int, _ip, C.c_int, C.c_double, C.c_double, C.c_double, _ip,
                                     C.c_int, C.c_double, C.c_int, C.POINTER(ClothOptions)]
    L.pdipc_stretch_gradient_per_triangle.argtypes = [vp, C.c_int, _dp, _dp]
    L.pdipc_partition_instances.argtypes = [_i64p, C.c_int, C.c_int, _ip]
    L.pdipc_add_static.argtypes = [vp, _dp, C.c_int, _ip, C.c_int, C.c_int]
    L.pdipc_tet_surface.argtypes = [_dp, C.c_int, _ip, C.c_int, _ip, C.c_int, _ip]
    L.pdipc_scene_load.argtypes = [C.c_char_p, C.POINTER(vp), C.c_char_p, C.c_int]
    L.pdipc_scene_model_count.argtypes = [vp]
    L.pdipc_scene_model_count.restype = C.c_int
    L.pdipc_scene_get_model.argtypes = [vp, C.c_int, C.POINTER(SceneModel)]
    L.pdipc_scene_apply_params.argtypes = [vp, C.POINTER(Params)]
    L.pdipc_scene_add_models.argtypes = [vp, vp]
    L.pdipc_scene_free.argtypes = [vp]
    L.pdipc_scene_free.restype = None
    L.pdipc_add_volumetric.argtypes = [vp, _dp, C.c_int, _ip, C.c_int, C.c_double, C.c_double, C.c_double, _ip,
                                       C.c_int, C.c_double, C.c_int]
    L.pdipc_initialize.argtypes = [vp]
    L.pdipc_step.argtypes = [vp, C.c_int]
    L.pdipc_set_wait_limit.argtypes = [vp, C.c_int]
    L.pdipc_animate.argtypes = [vp, _dp]
    L.pdipc_get_positions.argtypes = [vp, _dp]
    L.pdipc_get_velocities.argtypes = [vp, _dp]
    L.pdipc_set_state.argtypes = [vp, _dp, _dp]
    L.pdipc_reset.argtypes = [vp]
    L.pdipc_get_stats.argtypes = [vp, C.POINTER(Stats)]
    L.pdipc_get_tuning.argtypes = [vp, C.POINTER(Tuning)]
    L.pdipc_save.argtypes = [vp, C.c_char_p]
    L.pdipc_load.argtypes = [vp, C.c_char_p]
    L.pdipc_destroy.argtypes = [vp]
    L.pdipc_destroy.restype = None
    L.pdipc_status_string.argtypes = [C.c_int]
    L.pdipc_status_string.restype = C.c_char_p
    L.pdipc_last_error.argtypes = [vp]
    L.pdipc_last_error.restype = C.c_char_p
    L.pdipc_abi_version.restype = C.c_int
    L.pdipc_stage_broadphase.argtypes = [vp, _dp, _dp, _ip, C.c_int64, _i64p, _ip, C.c_int64, _i64p, _ip,
                                         C.c_int64, _i64p]
    L.pdipc_stage_morton.argtypes = [vp, C.POINTER(C.c_uint64), _ip, C.c_int]
    L.pdipc_stage_toi.argtypes = [vp, _dp, _dp, _dp, _dp, _dp]
    L.pdipc_stage_penalty_predict.argtypes = [vp, _dp, _dp, _dp]
    L.pdipc_stage_penalty_ccd.argtypes = [vp, _dp, _dp, C.c_double, C.c_double, _dp, _dp, _ip]
    L.pdipc_stage_penalty_floor.argtypes = [vp, _dp, C.c_double, C.c_double, _dp, _dp, _ip]
    L.pdipc_stage_penalty_dcd.argtypes = [vp, _dp, _ip, C.c_int64, C.c_double, C.c_double, C.c_double, _dp, _dp,
                                          _ip]
    L.pdipc_stage_toi_noalloc.argtypes = [vp, _dp, _dp, _dp, _dp, _dp]
    L.pdipc_adjoint_record.argtypes = [vp, C.c_int]
    L.pdipc_adjoint_backward.argtypes = [vp, _dp, _dp, _dp, _dp, _dp]
    L.pdipc_stage_contact.argtypes = [vp, _dp, _dp, _dp, _i64p]
    L.pdipc_stage_pd.argtypes = [vp, _dp, _dp, _dp]
    L.pdipc_stage_sweep_timing.argtypes = [vp, C.c_int, _dp, _dp]
    L.pdipc_stage_local_timing.argtypes = [vp, C.c_int, _dp, _dp]
    L.pdipc_mesh_topology.argtypes = [_dp, C.c_int, _ip, C.c_int, C.c_int, _ip, C.c_int, _ip, _ip, C.c_int, _ip,
                                      C.c_int, _ip, _ip, _ip]
    if L.pdipc_abi_version() != ABI_VERSION:
        raise ImportError(f"{path}: ABI version {L.pdipc_abi_version()}, this binding expects {ABI_VERSION}; "
                          "rebuild the library")
    _lib = L
    return L


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


class Simulator:
    """One PD-IPC context (one CUDA stream, all its device memory) on one GPU."""

    def __init__(self, scene=None, precision="fp32", params: Params | None = None, initialize=True, **overrides):
        L = load_library()
        if params is None:
            params = params_for_scene(scene, precision, **overrides) if scene is not None else default_params()
        self.params = params
        self.h = C.c_void_p()
        rc = L.pdipc_create(C.byref(params), C.byref(self.h))
        if rc != PDIPC_OK:
            self.h = None
            raise PdipcError(rc, "pdipc_create", "no usable GB300 (sm_103) device" if rc == PDIPC_ERR_CUDA else "")
        self.n_sim = 0
        self.n_total = 0
        self.cloth_faces = []
        if scene is not None:
            for c in scene.cloths:
                self.add_cloth(c.X, c.F, c.pins, c.density, c.k_stretch, c.k_bend, c.k_pin, c.patch_dim,
                               tri_stretch=getattr(c, "tri_stretch", None), k_tri_strain=getattr(c, "k_tri_strain", 0.0),
                               tri_strain=getattr(c, "tri_strain", None))
            for v in getattr(scene, "solids", []):
                self.add_volumetric(v.X, v.T, v.pins, v.density, v.k_strain, v.k_volume, v.k_pin, v.patch_dim)
            for s in scene.statics:
                self.add_static(s.X, s.F, s.patch_dim)
            if initialize:
                self.initialization()

    # -- lifecycle -------------------------------------------------------------------------
    def _check(self, rc, what):
        if rc != PDIPC_OK:
            detail = load_library().pdipc_last_error(self.h).decode(errors="replace") if self.h else ""
            raise PdipcError(rc, what, detail)

    def add_cloth(self, X, F, pins=(), density=0.1, k_stretch=1e4, k_bend=1e-3, k_pin=1e6, patch_dim=10,
                  tri_stretch=None, k_tri_strain=0.0, tri_strain=None):
        """pdipc_add_cloth_ex: optional per-triangle stretch stiffness (nf), and a
        triangle strain limit (weight k_tri_strain, or per-triangle tri_strain,
        times rest area)."""
        X = np.ascontiguousarray(X, dtype=np.float64)
        F = np.ascontiguousarray(F, dtype=np.int32)
        P = np.ascontiguousarray(pins, dtype=np.int32)
        opt = ClothOptions()
        keep = []
        if tri_stretch is not None:
            ts = np.ascontiguousarray(tri_stretch, dtype=np.float64).reshape(F.shape[0])
            keep.append(ts)
            opt.per_tri_stretch = _d(ts)
        opt.k_tri_strain = float(k_tri_strain)
        if tri_strain is not None:
            tk = np.ascontiguousarray(tri_strain, dtype=np.float64).reshape(F.shape[0])
            keep.append(tk)
            opt.per_tri_strain = _d(tk)
        self._check(load_library().pdipc_add_cloth_ex(self.h, _d(X), X.shape[0], _i(F), F.shape[0], density,
                                                      k_stretch, k_bend, _i(P), P.shape[0], k_pin, patch_dim,
                                                      C.byref(opt)), "pdipc_add_cloth_ex")
        self.cloth_faces.append(F.shape[0])
        self.n_sim += X.shape[0]
        self.n_total += X.shape[0]

    def stretch_gradient_per_triangle(self, dl_dvertex, cloth_index=0):
        """dL/d(per-triangle stretch stiffness) of one cloth from dL/d(per-vertex
        stretch stiffness) (pdipc_stretch_gradient_per_triangle)."""
        g = np.ascontiguousarray(dl_dvertex, dtype=np.float64).reshape(self.n_sim)
        out = np.empty(self.cloth_faces[cloth_index], np.float64)
        self._check(load_library().pdipc_stretch_gradient_per_triangle(self.h, int(cloth_index), _d(g), _d(out)),
                    "pdipc_stretch_gradient_per_triangle")
        return out

    def add_volumetric(self, X, T, pins=(), density=1000.0, k_strain=1e6, k_volume=1e3, k_pin=1e12, patch_dim=10):
        X = np.ascontiguousarray(X, dtype=np.float64)
        T = np.ascontiguousarray(T, dtype=np.int32)
        P = np.ascontiguousarray(pins, dtype=np.int32)
        self._check(load_library().pdipc_add_volumetric(self.h, _d(X), X.shape[0], _i(T), T.shape[0], density,
                                                        k_strain, k_volume, _i(P), P.shape[0], k_pin, patch_dim),
                    "pdipc_add_volumetric")
        self.n_sim += X.shape[0]
        self.n_total += X.shape[0]

    def add_static(self, X, F, patch_dim=10):
        X = np.ascontiguousarray(X, dtype=np.float64)
        F = np.ascontiguousarray(F, dtype=np.int32)
        self._check(load_library().pdipc_add_static(self.h, _d(X), X.shape[0], _i(F), F.shape[0], patch_dim),
                    "pdipc_add_static")
        self.n_total += X.shape[0]

    def initialization(self):
        self._check(load_library().pdipc_initialize(self.h), "pdipc_initialize")
        self._pos = np.empty((self.n_total, 3), np.float64)

    def run(self, nsteps: int = 1):
        self._check(load_library().pdipc_step(self.h, int(nsteps)), "pdipc_step")

    step = run

    def set_wait_limit(self, us: int):
        """Limit of the persistent solve's device-side waits in microseconds (0 = 2 s)."""
        self._check(load_library().pdipc_set_wait_limit(self.h, int(us)), "pdipc_set_wait_limit")

    def animate(self, out: np.ndarray | None = None) -> np.ndarray:
        """run(frame); postRun(): one step and the positions copied to the host."""
        out = self._pos if out is None else out
        if out.shape != (self.n_total, 3) or out.dtype != np.float64 or not out.flags.c_contiguous:
            raise ValueError(f"animate: out must be a C-contiguous float64 array of shape ({self.n_total}, 3)")
        self._check(load_library().pdipc_animate(self.h, _d(out)), "pdipc_animate")
        return out

    def positions(self) -> np.ndarray:
        out = np.empty((self.n_total, 3), np.float64)
        self._check(load_library().pdipc_get_positions(self.h, _d(out)), "pdipc_get_positions")
        return out

    def velocities(self) -> np.ndarray:
        out = np.empty((self.n_sim, 3), np.float64)
        self._check(load_library().pdipc_get_velocities(self.h, _d(out)), "pdipc_get_velocities")
        return out

    def _vec(self, A, n, what):
        A = np.ascontiguousarray(A, dtype=np.float64)
        if A.shape != (n, 3):
            raise ValueError(f"{what}: expected shape ({n}, 3), got {A.shape}")
        return A

    def set_state(self, X, V=None):
        X = self._vec(X, self.n_total, "positions")
        Vp = None
        if V is not None:
            V = self._vec(V, self.n_sim, "velocities")
            Vp = _d(V)
        self._check(load_library().pdipc_set_state(self.h, _d(X), Vp), "pdipc_set_state")

    def reset(self):
        self._check(load_library().pdipc_reset(self.h), "pdipc_reset")

    def stats(self) -> dict:
        s = Stats()
        self._check(load_library().pdipc_get_stats(self.h, C.byref(s)), "pdipc_get_stats")
        return s.as_dict()

    def tuning(self) -> dict:
        """The launch configuration (pdipc_get_tuning): chosen by the autotuner
        when the context was created with autotune=1."""
        t = Tuning()
        self._check(load_library().pdipc_get_tuning(self.h, C.byref(t)), "pdipc_get_tuning")
        return t.as_dict()

    def save(self, path: str):
        self._check(load_library().pdipc_save(self.h, path.encode()), "pdipc_save")

    def load(self, path: str):
        self._check(load_library().pdipc_load(self.h, path.encode()), "pdipc_load")

    def close(self):
        if self.h:
            load_library().pdipc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- stages ----------------------------------------------------------------------------
    def stage_broadphase(self, x_old, dx, cap=1 << 16):
        x_old = self._vec(x_old, self.n_total, "x_old")
        dx = self._vec(dx, self.n_total, "dx")
        n1, n2, n3 = C.c_int64(), C.c_int64(), C.c_int64()
        L = load_library()
        while True:
            pairs = np.empty((cap, 2), np.int32)
            pt = np.empty((cap, 4), np.int32)
            ee = np.empty((cap, 4), np.int32)
            rc = L.pdipc_stage_broadphase(self.h, _d(x_old), _d(dx), _i(pairs), cap, C.byref(n1), _i(pt), cap,
                                          C.byref(n2), _i(ee), cap, C.byref(n3))
            if rc == PDIPC_ERR_OVERFLOW:
                cap = max(n1.value, n2.value, n3.value)
                continue
            self._check(rc, "pdipc_stage_broadphase")
            return pairs[:n1.value].copy(), pt[:n2.value].copy(), ee[:n3.value].copy()

    def stage_morton(self, npatch):
        codes = np.empty(max(npatch, 1), np.uint64)
        order = np.empty(max(npatch, 1), np.int32)
        self._check(load_library().pdipc_stage_morton(self.h, codes.ctypes.data_as(C.POINTER(C.c_uint64)),
                                                      _i(order), npatch), "pdipc_stage_morton")
        return codes[:npatch], order[:npatch]

    def stage_toi(self, x0, x1, npt, nee):
        x0 = self._vec(x0, self.n_total, "x0")
        x1 = self._vec(x1, self.n_total, "x1")
        tp = np.empty(max(npt, 1), np.float64)
        te = np.empty(max(nee, 1), np.float64)
        g = C.c_double()
        self._check(load_library().pdipc_stage_toi(self.h, _d(x0), _d(x1), _d(tp), _d(te), C.byref(g)),
                    "pdipc_stage_toi")
        return tp[:npt], te[:nee], g.value

    # -- penalty / discrete-collision stages (PdIpcGpuFunc.cu:2933-3740) -------------------
    def penalty_predict(self, X, V):
        """prediticeDCPositionKernel: predicted positions sn (n_sim x 3) and the velocities
        (pinned ones zeroed)."""
        X = self._vec(X, self.n_sim, "X")
        V = self._vec(V, self.n_sim, "V").copy()
        sn = np.empty((self.n_sim, 3), np.float64)
        self._check(load_library().pdipc_stage_penalty_predict(self.h, _d(X), _d(V), _d(sn)),
                    "pdipc_stage_penalty_predict")
        return sn, V

    def _penalty_out(self, V):
        V = self._vec(V, self.n_sim, "V").copy()
        return V, np.empty((self.n_total, 3), np.float64), np.empty(self.n_total, np.int32)

    def penalty_ccd(self, x0, d, stiffness, damping, V):
        """computePenaltyForceHost over the candidates of the last broad phase: (force, hits, V)."""
        x0 = self._vec(x0, self.n_total, "x0")
        d = self._vec(d, self.n_total, "dir")
        V, F, t = self._penalty_out(V)
        self._check(load_library().pdipc_stage_penalty_ccd(self.h, _d(x0), _d(d), stiffness, damping, _d(V),
                                                           _d(F), _i(t)), "pdipc_stage_penalty_ccd")
        return F, t, V

    def penalty_floor(self, x, stiffness, damping, V):
        """applyPenaltyForceForFloorHost: (force, hits, V)."""
        x = self._vec(x, self.n_total, "x")
        V, F, t = self._penalty_out(V)
        self._check(load_library().pdipc_stage_penalty_floor(self.h, _d(x), stiffness, damping, _d(V), _d(F),
                                                             _i(t)), "pdipc_stage_penalty_floor")
        return F, t, V

    def penalty_dcd(self, x, face_pairs, stiffness, self_stiffness, damping, V):
        """computeDcdPenaltyForceHost over face pairs (m x 2 collision-face indices): (force, hits, V)."""
        x = self._vec(x, self.n_total, "x")
        fp = np.ascontiguousarray(face_pairs, dtype=np.int32).reshape(-1, 2)
        V, F, t = self._penalty_out(V)
        self._check(load_library().pdipc_stage_penalty_dcd(self.h, _d(x), _i(fp) if fp.size else None,
                                                           fp.shape[0], stiffness, self_stiffness, damping,
                                                           _d(V), _d(F), _i(t)), "pdipc_stage_penalty_dcd")
        return F, t, V

    def adjoint_record(self, checkpoint_every=1):
        """Record the following steps for adjoint_backward, keeping a checkpoint
        every `checkpoint_every` steps (0 drops the recording)."""
        self._check(load_library().pdipc_adjoint_record(self.h, int(checkpoint_every)), "pdipc_adjoint_record")

    def adjoint_backward(self, dl_dx, dl_dv=None):
        """Gradients through the recorded steps: given dL/d(positions) and
        dL/d(velocities) of the simulated vertices after the last recorded step,
        return dL/d(positions), dL/d(velocities) before the first one and
        dL/d(stretch stiffness) per simulated vertex."""
        gx = self._vec(dl_dx, self.n_sim, "dl_dx")
        gv = None if dl_dv is None else self._vec(dl_dv, self.n_sim, "dl_dv")
        gx0 = np.empty((self.n_sim, 3), np.float64)
        gv0 = np.empty((self.n_sim, 3), np.float64)
        gk = np.empty(self.n_sim, np.float64)
        self._check(load_library().pdipc_adjoint_backward(self.h, _d(gx), _d(gv) if gv is not None else None,
                                                          _d(gx0), _d(gv0), _d(gk)), "pdipc_adjoint_backward")
        return gx0, gv0, gk

    def stage_toi_noalloc(self, x0, x1, npt, nee, per_candidate=True):
        """stage_toi through the no-allocation entry point (FP64 and mixed modes)."""
        x0 = self._vec(x0, self.n_total, "x0")
        x1 = self._vec(x1, self.n_total, "x1")
        tp = np.empty(max(npt, 1), np.float64) if per_candidate else None
        te = np.empty(max(nee, 1), np.float64) if per_candidate else None
        g = C.c_double()
        self._check(load_library().pdipc_stage_toi_noalloc(self.h, _d(x0), _d(x1), _d(tp) if per_candidate else None,
                                                           _d(te) if per_candidate else None, C.byref(g)),
                    "pdipc_stage_toi_noalloc")
        if not per_candidate:
            return None, None, g.value
        return tp[:npt], te[:nee], g.value

    def stage_contact(self, x):
        x = self._vec(x, self.n_total, "x")
        diag = np.empty(self.n_total, np.float64)
        rhs = np.empty((self.n_total, 3), np.float64)
        na = C.c_int64()
        self._check(load_library().pdipc_stage_contact(self.h, _d(x), _d(diag), _d(rhs), C.byref(na)),
                    "pdipc_stage_contact")
        return diag, rhs, na.value

    def sweep_timing(self, launches=200):
        """(mean ms per launch, algorithmic bytes per launch) of the J sweep kernel."""
        ms, b = C.c_double(), C.c_double()
        self._check(load_library().pdipc_stage_sweep_timing(self.h, int(launches), C.byref(ms), C.byref(b)),
                    "pdipc_stage_sweep_timing")
        return ms.value, b.value

    def local_timing(self, launches=200):
        """(mean ms, algorithmic bytes) of one local step of the per-sweep path."""
        ms, b = C.c_double(), C.c_double()
        self._check(load_library().pdipc_stage_local_timing(self.h, int(launches), C.byref(ms), C.byref(b)),
                    "pdipc_stage_local_timing")
        return ms.value, b.value

    def stage_pd(self, X, V):
        X = self._vec(X, self.n_total, "X")
        V = self._vec(V, self.n_sim, "V")
        out = np.empty((self.n_total, 3), np.float64)
        self._check(load_library().pdipc_stage_pd(self.h, _d(X), _d(V), _d(out)), "pdipc_stage_pd")
        return out


def mesh_topology(X, F, patch_dim):
    """Edges, grid patches and owner faces of one mesh (host precompute of the library)."""
    X = np.ascontiguousarray(X, dtype=np.float64)
    F = np.ascontiguousarray(F, dtype=np.int32)
    nv, nf = X.shape[0], F.shape[0]
    cap_e = 3 * nf
    edges = np.empty((cap_e, 2), np.int32)
    poff = np.empty(nf + 1, np.int32)
    pf = np.empty(nf, np.int32)
    own_p = np.full(nv, -1, np.int32)
    own_e = np.full(cap_e, -1, np.int32)
    ne, npch = C.c_int(), C.c_int()
    rc = load_library().pdipc_mesh_topology(_d(X), nv, _i(F), nf, patch_dim, _i(edges), cap_e, C.byref(ne),
                                            _i(poff), nf, _i(pf), nf, C.byref(npch), _i(own_p), _i(own_e))
    if rc != PDIPC_OK:
        raise PdipcError(rc, "pdipc_mesh_topology")
    n_e, n_p = ne.value, npch.value
    patches = [pf[poff[p]:poff[p + 1]].copy() for p in range(n_p)]
    return edges[:n_e].copy(), patches, own_p, own_e[:n_e].copy()


def partition_instances(sizes, ranks: int) -> np.ndarray:
    """pdipc_partition_instances (host only): instance ranges [first[r], first[r+1])
    of `ranks` processes balancing the cumulative simulated-vertex counts."""
    s = np.ascontiguousarray(sizes, dtype=np.int64)
    first = np.empty(ranks + 1, np.int32)
    rc = load_library().pdipc_partition_instances(s.ctypes.data_as(_i64p), int(s.shape[0]), int(ranks), _i(first))
    if rc != PDIPC_OK:
        raise PdipcError(rc, "pdipc_partition_instances")
    return first


def create_simulator(sim_name: str, scene=None, **kw):
    """createSimulator(simName, platform) (Simulator/SimulatorFactor.h:13-57): only
    "pd_ipc_simulator" is provided by this library."""
    if sim_name != "pd_ipc_simulator":
        raise ValueError(f"unknown simulator {sim_name!r}; this library provides 'pd_ipc_simulator'")
    return Simulator(scene, **kw)


def tet_surface(X, T):
    """Boundary faces of a tetrahedral mesh (pdipc_tet_surface; host only)."""
    X = np.ascontiguousarray(X, dtype=np.float64)
    T = np.ascontiguousarray(T, dtype=np.int32)
    cap = 4 * T.shape[0]
    out = np.empty((cap, 3), np.int32)
    nf = C.c_int()
    rc = load_library().pdipc_tet_surface(_d(X), X.shape[0], _i(T), T.shape[0], _i(out), cap, C.byref(nf))
    if rc != PDIPC_OK:
        raise PdipcError(rc, "pdipc_tet_surface")
    return out[:nf.value].copy()


def read_scene(config_path: str, lg_iterations: int = 10):
    """A reference config.xml (and the mesh files beside it) as a scenes.Scene,
    read by the library's host reader (pdipc_scene_load).  Cloths come first,
    then volumetric models, then static ones, each group in file order."""
    L = load_library()
    h = C.c_void_p()
    err = C.create_string_buffer(512)
    rc = L.pdipc_scene_load(config_path.encode(), C.byref(h), err, 512)
    if rc != PDIPC_OK:
        raise PdipcError(rc, "pdipc_scene_load", err.value.decode(errors="replace"))
    try:
        p = default_params()
        L.pdipc_scene_apply_params(h, C.byref(p))
        cloths, solids, statics = [], [], []
        for i in range(L.pdipc_scene_model_count(h)):
            m = SceneModel()
            L.pdipc_scene_get_model(h, i, C.byref(m))
            X = np.ctypeslib.as_array(m.X, (m.nv, 3)).copy()
            F = np.ctypeslib.as_array(m.F, (m.nf, 3)).copy()
            pins = np.ctypeslib.as_array(m.pins, (m.npins,)).copy() if m.npins else np.zeros(0, np.int32)
            if m.kind == 0:
                cloths.append(scenes.ClothSpec(X, F, pins.astype(np.int32), m.density, m.k[0], m.k[1], m.k[2],
                                               m.patch_dim))
            elif m.kind == 1:
                T = np.ctypeslib.as_array(m.T, (m.nt, 4)).copy()
                solids.append(scenes.SolidSpec(X, T, pins.astype(np.int32), m.density, m.k[0], m.k[1], m.k[2],
                                               m.patch_dim))
            else:
                statics.append(scenes.StaticSpec(X, F, m.patch_dim))
        name = os.path.basename(os.path.dirname(os.path.abspath(config_path)))
        return scenes.Scene(name, cloths, statics, dt=p.time_step, gravity=p.gravity, dhat=p.dhat, kappa=p.kappa,
                            lg_iterations=lg_iterations, solids=solids)
    finally:
        L.pdipc_scene_free(h)
