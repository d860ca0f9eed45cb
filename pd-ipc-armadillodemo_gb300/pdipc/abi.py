"""ctypes mirror of the structs and enums in include/pdipc.h.

Kept separate from the library loader so the CPU oracle wrapper can reuse the
exact same struct layout without loading the CUDA library.
"""
import ctypes as C

PDIPC_OK = 0
PDIPC_ERR_ARG = 1
PDIPC_ERR_CUDA = 2
PDIPC_ERR_OVERFLOW = 3
PDIPC_ERR_NONFINITE = 4
PDIPC_ERR_NOT_CONVERGED = 5
PDIPC_ERR_STATE = 6
PDIPC_ERR_ALLOC = 7
PDIPC_ERR_IO = 8

STATUS_NAMES = {
    0: "PDIPC_OK", 1: "PDIPC_ERR_ARG", 2: "PDIPC_ERR_CUDA", 3: "PDIPC_ERR_OVERFLOW",
    4: "PDIPC_ERR_NONFINITE", 5: "PDIPC_ERR_NOT_CONVERGED", 6: "PDIPC_ERR_STATE",
    7: "PDIPC_ERR_ALLOC", 8: "PDIPC_ERR_IO",
}

PREC_FP32 = 0
PREC_FP64 = 1
PREC_MIXED = 2
PRECISIONS = {"fp32": PREC_FP32, "fp64": PREC_FP64, "mixed": PREC_MIXED}


class Params(C.Structure):
    _fields_ = [
        ("time_step", C.c_double),
        ("gravity", C.c_double),
        ("dhat", C.c_double),
        ("kappa", C.c_double),
        ("inflation_radius", C.c_double),
        ("lg_iterations", C.c_int),
        ("cheby_iterations", C.c_int),
        ("cheby_rho", C.c_double),
        ("jacobi_relax", C.c_double),
        ("max_outer", C.c_int),
        ("outer_tol", C.c_double),
        ("ccd_slack", C.c_double),
        ("toi_scale", C.c_double),
        ("ccd_max_iter", C.c_int),
        ("ccd_eta", C.c_double),
        ("static_mass", C.c_double),
        ("precision", C.c_int),
        ("fixed_outer", C.c_int),
        ("use_graphs", C.c_int),
        ("device", C.c_int),
        ("rebuild_bvh", C.c_int),
        ("persistent", C.c_int),
        ("wait_limit_us", C.c_int),
        ("autotune", C.c_int),
        ("ccd_mode", C.c_int),
        ("instance_stop", C.c_int),
        ("pd_group_ctas", C.c_int),
        ("reserved", C.c_int * 1),
    ]


def default_params() -> Params:
    """The reference constants (mirrors pdipc_default_params)."""
    p = Params()
    p.time_step = 0.01
    p.gravity = -9.8
    p.dhat = 1e-3
    p.kappa = 1e4
    p.inflation_radius = -1.0
    p.lg_iterations = 10
    p.cheby_iterations = 15
    p.cheby_rho = 0.9992
    p.jacobi_relax = 2.0 / 3.0
    p.max_outer = 30
    p.outer_tol = 1e-5
    p.ccd_slack = 5e-3
    p.toi_scale = 0.98
    p.ccd_max_iter = 10
    p.ccd_eta = 0.1
    p.static_mass = 1e4
    p.precision = PREC_FP32
    p.fixed_outer = 0
    p.use_graphs = 1
    p.device = 0
    p.rebuild_bvh = 0
    p.persistent = 1
    return p


def params_for_scene(scene, precision="fp32", **overrides) -> Params:
    p = default_params()
    p.time_step = scene.dt
    p.gravity = scene.gravity
    p.dhat = scene.dhat
    p.kappa = scene.kappa
    p.lg_iterations = scene.lg_iterations
    p.precision = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
    for k, v in overrides.items():
        setattr(p, k, v)
    return p


class ClothOptions(C.Structure):
    """pdipc_cloth_options of pdipc_add_cloth_ex."""
    _fields_ = [
        ("per_tri_stretch", C.POINTER(C.c_double)),
        ("k_tri_strain", C.c_double),
        ("per_tri_strain", C.POINTER(C.c_double)),
        ("reserved", C.c_int32 * 8),
    ]


class SceneModel(C.Structure):
    _fields_ = [
        ("name", C.c_char_p),
        ("kind", C.c_int),
        ("nv", C.c_int),
        ("nf", C.c_int),
        ("nt", C.c_int),
        ("npins", C.c_int),
        ("X", C.POINTER(C.c_double)),
        ("F", C.POINTER(C.c_int)),
        ("T", C.POINTER(C.c_int)),
        ("pins", C.POINTER(C.c_int)),
        ("density", C.c_double),
        ("k", C.c_double * 3),
        ("patch_dim", C.c_int),
    ]


class Stats(C.Structure):
    _fields_ = [
        ("steps_done", C.c_int64),
        ("last_outer_iters", C.c_int32),
        ("max_outer_iters", C.c_int32),
        ("total_outer_iters", C.c_int64),
        ("patch_pairs", C.c_int64),
        ("pt_candidates", C.c_int64),
        ("ee_candidates", C.c_int64),
        ("active_contacts", C.c_int64),
        ("last_toi", C.c_double),
        ("last_residual", C.c_double),
        ("n_sim", C.c_int32),
        ("n_total", C.c_int32),
        ("n_patches", C.c_int32),
        ("precision", C.c_int32),
        ("device_bytes", C.c_int64),
        ("kernel_launches", C.c_int64),
        ("device_ms", C.c_double),
        ("pd_path", C.c_int32),
        ("pd_ctas", C.c_int32),
        ("pd_solves", C.c_int64),
        ("pd_solve_ms", C.c_double),
        ("pd_solve_bytes", C.c_double),
        ("ccd_ms", C.c_double),
        ("contact_ms", C.c_double),
        ("instances", C.c_int32),
        ("reserved_i", C.c_int32),
        ("instance_outer_iters", C.c_int64),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class Tuning(C.Structure):
    """pdipc_tuning: the launch configuration of a context and how it was chosen."""
    _fields_ = [
        ("autotuned", C.c_int32),
        ("from_cache", C.c_int32),
        ("pd_rows_per_thread", C.c_int32),
        ("pd_ctas", C.c_int32),
        ("pd_band", C.c_int32),
        ("pd_l1_gather", C.c_int32),
        ("pd_local_sync", C.c_int32),
        ("cand_grid", C.c_int32),
        ("traverse_block", C.c_int32),
        ("expand_block", C.c_int32),
        ("candidates_timed", C.c_int32),
        ("pd_launches", C.c_int32),
        ("pd_solve_ms", C.c_double),
        ("pd_default_ms", C.c_double),
        ("collision_ms", C.c_double),
        ("collision_default_ms", C.c_double),
        ("reserved", C.c_int32 * 8),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_ if not name.startswith("reserved")}
