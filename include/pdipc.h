/*
 * pdipc.h — C ABI of the GB300 PD-IPC cloth time step (libpdipc.so).
 *
 * The reference exposes this path as a C++ virtual class, not as an FFI:
 *   BaseSimulator / PD_IPC::PdIpcSimulator   (Simulator/BaseSimulator.h:32-136,
 *                                             Simulator/PD-IPC/PdIpcSimulator.h:441-642)
 * created through the factory createSimulator("pd_ipc_simulator", ...)
 * (Simulator/SimulatorFactor.h:13-57).  Each entry point below replaces one
 * member of that class; the citation on each names it.  A header-only C++
 * class with the reference's member names sits on top of this ABI in
 * include/pdipc_simulator.hpp.
 *
 * Conventions
 *   - plain pointers and sizes; no C++ or torch types cross the boundary;
 *   - every call returns a pdipc_status, no exceptions escape;
 *   - a context owns one CUDA stream and all of its device memory; contexts
 *     are independent, calls on one context are not re-entrant;
 *   - positions cross the boundary as float64 xyz triplets whatever the
 *     precision mode; vertex order is every cloth (sim) model in the order
 *     added, then every static model in the order added — the reference's
 *     devPoints layout (PdIpcSimulator.cpp:34-200);
 *   - there is no CPU fallback: without a usable GB300 (sm_103) pdipc_create
 *     fails with PDIPC_ERR_CUDA.
 */
#ifndef PDIPC_H
#define PDIPC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PDIPC_ABI_VERSION 9

typedef struct pdipc_ctx pdipc_ctx;

typedef enum {
    PDIPC_OK = 0,
    PDIPC_ERR_ARG = 1,           /* bad argument (null, size, index out of range) */
    PDIPC_ERR_CUDA = 2,          /* CUDA runtime error or no suitable device */
    PDIPC_ERR_OVERFLOW = 3,      /* a bounded device buffer or loop overflowed */
    PDIPC_ERR_NONFINITE = 4,     /* NaN/Inf appeared in the state */
    PDIPC_ERR_NOT_CONVERGED = 5, /* reserved: outer loop hit its cap in strict mode */
    PDIPC_ERR_STATE = 6,         /* call out of order (e.g. step before initialize) */
    PDIPC_ERR_ALLOC = 7,         /* host or device allocation failed */
    PDIPC_ERR_IO = 8             /* checkpoint file could not be read or written */
} pdipc_status;

typedef enum {
    PDIPC_PREC_FP32 = 0,  /* every kernel in float: the reference's own arithmetic (DataCore.h:8,19) */
    PDIPC_PREC_FP64 = 1,  /* every kernel in double: the plain FP64 GPU form */
    PDIPC_PREC_MIXED = 2  /* double state (positions, velocities, step direction, toi); float local step,
                             residual terms and sweeps on the correction; float CCD filter with double
                             re-evaluation of clamping candidates; double contact distances */
} pdipc_precision;

/* Solver parameters.  Defaults (pdipc_default_params) are the reference's
 * constants; each field names where the reference fixes it. */
typedef struct {
    double time_step;        /* _timeStep, BaseSimulator.h:37 (config <timeStep>) */
    double gravity;          /* _gravity along y, BaseSimulator.h:38 (-9.8) */
    double dhat;             /* dHat, PdIpcSimulator.h:444 (1e-3) */
    double kappa;            /* barrier stiffness, PdIpcSimulator.h:445 (1e4) */
    double inflation_radius; /* patch AABB inflation; <0 means 0.5*dhat (PdIpcSimulator.cpp:1154) */
    int lg_iterations;       /* local-global iterations per outer iteration, cpp:1592 (10) */
    int cheby_iterations;    /* R2 sweeps per global step, cpp:1597 (15) */
    double cheby_rho;        /* spectral radius estimate, PdIpcGpuFunc.cu:1318 (0.9992) */
    double jacobi_relax;     /* weighted-Jacobi w, PdIpcGpuFunc.cu:949,1051 (2/3) */
    int max_outer;           /* outer CCD iterations cap, cpp:1685 (30) */
    double outer_tol;        /* stop when ||dx||^2 < tol (after the first), cpp:1776 (1e-5) */
    double ccd_slack;        /* per-pair swept-AABB slack, PdIpcGpuFunc.cu:2656,2676 (5e-3) */
    double toi_scale;        /* applied to toi < 1, PdIpcGpuFunc.cu:2698-2699 (0.98) */
    int ccd_max_iter;        /* additive-CCD iterations, PdIpcGpuFunc.cu:2493 (10) */
    double ccd_eta;          /* additive-CCD gap fraction, PdIpcGpuFunc.cu:2488 (0.1) */
    double static_mass;      /* collision mass of static vertices, cpp:1494 (1e4) */
    int precision;           /* pdipc_precision (FP32) */
    int fixed_outer;         /* 0: reference stopping rule; >0: run exactly this many outer iterations */
    int use_graphs;          /* 1: replay each outer iteration's PD solve as a CUDA graph */
    int device;              /* CUDA device ordinal */
    int rebuild_bvh;         /* 0: build the patch BVH once at initialize and refit per step
                                (reference behaviour, cpp:1296-1320); 1: rebuild every step */
    int persistent;          /* FP32/mixed PD solve of an outer iteration as one cooperative launch when
                                the mesh allows it (matrix slice per CTA): 1 CTAs wait only for the CTAs
                                they exchange rows with; in mixed precision the CTA's column band of the
                                iterate lives in shared memory when it fits and each sweep sums the
                                entries on the CTA's own rows while the neighbours' rows are copied in
                                (else, and in FP32, gathers through L1); 2 neighbour waits, L2-only
                                gathers; 3 grid-wide barriers, gathers through L1; 4 neighbour waits,
                                gathers through L1 (no band); 0 one launch per sweep */
    int wait_limit_us;       /* limit of every device-side wait of the persistent solve (neighbour flags,
                                grid barrier, halo copies), in microseconds at the maximum SM clock; past
                                it the launch ends and the step returns PDIPC_ERR_CUDA; 0 = 2 s.  The
                                reference has no device-side waits (one launch per kernel). */
    int autotune;            /* 1: choose launch shapes by timing candidates at pdipc_initialize (see
                                pdipc_get_tuning); 0: the built-in defaults */
    int ccd_mode;            /* 0: the reference's additive CCD (PdIpcGpuFunc.cu:2460-2607); 1: plus an FP64
                                coplanarity-cubic root solve per candidate (the PolynomialSolver path the
                                reference compiles but never calls, Commom/PolynomialSolver.h:10-60), which
                                can only lower a candidate's time of impact; 2: the FP64 cubic alone, the
                                exact first-contact time of every candidate (the step then stops at
                                toi_scale of the first contact instead of the additive CCD's gap) */
    int instance_stop;       /* 0: the reference's stopping rule, one test over all vertices of the scene
                                (cpp:1776); 1: for batches of independent instances, the same rule per
                                simulated model: each model stops on its own |dx|^2 < outer_tol and clamps
                                its step by its own time of impact, and the step ends when every model has
                                stopped (or at max_outer).  A model that has stopped skips its sweeps.  Models
                                that touch one another should keep 0.  A stopped model's rows leave the
                                persistent PD solve (its CTAs return at entry when all their rows have
                                stopped). */
    int pd_group_ctas;       /* persistent PD solve: at most this many CTAs per launch (0: every CTA the
                                device holds at once).  A plan with more CTAs runs as one launch per group
                                of whole models (models share no matrix entry), in order. */
    int reserved[1];
} pdipc_params;

/* Per-context statistics of the most recent pdipc_step call. */
typedef struct {
    int64_t steps_done;          /* steps since initialize (or reset) */
    int32_t last_outer_iters;    /* outer iterations in the last step */
    int32_t max_outer_iters;     /* max over the steps of the last pdipc_step call */
    int64_t total_outer_iters;   /* sum over the steps of the last pdipc_step call */
    int64_t patch_pairs;         /* overlapping patch pairs found by the last broad phase */
    int64_t pt_candidates;       /* point-triangle candidates of the last broad phase */
    int64_t ee_candidates;       /* edge-edge candidates of the last broad phase */
    int64_t active_contacts;     /* pairs with d < dhat in the last contact pass */
    double last_toi;             /* clamped step fraction of the last outer iteration */
    double last_residual;        /* ||dx||^2 of the last outer iteration */
    int32_t n_sim;               /* simulated (cloth) vertices */
    int32_t n_total;             /* all vertices including static ones */
    int32_t n_patches;           /* collision patches (all models) */
    int32_t precision;           /* pdipc_precision in use */
    int64_t device_bytes;        /* device memory held by the context */
    int64_t kernel_launches;     /* kernels launched by the last pdipc_step call (graph nodes included) */
    double device_ms;            /* device time of the last pdipc_step call: CUDA events recorded on the
                                    context's stream around every step, summed */
    int32_t pd_path;             /* 0: one launch per sweep; 1: persistent, matrix from L2;
                                    2: persistent, matrix values in shared memory; 3: persistent,
                                    matrix values and the iterate's band in shared memory */
    int32_t pd_ctas;             /* CTAs of the persistent solve (0 if not used) */
    int64_t pd_solves;           /* projective-dynamics solves (one per outer iteration) in the last call */
    double pd_solve_ms;          /* their device time: CUDA events on the context's stream around each solve */
    double pd_solve_bytes;       /* algorithmic bytes of one solve: per vertex i and local-global iteration,
                                    local step 16 d_i + 68 plus (2 cheby) sweeps of 8 n_i + 28 plus
                                    (cheby - 1) Chebyshev reads of 12 (d_i stencil neighbours, n_i matrix
                                    off-diagonals; FP32 sizes, doubled value sizes in FP64 mode) */
    double ccd_ms;               /* device time of the time-of-impact passes (point-triangle and edge-edge
                                    candidates, global minimum) of the last call, CUDA events per outer
                                    iteration */
    double contact_ms;           /* device time of the contact-constraint passes of the last call */
    int32_t instances;           /* simulated models (the instances of params.instance_stop) */
    int32_t reserved_i;
    int64_t instance_outer_iters; /* sum over the steps of the last call and over the models of the outer
                                     iterations each model ran (params.instance_stop; else instances x
                                     total_outer_iters) */
} pdipc_stats;

/* Launch configuration a context runs with, and how it was chosen (no
 * counterpart in the reference, whose launch shapes are fixed macros:
 * PdIpcGpuFunc.cuh:133-134, PdIpcSimulator.cpp:418-431, 1121-1137). */
typedef struct {
    int32_t autotuned;          /* 1: chosen by timing candidates at pdipc_initialize (params.autotune) */
    int32_t from_cache;         /* 1: taken from an earlier context of the same shape in this process */
    int32_t pd_rows_per_thread; /* persistent PD solve: rows per thread (slices per warp); 0: one launch
                                   per sweep */
    int32_t pd_ctas;            /* CTAs of the persistent solve */
    int32_t pd_band;            /* 1: the iterate's column band in shared memory */
    int32_t pd_l1_gather;       /* 1: gathers through L1 */
    int32_t pd_local_sync;      /* 1: neighbour waits, 0: grid barriers */
    int32_t cand_grid;          /* blocks of the time-of-impact and contact kernels (grid-stride) */
    int32_t traverse_block;     /* threads per block of the broad-phase traversal */
    int32_t expand_block;       /* threads per block of the candidate expansion */
    int32_t candidates_timed;   /* configurations the autotuner timed */
    int32_t pd_launches;        /* launches of one persistent PD solve (groups of whole models) */
    double pd_solve_ms;         /* one outer iteration's PD solve, chosen configuration (0: not timed) */
    double pd_default_ms;       /* the same with the default configuration */
    double collision_ms;        /* broad phase + time of impact + contact, chosen shapes */
    double collision_default_ms;/* the same with the default shapes */
    int32_t reserved[8];
} pdipc_tuning;

/* Fill *p with the reference defaults listed beside each field. */
void pdipc_default_params(pdipc_params* p);

/* Create a context: BaseSimulator(simName, RunPlatform::CUDA) ctor plus the
 * PdIpcSimulator constructor (BaseSimulator.h:35-45, PdIpcSimulator.h:441-449).
 * Selects p->device, checks it is sm_103, creates the context's stream. */
pdipc_status pdipc_create(const pdipc_params* p, pdipc_ctx** out);

/* Add a simulated cloth model: PdIpcSimulator::addModelFromConfigFile with
 * <type> 0 k_stretch k_bend k_pin, <density>, <patchDim>
 * (PdIpcSimulator.h:462-534) plus readFixedInfo (PdIpcModel.h:56-77).
 * X: 3*nv float64, F: 3*nf int32 (0-based), pins: npins local vertex ids. */
pdipc_status pdipc_add_cloth(pdipc_ctx* ctx, const double* X, int nv, const int* F, int nf,
                             double density, double k_stretch, double k_bend,
                             const int* pins, int npins, double k_pin, int patch_dim);

/* Options of pdipc_add_cloth_ex beyond pdipc_add_cloth's. */
typedef struct {
    /* nf per-triangle stretch stiffnesses, or NULL for k_stretch everywhere.  The
     * reference weighs a vertex's springs by one per-vertex stiffness
     * (devStrainStiffness[offset], PdIpcGpuFunc.cu:673), so a vertex takes the mean
     * over its triangles. */
    const double* per_tri_stretch;
    /* Triangle strain limit: each triangle (where the stiffness is > 0) gets the
     * strain constraint of solveVolumetricStrainConstraintKernel (PdIpcGpuFunc.cu:
     * 439-599) on its 3 x 2 deformation gradient F = Ds Dm^-1: a 3 x 3 SVD (F with
     * the deformed unit normal as third column), singular values clamped to
     * [0.999, 1.001], weight = stiffness x rest area.  k_tri_strain applies to
     * every triangle, per_tri_strain (nf values, or NULL) overrides it.  The
     * reference applies this constraint to tets only. */
    double k_tri_strain;
    const double* per_tri_strain;
    int32_t reserved[8];
} pdipc_cloth_options;

/* pdipc_add_cloth with the options above (opt may be NULL: pdipc_add_cloth). */
pdipc_status pdipc_add_cloth_ex(pdipc_ctx* ctx, const double* X, int nv, const int* F, int nf, double density,
                                double k_stretch, double k_bend, const int* pins, int npins, double k_pin,
                                int patch_dim, const pdipc_cloth_options* opt);

/* Partition of a batch of independent instances (each cloth with its own
 * obstacles, nothing shared between instances) over `ranks` processes, one GPU
 * each, on the host: instance i has sizes[i] simulated vertices; rank r takes
 * instances [first[r], first[r + 1]) (first: ranks + 1 ints), contiguous runs
 * whose cumulative vertex counts split the total as evenly as whole instances
 * allow (the boundary after rank r is the instance boundary nearest to r + 1
 * shares of the total).  The step needs no exchange between ranks.  No
 * counterpart in the reference (one process, one GPU). */
pdipc_status pdipc_partition_instances(const int64_t* sizes, int n, int ranks, int* first);

/* Chain rule of the per-triangle stretch mapping, on the host: given the
 * gradient of a loss with respect to every simulated vertex's stretch stiffness
 * (dl_dvertex, n_sim, as pdipc_adjoint_backward returns it), the gradient with
 * respect to the per-triangle stretch stiffnesses of the cloth added
 * `cloth_index`-th (0-based among cloths): dl/dk_t = sum over t's vertices i of
 * dl/dk_i / (triangles at i).  dl_dtri: nf of that cloth. */
pdipc_status pdipc_stretch_gradient_per_triangle(pdipc_ctx* ctx, int cloth_index, const double* dl_dvertex,
                                                 double* dl_dtri);

/* Add a simulated tetrahedral (volumetric) model: PdIpcSimulator::addModelFromConfigFile
 * with <type> 1 k_strain k_volume k_pin, <density>, <patchDim> (PdIpcSimulator.h:462-534,
 * PdIpcVolumetricModel(s0, s1, s2), PdIpcVolumetricModel.h:21-25) read from a tetgen
 * .node/.ele pair.  X: 3*nv float64, T: 4*nt int32 (0-based), pins: local vertex ids.
 * Node mass is density times the summed volume of the node's tets (the reference's
 * BaseTetMeshHandle::computeVolume); every tet adds the strain constraint of
 * solveVolumetricStrainConstraintKernel (PdIpcGpuFunc.cu:439-599) with weight
 * k_strain * volume.  k_volume is accepted and unused, as in the reference (its
 * volume-constraint list is never filled).  The tets' boundary faces (faces of one tet)
 * collide; collision patches are a patch_dim^3 grid (PdIpcVolumetricModel.h:114-182). */
pdipc_status pdipc_add_volumetric(pdipc_ctx* ctx, const double* X, int nv, const int* T, int nt,
                                  double density, double k_strain, double k_volume,
                                  const int* pins, int npins, double k_pin, int patch_dim);

/* Boundary surface of a tetrahedral mesh, on the host (no device needed): the faces
 * that belong to exactly one tet, turned to face away from it
 * (PdIpcVolumetricModel::registerBoundaryInfo, PdIpcVolumetricModel.h:27-112; the
 * reference walks a hash map, here faces come in ascending order of their sorted
 * vertex triple).  These are the faces pdipc_add_volumetric makes collide.
 * faces: 3*cap_faces ints; *n_faces gets the count even when it exceeds cap_faces
 * (PDIPC_ERR_OVERFLOW). */
pdipc_status pdipc_tet_surface(const double* X, int nv, const int* T, int nt,
                               int* faces, int cap_faces, int* n_faces);

/* ---------------------------------------------------------------------------
 * Scene files (host only).  pdipc_scene_load reads a reference config.xml:
 * <timeStep>, <gravity>, <dhat>, <kappa> and every <object>/<static_object>
 * with its <name>/<name>.obj, tetgen .node/.ele (volumetric_mesh="tet"),
 * fixed_points.txt, and placement (origin/uniform attributes, <scale>,
 * <translation>, <rotation>) as BaseSimulator::readSimulatorFromConfigFile and
 * PdIpcSimulator::addModelFromConfigFile do (Simulator/BaseSimulator.cpp:4-65,
 * PdIpcSimulator.h:462-642, Model/BaseModel.cpp:21-66, 411-471).
 * ------------------------------------------------------------------------- */
typedef struct pdipc_scene pdipc_scene;

typedef struct {
    const char* name;     /* the object's name attribute */
    int kind;             /* 0 cloth (<type> 0), 1 volumetric (<type> 1), 2 static */
    int nv, nf, nt, npins;
    const double* X;      /* 3*nv placed positions (the tet nodes of a volumetric model) */
    const int* F;         /* 3*nf OBJ faces, 0-based (render surface of a volumetric model) */
    const int* T;         /* 4*nt tets, 0-based, or NULL */
    const int* pins;      /* fixed_points.txt ids, or NULL */
    double density;
    double k[3];          /* <type> stiffness triple: cloth (stretch, bend, pin),
                             volumetric (strain, volume, pin) */
    int patch_dim;
} pdipc_scene_model;

/* err (err_len bytes) receives a message on failure; *out owns every array. */
pdipc_status pdipc_scene_load(const char* config_path, pdipc_scene** out, char* err, int err_len);
int pdipc_scene_model_count(const pdipc_scene* s);
pdipc_status pdipc_scene_get_model(const pdipc_scene* s, int i, pdipc_scene_model* out);
/* time_step, gravity, dhat and kappa the config sets; other fields are kept */
pdipc_status pdipc_scene_apply_params(const pdipc_scene* s, pdipc_params* p);
/* pdipc_add_cloth / pdipc_add_volumetric / pdipc_add_static for every model, in file order */
pdipc_status pdipc_scene_add_models(const pdipc_scene* s, pdipc_ctx* ctx);
void pdipc_scene_free(pdipc_scene* s);

/* Add a static (kinematically fixed) triangle mesh:
 * PdIpcSimulator::addStaticModelFromConfigFile (PdIpcSimulator.h:536-600). */
pdipc_status pdipc_add_static(pdipc_ctx* ctx, const double* X, int nv, const int* F, int nf,
                              int patch_dim);

/* PdIpcSimulator::initialization (PdIpcSimulator.cpp:34-268): per-model
 * precompute, system assembly (setupHessMat cpp:270-414), device upload
 * (gpuGeneralInit/gpuSolverInit cpp:416-1149) and collision set-up including
 * the patch BVH build (gpuCollisionInit cpp:1151-1504). */
pdipc_status pdipc_initialize(pdipc_ctx* ctx);

/* nsteps x PdIpcSimulator::run(frame) (cpp:18-21 -> doTime cpp:1538 -> advance cpp:1683-1796).
 * The state stays on the device. */
pdipc_status pdipc_step(pdipc_ctx* ctx, int nsteps);

/* Change pdipc_params.wait_limit_us of an initialised context (no counterpart in
 * the reference, whose kernels never wait on one another).  A launch whose wait
 * runs past the limit ends early, the step returns PDIPC_ERR_CUDA with the state
 * of a partial step, and the context stays usable: set the state again
 * (pdipc_set_state / pdipc_load / pdipc_reset) and step on. */
pdipc_status pdipc_set_wait_limit(pdipc_ctx* ctx, int wait_limit_us);

/* BaseSimulator::animate(frame) = run(frame); postRun() (BaseSimulator.h:73-76):
 * one step, then copy every vertex position to out (3*n_total float64) —
 * the reference's postRun D2H of devPoints (cpp:23-32) into a headless buffer. */
pdipc_status pdipc_animate(pdipc_ctx* ctx, double* out);

/* postRun's device-to-host copy alone: out receives 3*n_total float64. */
pdipc_status pdipc_get_positions(pdipc_ctx* ctx, double* out);

/* Velocities of the simulated vertices: out receives 3*n_sim float64. */
pdipc_status pdipc_get_velocities(pdipc_ctx* ctx, double* out);

/* Overwrite positions (3*n_total) and optionally velocities (3*n_sim; NULL keeps them). */
pdipc_status pdipc_set_state(pdipc_ctx* ctx, const double* X, const double* V);

/* PdIpcSimulator::reset (BaseSimulator.h:79, empty in the reference): restore the
 * positions given at add time and zero velocities. */
pdipc_status pdipc_reset(pdipc_ctx* ctx);

pdipc_status pdipc_get_stats(pdipc_ctx* ctx, pdipc_stats* out);

/* The launch configuration of an initialised context (see pdipc_tuning). */
pdipc_status pdipc_get_tuning(pdipc_ctx* ctx, pdipc_tuning* out);

/* PdIpcSimulator::saveSimulator(frame) (PdIpcSimulator.h:879-916): writes the
 * EigenMatrixIO::write_binary layout (int64 rows=3, int64 cols=n_total, float32
 * column-major xyz; Commom/EigenMatrixIO.h:11-27) followed by a second block of
 * the same layout holding the n_sim velocities.  pdipc_load reads it back. */
pdipc_status pdipc_save(pdipc_ctx* ctx, const char* path);
pdipc_status pdipc_load(pdipc_ctx* ctx, const char* path);

/* Destroy the context and free everything it holds (the reference frees nothing). */
void pdipc_destroy(pdipc_ctx* ctx);

const char* pdipc_status_string(pdipc_status s);
/* Message of the last failing call on ctx (never NULL; "" if none). */
const char* pdipc_last_error(const pdipc_ctx* ctx);
int pdipc_abi_version(void);

/* ---------------------------------------------------------------------------
 * Stage entry points.  Each runs one stage of the step on the context's
 * device tables with caller-supplied host inputs, so a stage can be checked
 * on its own against the oracle.  They need pdipc_initialize first and leave
 * the simulation state untouched.
 * ------------------------------------------------------------------------- */

/* The patch broad phase of gpuCcdCulling (PdIpcSimulator.cpp:1799-1869):
 * swept patch AABBs from x_old (3*n_total) and dir (3*n_total), BVH refit,
 * overlapping patch pairs (a<b), expansion to point-triangle records
 * (v, f0, f1, f2) and edge-edge records (a0, a1, b0, b1).
 * Arrays of capacity cap_* receive up to that many records; *n_* receive the
 * full counts (PDIPC_ERR_OVERFLOW if a count exceeds its capacity). */
pdipc_status pdipc_stage_broadphase(pdipc_ctx* ctx, const double* x_old, const double* dir,
                                    int* pairs, int64_t cap_pairs, int64_t* n_pairs,
                                    int* pt, int64_t cap_pt, int64_t* n_pt,
                                    int* ee, int64_t cap_ee, int64_t* n_ee);

/* Morton codes (63-bit, 21 bits per axis) of the patch AABB centres computed
 * at initialize, and the stable sort order of the patches by code
 * (AipcBvhs::init, Simulator/Bvhs/AipcBvhs.cpp:134-213). */
pdipc_status pdipc_stage_morton(pdipc_ctx* ctx, uint64_t* codes, int* order, int cap);

/* getImpactOfTimeHost (PdIpcGpuFunc.cu:2706-2742) over the candidate set of the
 * last broad phase: per-candidate toi (1 where skipped) and the clamped global
 * toi (0.98*min if min<1).  x0, x1: 3*n_total. toi_pt/toi_ee may be NULL. */
pdipc_status pdipc_stage_toi(pdipc_ctx* ctx, const double* x0, const double* x1,
                             double* toi_pt, double* toi_ee, double* toi_global);

/* No-allocation variant of pdipc_stage_toi; this entry point has no counterpart
 * in the reference.  Same inputs and outputs (FP64 and mixed modes only:
 * PDIPC_ERR_ARG in FP32 mode), but it allocates nothing on the device or the
 * host: the per-candidate times of impact are written to one file-scope device
 * array of 2^20 doubles (8 MiB, reserved when the library's module loads) and
 * copied from there to toi_pt / toi_ee.  For callers that must not allocate
 * between steps: cudaFree synchronises the whole device, which stalls a host
 * that keeps other work queued, and cudaMalloc can fail when another allocator
 * already holds the device's memory.
 *   - Limit: n_pt + n_ee <= 2^20 candidates of the last broad phase, else
 *     PDIPC_ERR_OVERFLOW (with the counts in pdipc_last_error) and nothing runs.
 *   - The first call on a device looks up the array's address
 *     (cudaGetSymbolAddress) and caches it; make that first call before any
 *     stream capture begins.
 *   - Nothing has to start at zero: each call writes entries [0, n) before
 *     reading them.
 *   - The array is shared by every context of the process on that device, so
 *     overlapping calls would race on it; the library serialises them with a
 *     per-device lock held until the results are on the host. */
pdipc_status pdipc_stage_toi_noalloc(pdipc_ctx* ctx, const double* x0, const double* x1,
                                     double* toi_pt, double* toi_ee, double* toi_global);

/* setCollisionConstraintsHost (PdIpcGpuFunc.cu:2894-2930) over the candidate set
 * of the last broad phase at positions x (3*n_total): collision diagonal
 * (n_total) and right-hand side (3*n_total); *n_active gets the pair count. */
pdipc_status pdipc_stage_contact(pdipc_ctx* ctx, const double* x,
                                 double* coll_diag, double* coll_rhs, int64_t* n_active);

/* predictiveKernel (PdIpcGpuFunc.cu:88-147) from the state (X: 3*n_total,
 * V: 3*n_sim) followed by one outer iteration's projective-dynamics solve:
 * lg_iterations x (doLocalProjection cpp:1624-1681 + Chebyshev-accelerated
 * Jacobi cu:1245-1346) with no contact terms.  out_X receives 3*n_total
 * positions.  The context's state is restored afterwards. */
pdipc_status pdipc_stage_pd(pdipc_ctx* ctx, const double* X, const double* V, double* out_X);

/* Times the unit of the projective-dynamics solve launched on its own: one
 * plain weighted-Jacobi sweep over the system matrix (the R2 sweep of
 * chebyshevJacobiR2IterationKernel, PdIpcGpuFunc.cu:1076-1129, here applied
 * as one of two J sweeps; on the correction in the mixed mode), `launches`
 * back-to-back launches on the context's stream between two CUDA events.
 * *avg_ms = mean duration of one launch; *bytes = algorithmic bytes one launch
 * must move (8 per stored matrix entry + 40 per row: x, rhs and output xyz,
 * inverse diagonal; FP32 sizes, double value sizes in FP64 mode). */
pdipc_status pdipc_stage_sweep_timing(pdipc_ctx* ctx, int launches, double* avg_ms, double* bytes);

/* Times the local step (solveClothPointsStrainAndBendingConstraintKernel +
 * solvePointsConstraintKernel, PdIpcGpuFunc.cu:627-790, with the right-hand
 * side's first Jacobi sweep fused as the per-sweep solve runs it) launched on
 * its own: the curvature kernel and the right-hand-side kernel, `launches`
 * times back to back between two CUDA events on the context's stream, at the
 * current positions (which stay untouched).  *avg_ms = mean duration of one
 * local step (two launches); *bytes = its algorithmic bytes: per vertex i,
 * 16 d_i + 68 for the local step (d_i stencil neighbours) plus 8 n_i + 28 for
 * the fused sweep (n_i matrix off-diagonals; FP32 sizes, double value sizes
 * in FP64 mode). */
pdipc_status pdipc_stage_local_timing(pdipc_ctx* ctx, int launches, double* avg_ms, double* bytes);

/* The reference's penalty / discrete-collision contact path
 * (Simulator/PD-IPC/PdIpcGpuFunc.cu:2933-3740).  The reference declares these
 * kernels beside the IPC path, but its step never calls them (PdIpcSimulator.cpp
 * only allocates the zero force buffer that predictiveKernel reads), so the
 * library offers them as stages on a context's tables and the step does not
 * use them either.
 *   - Each penalty stage starts from zero forces and hit counts, accumulates a
 *     per-vertex penalty force (force: 3*n_total) and hit count (times: n_total),
 *     then applies uniformPenaltyForceKernal (cu:3140-3195) to the n_sim
 *     simulated vertices with at least one hit: the force becomes its mean over
 *     the hits minus damping*v, and v (V: 3*n_sim, read and overwritten) keeps
 *     0.9 of its part across the mean force and -0.4 of its part along it.
 *   - Arithmetic in the state precision (double in the FP64 and mixed modes). */

/* prediticeDCPositionKernel (cu:2933-2981): sn = x + dt (v + dt m^-1 f_gravity)
 * for the n_sim simulated vertices (X, sn: 3*n_sim); a pinned vertex keeps x and
 * its velocity in V (3*n_sim, in/out) becomes 0. */
pdipc_status pdipc_stage_penalty_predict(pdipc_ctx* ctx, const double* X, double* V, double* sn);

/* computePenaltyForceHost (cu:3198-3246) over the candidates of the last broad
 * phase: a pair sharing no vertex whose swept boxes (from x0 along dir, both
 * 3*n_total) meet within 1e-4 and whose additive CCD time of impact is below 1
 * is pushed apart at x0 + dir with stiffness * distance along the closest-point
 * vector (point-triangle: -3f on the point, f on each face vertex, f = n d k/3;
 * edge-edge: -f on the first edge's vertices, f on the second's, f = n d k/2). */
pdipc_status pdipc_stage_penalty_ccd(pdipc_ctx* ctx, const double* x0, const double* dir, double stiffness,
                                     double damping, double* V, double* force, int* times);

/* applyPenaltyForceForFloorHost (cu:3273-3305): a simulated vertex of x
 * (3*n_total) below y = 0 gets the force (0, -y*stiffness, 0) and one hit. */
pdipc_status pdipc_stage_penalty_floor(pdipc_ctx* ctx, const double* x, double stiffness, double damping,
                                       double* V, double* force, int* times);

/* computeDcdPenaltyForceHost (cu:3690-3738) over n_pairs face pairs (2 ints
 * each: indices into the context's collision faces, numbered like its vertices:
 * cloths and volumetric boundaries in add order, then statics): a pair sharing
 * no vertex whose triangles intersect (separating-axis test, triContact
 * cu:3391-3468) pushes each vertex of a triangle whose first vertex is simulated
 * out of the other triangle's plane (through its second vertex) along that
 * plane's unit normal with stiffness * depth, when it lies behind the plane; the
 * other triangle's vertices take -1/3 of each such force.  Two faces of the
 * same model use self_stiffness.  PDIPC_ERR_ARG for a face index out of range. */
pdipc_status pdipc_stage_penalty_dcd(pdipc_ctx* ctx, const double* x, const int* face_pairs, int64_t n_pairs,
                                     double stiffness, double self_stiffness, double damping, double* V,
                                     double* force, int* times);

/* Discrete adjoint of a recorded rollout (no counterpart in the reference,
 * whose simulator is not differentiable).  pdipc_adjoint_record(ctx, k) with
 * k > 0 starts recording the following pdipc_step calls, keeping the state of
 * the simulated vertices at the start of every k-th step; k = 0 drops the
 * recording, and so do pdipc_set_state, pdipc_reset and pdipc_load.
 * pdipc_adjoint_backward takes the gradient of a loss with respect to the
 * simulated vertices' positions (dl_dx, 3*n_sim) and velocities (dl_dv, 3*n_sim,
 * NULL = 0) after the last recorded step and returns the gradient with
 * respect to their positions and velocities before the first recorded step
 * (dl_dx0, dl_dv0, 3*n_sim), and, if dl_dstrain is not NULL, with respect to each
 * simulated vertex's stretch stiffness (n_sim; the per-vertex strain weight
 * that the model's k_stretch sets, PdIpcClothModel.h:177-328).  It is the exact
 * derivative of the executed iteration: every local-global iteration, every
 * weighted-Jacobi sweep and Chebyshev step, the strain-limit projections of
 * tets and cloth triangles (through the derivative of their clamped SVD), the
 * prediction and the velocity update, for the outer-iteration counts the
 * recorded steps ran (fix them with pdipc_params.fixed_outer for a smooth
 * rollout).  It replays the recorded steps from the checkpoints (two replays
 * per step) and leaves the context's state and stats as they were.
 * PDIPC_ERR_STATE unless the context is in the plain FP64 form
 * (PDIPC_PREC_FP64) without per-instance stopping, steps were recorded, and
 * every replayed outer iteration ran a full, contact-free step (time of impact
 * 1, no active contact constraints). */
pdipc_status pdipc_adjoint_record(pdipc_ctx* ctx, int checkpoint_every);
pdipc_status pdipc_adjoint_backward(pdipc_ctx* ctx, const double* dl_dx, const double* dl_dv, double* dl_dx0,
                                    double* dl_dv0, double* dl_dstrain);

/* Topology precompute of one mesh, on the host (no device needed):
 * sorted unique edges (Model/TriangleMesh/BaseSurfaceMesh.cpp:219-275), the grid
 * collision patches (PdIpcClothModel::setCollisionPatches, PdIpcClothModel.h:45-140)
 * and the one-owner-face assignment of points and edges
 * (PdIpcModel::postProcessBoundaryInfo, PdIpcModel.h:84-172).
 * edges: 2*cap_edges ints; patch_off: npatch+1 ints (cap_patches+1), patch_faces:
 * cap_faces ints; owner_of_point: nv ints; owner_of_edge: cap_edges ints.
 * The counts are returned even when a capacity is too small (PDIPC_ERR_OVERFLOW). */
pdipc_status pdipc_mesh_topology(const double* X, int nv, const int* F, int nf, int patch_dim,
                                 int* edges, int cap_edges, int* n_edges,
                                 int* patch_off, int cap_patches, int* patch_faces, int cap_faces,
                                 int* n_patches, int* owner_of_point, int* owner_of_edge);

#ifdef __cplusplus
}
#endif
#endif /* PDIPC_H */
