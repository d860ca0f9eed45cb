// capi.cpp — the extern "C" boundary of libpdipc.so (include/pdipc.h).
//
// Mirrors the lifecycle of PD_IPC::PdIpcSimulator (Simulator/PD-IPC/PdIpcSimulator.h):
// construct, add models, initialization(), run(frame)/animate(frame),
// postRun(), saveSimulator(frame).  No exception crosses the boundary.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <algorithm>
#include <cstring>
#include <exception>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "../../include/pdipc.h"
#include "host_tables.h"
#include "solver.h"

struct pdipc_ctx {
    pdipc_params prm{};
    std::vector<pdipc::ModelInput> models;
    std::unique_ptr<pdipc::SolverBase> solver;
    std::string err;
    bool initialized = false;
    // per cloth model, kept past initialize for pdipc_stretch_gradient_per_triangle:
    // its first simulated vertex, its faces and each vertex's triangle count
    struct Cloth {
        int first = 0;
        std::vector<int> F;
        std::vector<int> ntri;
    };
    std::vector<Cloth> cloths;
};

namespace {

pdipc_status fail(pdipc_ctx* c, pdipc_status s, const std::string& msg) {
    if (c) c->err = msg;
    return s;
}

template <typename F>
pdipc_status guarded(pdipc_ctx* c, F&& f) {
    try {
        return f();
    } catch (const std::bad_alloc&) {
        return fail(c, PDIPC_ERR_ALLOC, "host allocation failed");
    } catch (const std::exception& e) {
        return fail(c, PDIPC_ERR_ARG, e.what());
    } catch (...) {
        return fail(c, PDIPC_ERR_ARG, "unknown error");
    }
}

// Every call on an initialised context runs on the context's device: two
// contexts on different devices can share one host thread, and device-keyed
// state (the no-allocation stage's scratch address) follows the current device.
pdipc_status need_init(pdipc_ctx* c) {
    if (!c) return PDIPC_ERR_ARG;
    if (!c->initialized || !c->solver) return fail(c, PDIPC_ERR_STATE, "call pdipc_initialize first");
    if (cudaSetDevice(c->prm.device) != cudaSuccess) {
        cudaGetLastError();
        return fail(c, PDIPC_ERR_CUDA, "cudaSetDevice failed");
    }
    return PDIPC_OK;
}

pdipc_status add_model(pdipc_ctx* c, const double* X, int nv, const int* F, int nf, bool is_static, double density,
                       double ks, double kb, const int* pins, int npins, double kp, int patch_dim) {
    if (!c) return PDIPC_ERR_ARG;
    if (c->initialized) return fail(c, PDIPC_ERR_STATE, "models must be added before pdipc_initialize");
    if (!X || !F || nv <= 0 || nf <= 0 || npins < 0 || (npins > 0 && !pins) || patch_dim <= 0)
        return fail(c, PDIPC_ERR_ARG, "bad mesh arguments");
    if (!is_static && !(density > 0.0)) return fail(c, PDIPC_ERR_ARG, "cloth density must be positive");
    for (int i = 0; i < 3 * nf; ++i)
        if (F[i] < 0 || F[i] >= nv) return fail(c, PDIPC_ERR_ARG, "face index out of range");
    for (int i = 0; i < npins; ++i)
        if (pins[i] < 0 || pins[i] >= nv) return fail(c, PDIPC_ERR_ARG, "pin index out of range");
    return guarded(c, [&]() {
        pdipc::ModelInput m;
        m.X.assign(X, X + 3 * (size_t)nv);
        m.F.assign(F, F + 3 * (size_t)nf);
        m.nv = nv;
        m.nf = nf;
        m.is_static = is_static;
        m.density = density;
        m.k_stretch = ks;
        m.k_bend = kb;
        m.k_pin = kp;
        if (npins > 0) m.pins.assign(pins, pins + npins);
        m.patch_dim = patch_dim;
        c->models.push_back(std::move(m));
        return PDIPC_OK;
    });
}

// One float32 column-major 3 x n block in EigenMatrixIO::write_binary layout.
bool write_block(FILE* f, const std::vector<double>& xyz, int64_t n) {
    int64_t rows = 3, cols = n;
    if (fwrite(&rows, sizeof(rows), 1, f) != 1 || fwrite(&cols, sizeof(cols), 1, f) != 1) return false;
    std::vector<float> buf(3 * (size_t)n);
    for (size_t i = 0; i < buf.size(); ++i) buf[i] = (float)xyz[i];
    return fwrite(buf.data(), sizeof(float), buf.size(), f) == buf.size();
}
bool read_block(FILE* f, std::vector<double>& xyz, int64_t n) {
    int64_t rows = 0, cols = 0;
    if (fread(&rows, sizeof(rows), 1, f) != 1 || fread(&cols, sizeof(cols), 1, f) != 1) return false;
    if (rows != 3 || cols != n) return false;
    std::vector<float> buf(3 * (size_t)n);
    if (fread(buf.data(), sizeof(float), buf.size(), f) != buf.size()) return false;
    xyz.resize(buf.size());
    for (size_t i = 0; i < buf.size(); ++i) xyz[i] = (double)buf[i];
    return true;
}

}  // namespace

extern "C" {

int pdipc_abi_version(void) { return PDIPC_ABI_VERSION; }

void pdipc_default_params(pdipc_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->time_step = 0.01;
    p->gravity = -9.8;
    p->dhat = 1e-3;
    p->kappa = 1e4;
    p->inflation_radius = -1.0;
    p->lg_iterations = 10;
    p->cheby_iterations = 15;
    p->cheby_rho = 0.9992;
    p->jacobi_relax = 2.0 / 3.0;
    p->max_outer = 30;
    p->outer_tol = 1e-5;
    p->ccd_slack = 5e-3;
    p->toi_scale = 0.98;
    p->ccd_max_iter = 10;
    p->ccd_eta = 0.1;
    p->static_mass = 1e4;
    p->precision = PDIPC_PREC_FP32;
    p->fixed_outer = 0;
    p->use_graphs = 1;
    p->device = 0;
    p->rebuild_bvh = 0;
    p->persistent = 1;
}

const char* pdipc_status_string(pdipc_status s) {
    switch (s) {
        case PDIPC_OK: return "PDIPC_OK";
        case PDIPC_ERR_ARG: return "PDIPC_ERR_ARG";
        case PDIPC_ERR_CUDA: return "PDIPC_ERR_CUDA";
        case PDIPC_ERR_OVERFLOW: return "PDIPC_ERR_OVERFLOW";
        case PDIPC_ERR_NONFINITE: return "PDIPC_ERR_NONFINITE";
        case PDIPC_ERR_NOT_CONVERGED: return "PDIPC_ERR_NOT_CONVERGED";
        case PDIPC_ERR_STATE: return "PDIPC_ERR_STATE";
        case PDIPC_ERR_ALLOC: return "PDIPC_ERR_ALLOC";
        case PDIPC_ERR_IO: return "PDIPC_ERR_IO";
    }
    return "PDIPC_ERR_UNKNOWN";
}

const char* pdipc_last_error(const pdipc_ctx* ctx) { return ctx ? ctx->err.c_str() : ""; }

pdipc_status pdipc_create(const pdipc_params* p, pdipc_ctx** out) {
    if (!p || !out) return PDIPC_ERR_ARG;
    *out = nullptr;
    if (p->precision < 0 || p->precision > 2) return PDIPC_ERR_ARG;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= p->device || p->device < 0) {
        cudaGetLastError();
        return PDIPC_ERR_CUDA;
    }
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, p->device) != cudaSuccess) return PDIPC_ERR_CUDA;
    if (!(prop.major == 10 && prop.minor == 3)) return PDIPC_ERR_CUDA;  // built for sm_103a only
    if (cudaSetDevice(p->device) != cudaSuccess) return PDIPC_ERR_CUDA;
    pdipc_ctx* c = new (std::nothrow) pdipc_ctx();
    if (!c) return PDIPC_ERR_ALLOC;
    c->prm = *p;
    *out = c;
    return PDIPC_OK;
}

pdipc_status pdipc_add_cloth(pdipc_ctx* ctx, const double* X, int nv, const int* F, int nf, double density,
                             double k_stretch, double k_bend, const int* pins, int npins, double k_pin,
                             int patch_dim) {
    return pdipc_add_cloth_ex(ctx, X, nv, F, nf, density, k_stretch, k_bend, pins, npins, k_pin, patch_dim, nullptr);
}

pdipc_status pdipc_add_cloth_ex(pdipc_ctx* ctx, const double* X, int nv, const int* F, int nf, double density,
                                double k_stretch, double k_bend, const int* pins, int npins, double k_pin,
                                int patch_dim, const pdipc_cloth_options* opt) {
    if (opt) {
        if (!ctx) return PDIPC_ERR_ARG;
        if (!(opt->k_tri_strain >= 0.0) || !std::isfinite(opt->k_tri_strain))
            return fail(ctx, PDIPC_ERR_ARG, "k_tri_strain must be a finite value >= 0");
        for (const double* a : {opt->per_tri_stretch, opt->per_tri_strain})
            if (a && F && nf > 0)
                for (int f = 0; f < nf; ++f)
                    if (!(a[f] >= 0.0) || !std::isfinite(a[f]))
                        return fail(ctx, PDIPC_ERR_ARG, "per-triangle stiffness must be finite and >= 0");
    }
    pdipc_status s = add_model(ctx, X, nv, F, nf, false, density, k_stretch, k_bend, pins, npins, k_pin, patch_dim);
    if (s != PDIPC_OK) return s;
    return guarded(ctx, [&]() {
        pdipc::ModelInput& m = ctx->models.back();
        if (opt) {
            if (opt->per_tri_stretch) m.tri_stretch.assign(opt->per_tri_stretch, opt->per_tri_stretch + nf);
            m.k_tri_strain = opt->k_tri_strain;
            if (opt->per_tri_strain) m.tri_strain.assign(opt->per_tri_strain, opt->per_tri_strain + nf);
        }
        pdipc_ctx::Cloth c;  // simulated models come first, in add order
        for (size_t q = 0; q + 1 < ctx->models.size(); ++q)
            if (!ctx->models[q].is_static) c.first += ctx->models[q].nv;
        c.F.assign(F, F + 3 * (size_t)nf);
        c.ntri.assign(nv, 0);
        for (int q = 0; q < 3 * nf; ++q) ++c.ntri[F[q]];
        ctx->cloths.push_back(std::move(c));
        return PDIPC_OK;
    });
}

pdipc_status pdipc_partition_instances(const int64_t* sizes, int n, int ranks, int* first) {
    if (!sizes || !first || n < 0 || ranks < 1) return PDIPC_ERR_ARG;
    int64_t total = 0;
    for (int i = 0; i < n; ++i) {
        if (sizes[i] < 0) return PDIPC_ERR_ARG;
        total += sizes[i];
    }
    // rank r ends after the first instance whose running count reaches
    // (r + 1) / ranks of the total, rounding the boundary to the nearer side
    first[0] = 0;
    int i = 0;
    int64_t run = 0;
    for (int r = 0; r < ranks; ++r) {
        const double goal = (double)total * (double)(r + 1) / (double)ranks;
        while (i < n && (double)(run + sizes[i]) <= goal) run += sizes[i++];
        if (i < n && r + 1 < ranks) {  // the instance that crosses the goal: to whichever side is nearer
            const double over = (double)(run + sizes[i]) - goal, under = goal - (double)run;
            if (over < under) run += sizes[i++];
        }
        first[r + 1] = (r + 1 == ranks) ? n : i;
    }
    return PDIPC_OK;
}

pdipc_status pdipc_stretch_gradient_per_triangle(pdipc_ctx* ctx, int cloth_index, const double* dl_dvertex,
                                                 double* dl_dtri) {
    if (!ctx) return PDIPC_ERR_ARG;
    if (!dl_dvertex || !dl_dtri) return fail(ctx, PDIPC_ERR_ARG, "null argument");
    if (cloth_index < 0 || cloth_index >= (int)ctx->cloths.size())
        return fail(ctx, PDIPC_ERR_ARG, "no cloth with that index");
    const pdipc_ctx::Cloth& c = ctx->cloths[cloth_index];
    const int nf = (int)c.F.size() / 3;
    for (int f = 0; f < nf; ++f) {
        double g = 0.0;
        for (int k = 0; k < 3; ++k) {
            const int v = c.F[3 * f + k];
            g += dl_dvertex[c.first + v] / (double)c.ntri[v];
        }
        dl_dtri[f] = g;
    }
    return PDIPC_OK;
}

pdipc_status pdipc_add_volumetric(pdipc_ctx* ctx, const double* X, int nv, const int* T, int nt, double density,
                                  double k_strain, double k_volume, const int* pins, int npins, double k_pin,
                                  int patch_dim) {
    if (!ctx) return PDIPC_ERR_ARG;
    if (ctx->initialized) return fail(ctx, PDIPC_ERR_STATE, "models must be added before initialize");
    if (!X || !T || nv <= 0 || nt <= 0) return fail(ctx, PDIPC_ERR_ARG, "empty tetrahedral mesh");
    if (npins < 0 || (npins > 0 && !pins)) return fail(ctx, PDIPC_ERR_ARG, "bad pin list");
    if (patch_dim < 1) return fail(ctx, PDIPC_ERR_ARG, "patch_dim must be positive");
    if (!(density > 0.0) || !(k_strain >= 0.0) || !(k_pin >= 0.0))
        return fail(ctx, PDIPC_ERR_ARG, "density must be positive and stiffnesses non-negative");
    for (int i = 0; i < 4 * nt; ++i)
        if (T[i] < 0 || T[i] >= nv) return fail(ctx, PDIPC_ERR_ARG, "tet index out of range");
    for (int i = 0; i < npins; ++i)
        if (pins[i] < 0 || pins[i] >= nv) return fail(ctx, PDIPC_ERR_ARG, "pin index out of range");
    return guarded(ctx, [&]() {
        pdipc::ModelInput m;
        m.X.assign(X, X + 3 * (size_t)nv);
        m.T.assign(T, T + 4 * (size_t)nt);
        m.nv = nv;
        m.nt = nt;
        m.is_volumetric = true;
        m.density = density;
        m.k_strain = k_strain;
        m.k_volume = k_volume;
        m.k_pin = k_pin;
        if (npins > 0) m.pins.assign(pins, pins + npins);
        m.patch_dim = patch_dim;
        ctx->models.push_back(std::move(m));
        return PDIPC_OK;
    });
}

pdipc_status pdipc_tet_surface(const double* X, int nv, const int* T, int nt, int* faces, int cap_faces,
                               int* n_faces) {
    if (!X || !T || !n_faces || nv <= 0 || nt <= 0 || (cap_faces > 0 && !faces)) return PDIPC_ERR_ARG;
    try {
        std::vector<int> f;
        if (!pdipc::tet_boundary_faces(X, nv, T, nt, f).empty()) return PDIPC_ERR_ARG;
        *n_faces = (int)f.size() / 3;
        if (*n_faces > cap_faces) return PDIPC_ERR_OVERFLOW;
        std::copy(f.begin(), f.end(), faces);
        return PDIPC_OK;
    } catch (const std::bad_alloc&) {
        return PDIPC_ERR_ALLOC;
    }
}

pdipc_status pdipc_add_static(pdipc_ctx* ctx, const double* X, int nv, const int* F, int nf, int patch_dim) {
    return add_model(ctx, X, nv, F, nf, true, 0.0, 0.0, 0.0, nullptr, 0, 0.0, patch_dim);
}

pdipc_status pdipc_initialize(pdipc_ctx* ctx) {
    if (!ctx) return PDIPC_ERR_ARG;
    if (ctx->initialized) return fail(ctx, PDIPC_ERR_STATE, "already initialized");
    return guarded(ctx, [&]() {
        pdipc::HostTables H;
        std::string e = pdipc::build_host_tables(ctx->models, ctx->prm.gravity, H);
        if (!e.empty()) return fail(ctx, PDIPC_ERR_ARG, e);
        if (cudaSetDevice(ctx->prm.device) != cudaSuccess) return fail(ctx, PDIPC_ERR_CUDA, "cudaSetDevice failed");
        ctx->solver = pdipc::make_solver(ctx->prm.precision);
        pdipc_status s = ctx->solver->init(H, ctx->prm, ctx->err);
        if (s != PDIPC_OK) {
            ctx->solver.reset();
            return s;
        }
        ctx->initialized = true;
        ctx->models.clear();
        ctx->models.shrink_to_fit();
        return PDIPC_OK;
    });
}

pdipc_status pdipc_step(pdipc_ctx* ctx, int nsteps) {
    pdipc_status s = need_init(ctx);
    if (s != PDIPC_OK) return s;
    return guarded(ctx, [&]() { return ctx->solver->step(nsteps, ctx->err); });
}

pdipc_status pdipc_set_wait_limit(pdipc_ctx* ctx, int wait_limit_us) {
    pdipc_status s = need_init(ctx);
    if (s != PDIPC_OK) return s;
    if (wait_limit_us < 0) return fail(ctx, PDIPC_ERR_ARG, "wait_limit_us must not be negative");
    ctx->prm.wait_limit_us = wait_limit_us;
    ctx->solver->set_wait_limit(wait_limit_us);
    return PDIPC_OK;
}

pdipc_status pdipc_get_positions(pdipc_ctx* ctx, double* out) {
    pdipc_status s = need_init(ctx);
    if (s != PDIPC_OK) return s;
    if (!out) return fail(ctx, PDIPC_ERR_ARG, "null output");
    return guarded(ctx, [&]() { return ctx->solver->get_positions(out, ctx->err); });
}

pdipc_status pdipc_animate(pdipc_ctx* ctx, double* out) {
    pdipc_status s = pdipc_step(ctx, 1);
    if (s != PDIPC_OK) return s;
    return pdipc_get_positions(ctx, out);
}

pdipc_status pdipc_get_velocities(pdipc_ctx* ctx, double* out) {
    pdipc_status s = need_init(ctx);
    if (s != PDIPC_OK) return s;
    if (!out) return fail(ctx, PDIPC_ERR_ARG, "null output");
    return guarded(ctx, [&]() { return ctx->solver->get_velocities(out, ctx->err); });
}

pdipc_status pdipc_set_state(pdipc_ctx* ctx, const double* X, const double* V) {
    pdipc_status s = need_init(ctx);
    if (s != PDIPC_OK) return s;
    if (!X) return fail(ctx, PDIPC_ERR_ARG, "null positions");
    return guarded(ctx, [&]() { return ctx->solver->set_state(X, V, ctx->err); });
}

pdipc_status pdipc_reset(pdipc_ctx* ctx) {
    pdipc_status s = need_init(ctx);
    if (s != PDIPC_OK) return s;
    return guarded(ctx, [&]() { return ctx->solver->reset(ctx->err); });
}

pdipc_status pdipc_get_stats(pdipc_ctx* ctx, pdipc_stats* out) {
    pdipc_status s = need_init(ctx);
    if (s != PDIPC_OK) return s;
    if (!out) return fail(ctx, PDIPC_ERR_ARG, "null output");
    ctx->solver->stats(out);
    return PDIPC_OK;
}

pdipc_status pdipc_get_tuning(pdipc_ctx* ctx, pdipc_tuning* out) {
    pdipc_status s = need_init(ctx);
    if (s != PDIPC_OK) return s;
    if (!out) return fail(ctx, PDIPC_ERR_ARG, "null output");
    ctx->solver->tuning(out);
    return PDIPC_OK;
}

pdipc_status pdipc_save(pdipc_ctx* ctx, const char* path) {
    pdipc_status s = need_init(ctx);
    if (s != PDIPC_OK) return s;
    if (!path) return fail(ctx, PDIPC_ERR_ARG, "null path");
    return guarded(ctx, [&]() {
        const int nt = ctx->solver->n_total(), ns = ctx->solver->n_sim();
        std::vector<double> X(3 * (size_t)nt), V(3 * (size_t)ns);
        pdipc_status r = ctx->solver->get_positions(X.data(), ctx->err);
        if (r == PDIPC_OK) r = ctx->solver->get_velocities(V.data(), ctx->err);
        if (r != PDIPC_OK) return r;
        FILE* f = std::fopen(path, "wb");
        if (!f) return fail(ctx, PDIPC_ERR_IO, std::string("cannot open ") + path);
        bool ok = write_block(f, X, nt) && write_block(f, V, ns);
        ok = (std::fclose(f) == 0) && ok;
        return ok ? PDIPC_OK : fail(ctx, PDIPC_ERR_IO, "write failed");
    });
}

pdipc_status pdipc_load(pdipc_ctx* ctx, const char* path) {
    pdipc_status s = need_init(ctx);
    if (s != PDIPC_OK) return s;
    if (!path) return fail(ctx, PDIPC_ERR_ARG, "null path");
    return guarded(ctx, [&]() {
        const int nt = ctx->solver->n_total(), ns = ctx->solver->n_sim();
        std::vector<double> X, V;
        FILE* f = std::fopen(path, "rb");
        if (!f) return fail(ctx, PDIPC_ERR_IO, std::string("cannot open ") + path);
        bool ok = read_block(f, X, nt);
        bool okv = ok && read_block(f, V, ns);
        std::fclose(f);
        if (!ok) return fail(ctx, PDIPC_ERR_IO, "bad checkpoint header or size");
        return ctx->solver->set_state(X.data(), okv ? V.data() : nullptr, ctx->err);
    });
}

void pdipc_destroy(pdipc_ctx* ctx) {
    if (!ctx) return;
    if (ctx->solver) cudaSetDevice(ctx->prm.device);
    delete ctx;
}

pdipc_status pdipc_stage_broadphase(pdipc_ctx* ctx, const double* x_old, const double* dir, int* pairs,
                                    int64_t cap_pairs, int64_t* n_pairs, int* pt, int64_t cap_pt, int64_t* n_pt,
                                    int* ee, int64_t cap_ee, int64_t* n_ee) {
    pdipc_status s = need_init(ctx);
    if (s != PDIPC_OK) return s;
    if (!x_old || !dir || !n_pairs || !n_pt || !n_ee) return fail(ctx, PDIPC_ERR_ARG, "null argument");
    return guarded(ctx, [&]() {
        return ctx->solver->stage_broadphase(x_old, dir, pairs, cap_pairs, n_pairs, pt, cap_pt, n_pt, ee, cap_ee,
                                             n_ee, ctx->err);
    });
}

pdipc_status pdipc_stage_morton(pdipc_ctx* ctx, uint64_t* codes, int* order, int cap) {
    pdipc_status s = need_init(ctx);
    if (s != PDIPC_OK) return s;
    if (!codes || !order) return fail(ctx, PDIPC_ERR_ARG, "null argument");
    return guarded(ctx, [&]() { return ctx->solver->stage_morton(codes, order, cap, ctx->err); });
}

pdipc_status pdipc_stage_toi(pdipc_ctx* ctx, const double* x0, const double* x1, double* toi_pt, double* toi_ee,
                             double* toi_global) {
    pdipc_status s = need_init(ctx);
    if (s != PDIPC_OK) return s;
    if (!x0 || !x1) return fail(ctx, PDIPC_ERR_ARG, "null argument");
    return guarded(ctx, [&]() { return ctx->solver->stage_toi(x0, x1, toi_pt, toi_ee, toi_global, ctx->err); });
}

pdipc_status pdipc_stage_toi_noalloc(pdipc_ctx* ctx, const double* x0, const double* x1, double* toi_pt,
                                     double* toi_ee, double* toi_global) {
    pdipc_status s = need_init(ctx);
    if (s != PDIPC_OK) return s;
    if (!x0 || !x1) return fail(ctx, PDIPC_ERR_ARG, "null argument");
    return guarded(ctx, [&]() {
        return ctx->solver->stage_toi_noalloc(x0, x1, toi_pt, toi_ee, toi_global, ctx->err);
    });
}

pdipc_status pdipc_stage_contact(pdipc_ctx* ctx, const double* x, double* coll_diag, double* coll_rhs,
                                 int64_t* n_active) {
    pdipc_status s = need_init(ctx);
    if (s != PDIPC_OK) return s;
    if (!x || !coll_diag || !coll_rhs) return fail(ctx, PDIPC_ERR_ARG, "null argument");
    return guarded(ctx, [&]() { return ctx->solver->stage_contact(x, coll_diag, coll_rhs, n_active, ctx->err); });
}

pdipc_status pdipc_stage_pd(pdipc_ctx* ctx, const double* X, const double* V, double* out_X) {
    pdipc_status s = need_init(ctx);
    if (s != PDIPC_OK) return s;
    if (!X || !V || !out_X) return fail(ctx, PDIPC_ERR_ARG, "null argument");
    return guarded(ctx, [&]() { return ctx->solver->stage_pd(X, V, out_X, ctx->err); });
}

pdipc_status pdipc_stage_sweep_timing(pdipc_ctx* ctx, int launches, double* avg_ms, double* bytes) {
    pdipc_status s = need_init(ctx);
    if (s != PDIPC_OK) return s;
    if (!avg_ms || !bytes || launches <= 0) return fail(ctx, PDIPC_ERR_ARG, "bad argument");
    return guarded(ctx, [&]() { return ctx->solver->sweep_timing(launches, avg_ms, bytes, ctx->err); });
}

pdipc_status pdipc_stage_local_timing(pdipc_ctx* ctx, int launches, double* avg_ms, double* bytes) {
    pdipc_status s = need_init(ctx);
    if (s != PDIPC_OK) return s;
    if (!avg_ms || !bytes || launches <= 0) return fail(ctx, PDIPC_ERR_ARG, "bad argument");
    return guarded(ctx, [&]() { return ctx->solver->local_timing(launches, avg_ms, bytes, ctx->err); });
}

pdipc_status pdipc_stage_penalty_predict(pdipc_ctx* ctx, const double* X, double* V, double* sn) {
    pdipc_status s = need_init(ctx);
    if (s != PDIPC_OK) return s;
    if (!X || !V || !sn) return fail(ctx, PDIPC_ERR_ARG, "null argument");
    return guarded(ctx, [&]() { return ctx->solver->stage_penalty_predict(X, V, sn, ctx->err); });
}

pdipc_status pdipc_stage_penalty_ccd(pdipc_ctx* ctx, const double* x0, const double* dir, double stiffness,
                                     double damping, double* V, double* force, int* times) {
    pdipc_status s = need_init(ctx);
    if (s != PDIPC_OK) return s;
    if (!x0 || !dir || !V || !force || !times) return fail(ctx, PDIPC_ERR_ARG, "null argument");
    return guarded(ctx, [&]() {
        return ctx->solver->stage_penalty(0, x0, dir, nullptr, 0, stiffness, 0.0, damping, V, force, times,
                                          ctx->err);
    });
}

pdipc_status pdipc_stage_penalty_floor(pdipc_ctx* ctx, const double* x, double stiffness, double damping, double* V,
                                       double* force, int* times) {
    pdipc_status s = need_init(ctx);
    if (s != PDIPC_OK) return s;
    if (!x || !V || !force || !times) return fail(ctx, PDIPC_ERR_ARG, "null argument");
    return guarded(ctx, [&]() {
        return ctx->solver->stage_penalty(1, x, nullptr, nullptr, 0, stiffness, 0.0, damping, V, force, times,
                                          ctx->err);
    });
}

pdipc_status pdipc_stage_penalty_dcd(pdipc_ctx* ctx, const double* x, const int* face_pairs, int64_t n_pairs,
                                     double stiffness, double self_stiffness, double damping, double* V,
                                     double* force, int* times) {
    pdipc_status s = need_init(ctx);
    if (s != PDIPC_OK) return s;
    if (!x || !V || !force || !times || n_pairs < 0 || (n_pairs > 0 && !face_pairs))
        return fail(ctx, PDIPC_ERR_ARG, "null argument or negative pair count");
    return guarded(ctx, [&]() {
        return ctx->solver->stage_penalty(2, x, nullptr, face_pairs, n_pairs, stiffness, self_stiffness, damping,
                                          V, force, times, ctx->err);
    });
}

pdipc_status pdipc_adjoint_record(pdipc_ctx* ctx, int checkpoint_every) {
    pdipc_status s = need_init(ctx);
    if (s != PDIPC_OK) return s;
    return guarded(ctx, [&]() { return ctx->solver->adjoint_record(checkpoint_every, ctx->err); });
}

pdipc_status pdipc_adjoint_backward(pdipc_ctx* ctx, const double* dl_dx, const double* dl_dv, double* dl_dx0,
                                    double* dl_dv0, double* dl_dstrain) {
    pdipc_status s = need_init(ctx);
    if (s != PDIPC_OK) return s;
    if (!dl_dx || !dl_dx0 || !dl_dv0) return fail(ctx, PDIPC_ERR_ARG, "null argument");
    return guarded(ctx, [&]() {
        return ctx->solver->adjoint_backward(dl_dx, dl_dv, dl_dx0, dl_dv0, dl_dstrain, ctx->err);
    });
}

pdipc_status pdipc_mesh_topology(const double* X, int nv, const int* F, int nf, int patch_dim, int* edges,
                                 int cap_edges, int* n_edges, int* patch_off, int cap_patches, int* patch_faces,
                                 int cap_faces, int* n_patches, int* owner_of_point, int* owner_of_edge) {
    if (!X || !F || !n_edges || !n_patches || nv <= 0 || nf <= 0 || patch_dim <= 0) return PDIPC_ERR_ARG;
    return guarded(nullptr, [&]() {
        pdipc::MeshTopology t;
        std::string e = pdipc::build_mesh_topology(X, nv, F, nf, patch_dim, t);
        if (!e.empty()) return PDIPC_ERR_ARG;
        const int ne = (int)t.edges.size() / 2, np = (int)t.patches.size();
        *n_edges = ne;
        *n_patches = np;
        size_t nfaces = 0;
        for (auto& p : t.patches) nfaces += p.size();
        if (ne > cap_edges || np > cap_patches || (int64_t)nfaces > (int64_t)cap_faces) return PDIPC_ERR_OVERFLOW;
        if (edges) std::copy(t.edges.begin(), t.edges.end(), edges);
        if (patch_off && patch_faces) {
            int q = 0;
            patch_off[0] = 0;
            for (int p = 0; p < np; ++p) {
                for (int f : t.patches[p]) patch_faces[q++] = f;
                patch_off[p + 1] = q;
            }
        }
        if (owner_of_point)
            for (int f = 0; f < nf; ++f)
                for (int v : t.face_points_own[f]) owner_of_point[v] = f;
        if (owner_of_edge)
            for (int f = 0; f < nf; ++f)
                for (int v : t.face_edges_own[f]) owner_of_edge[v] = f;
        return PDIPC_OK;
    });
}

}  // extern "C"
