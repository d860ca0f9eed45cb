// solver.h — precision-independent interface of one PD-IPC context's device solver.
#pragma once

#include <memory>
#include <string>

#include "../../include/pdipc.h"
#include "host_tables.h"

namespace pdipc {

class SolverBase {
public:
    virtual ~SolverBase() = default;
    // Upload the tables and build the patch tree.  Returns "" or an error.
    virtual pdipc_status init(const HostTables& H, const pdipc_params& p, std::string& err) = 0;
    virtual pdipc_status step(int n, std::string& err) = 0;
    virtual pdipc_status get_positions(double* out, std::string& err) = 0;
    virtual pdipc_status get_velocities(double* out, std::string& err) = 0;
    virtual pdipc_status set_state(const double* X, const double* V, std::string& err) = 0;
    virtual pdipc_status reset(std::string& err) = 0;
    virtual void stats(pdipc_stats* s) = 0;
    virtual pdipc_status stage_broadphase(const double* xo, const double* dx, int* pairs, int64_t cap_pairs,
                                          int64_t* n_pairs, int* pt, int64_t cap_pt, int64_t* n_pt, int* ee,
                                          int64_t cap_ee, int64_t* n_ee, std::string& err) = 0;
    virtual pdipc_status stage_morton(uint64_t* codes, int* order, int cap, std::string& err) = 0;
    virtual pdipc_status stage_toi(const double* x0, const double* x1, double* tpt, double* tee, double* tg,
                                   std::string& err) = 0;
    virtual pdipc_status stage_toi_noalloc(const double* x0, const double* x1, double* tpt, double* tee,
                                           double* tg, std::string& err) = 0;
    virtual pdipc_status stage_contact(const double* x, double* diag, double* rhs, int64_t* n_active,
                                       std::string& err) = 0;
    virtual pdipc_status stage_pd(const double* X, const double* V, double* out, std::string& err) = 0;
    virtual pdipc_status sweep_timing(int launches, double* avg_ms, double* bytes, std::string& err) = 0;
    virtual pdipc_status local_timing(int launches, double* avg_ms, double* bytes, std::string& err) = 0;
    // penalty / discrete-collision stages; kind: 0 CCD candidates, 1 floor, 2 face pairs
    virtual pdipc_status stage_penalty_predict(const double* X, double* V, double* sn, std::string& err) = 0;
    virtual pdipc_status stage_penalty(int kind, const double* x, const double* dir, const int* face_pairs,
                                       int64_t n_pairs, double k, double k_self, double damping, double* V,
                                       double* force, int* times, std::string& err) = 0;
    // discrete adjoint of recorded contact-free steps (FP64 form): every > 0
    // starts recording with a checkpoint every `every` steps, 0 drops it
    virtual pdipc_status adjoint_record(int every, std::string& err) = 0;
    virtual pdipc_status adjoint_backward(const double* gx, const double* gv, double* gx0, double* gv0, double* gk,
                                          std::string& err) = 0;
    // limit of the persistent solve's device-side waits, microseconds (0 = 2 s)
    virtual void set_wait_limit(int us) = 0;
    virtual void tuning(pdipc_tuning* out) = 0;
    virtual int n_sim() const = 0;
    virtual int n_total() const = 0;
};

std::unique_ptr<SolverBase> make_solver(int precision);

}  // namespace pdipc
