// solver.cu — one PD-IPC context on one GPU: device tables, the step loop
// (PdIpcSimulator::advance, Simulator/PD-IPC/PdIpcSimulator.cpp:1683-1796),
// the patch broad phase (gpuCcdCulling, cpp:1799-1869) and the stage entry
// points.
//
// The reference's stopping rule (cpp:1774-1779) is tested on the device after
// each outer iteration; the host reads its 16-byte record, and with the
// persistent solve it has already enqueued the next iteration, whose kernels
// return at entry if the rule stopped the loop.  The time of impact stays on
// the device (the reference copies it to the host, cu:2738-2740).  On the
// per-sweep path the projective-dynamics solve of an outer iteration
// (1 + lg x (2 + 2 cheby - 1) kernels) is captured once as a CUDA graph and
// replayed.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include <array>
#include <map>
#include <mutex>
#include <string>
#include <type_traits>

#include "kernels.cuh"
#include "persistent.h"
#include "solver.h"

namespace pdipc {

namespace {

template <typename T>
T omega_first(T rho2) {  // PdIpcGpuFunc.cu:1321: 2.0 / (2 - rho), stored in the working type
    const T d = T(2) - rho2;
    return (T)(2.0 / (double)d);
}
template <typename T>
T omega_next(T rho2, T omega) {  // PdIpcGpuFunc.cu:1341
    const T d = T(4) - rho2 * omega;
    return (T)(4.0 / (double)d);
}

struct Pinned {
    int64_t n_pairs;
    int64_t n_pt;
    int64_t n_ee;
    int n_pair_total_i32;
    unsigned int err;
    unsigned long long active;
    double toi;
    float toi_f;
    OuterGate gate[2];  // stopping-test records of the last two outer iterations
};

}  // namespace

#define PD_CK(call)                                                                       \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess) {                                                          \
            err = std::string(#call) + ": " + cudaGetErrorString(e_);                     \
            return PDIPC_ERR_CUDA;                                                        \
        }                                                                                 \
    } while (0)

template <typename T, typename TC>
class Solver final : public SolverBase {
public:
    Solver() = default;
    ~Solver() override { release(); }

    int n_sim() const override { return d_.nsim; }
    int n_total() const override { return d_.ntot; }

    // Device-side wait limit of the persistent solve, converted to SM clock
    // cycles at the device's maximum clock (clock64 counts cycles); 0 = 2 s.
    void set_wait_limit(int us) override {
        const long long u = us > 0 ? (long long)us : 2000000ll;
        wait_cycles_ = std::max(1ll, u * (long long)clock_khz_ / 1000ll);
        if constexpr (std::is_same<T, float>::value) pargs_.timeout = wait_cycles_;
    }

    pdipc_status init(const HostTables& H, const pdipc_params& p, std::string& err) override {
        prm_ = p;
        c_.dt = p.time_step;
        c_.gravity = p.gravity;
        c_.dhat = p.dhat;
        c_.kappa = p.kappa;
        c_.infl = p.inflation_radius < 0 ? 0.5 * p.dhat : p.inflation_radius;
        c_.relax = p.jacobi_relax;
        c_.rho = p.cheby_rho;
        c_.toi_scale = p.toi_scale;
        c_.ccd_slack = p.ccd_slack;
        c_.ccd_eta = p.ccd_eta;
        c_.static_mass = p.static_mass;
        c_.lg = p.lg_iterations;
        c_.cheby = p.cheby_iterations;
        c_.ccd_max_iter = p.ccd_max_iter;
        if (c_.lg < 1 || c_.cheby < 1 || p.max_outer < 1 || p.time_step <= 0) {
            err = "lg_iterations, cheby_iterations, max_outer and time_step must be positive";
            return PDIPC_ERR_ARG;
        }
        if (p.wait_limit_us < 0) {
            err = "wait_limit_us must not be negative";
            return PDIPC_ERR_ARG;
        }
        if (p.ccd_mode < 0 || p.ccd_mode > 2) {
            err = "ccd_mode must be 0 (additive CCD), 1 (plus the FP64 coplanarity cubic) or 2 (the cubic alone)";
            return PDIPC_ERR_ARG;
        }
        c_.ccd_mode = p.ccd_mode;
        {
            int khz = 0;
            PD_CK(cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, p.device));
            clock_khz_ = khz > 0 ? khz : 2000000;
        }
        set_wait_limit(p.wait_limit_us);
        PD_CK(cudaStreamCreateWithFlags(&s_, cudaStreamNonBlocking));
        PD_CK(cudaEventCreate(&ev0_));
        PD_CK(cudaEventCreate(&ev1_));
        for (auto& ring : evo_)
            for (cudaEvent_t& e : ring) PD_CK(cudaEventCreate(&e));
        Dev<T, TC>& d = d_;
        d.nsim = H.nsim;
        d.ntot = H.ntot;
        num_sim_models_ = H.nsim > 0 ? 1 : 0;
        for (int i = 1; i < H.nsim; ++i) num_sim_models_ += H.vertexModel[i] != H.vertexModel[i - 1];
        d.nface = (int)H.faces.size() / 3;
        d.nedge = (int)H.edges.size() / 2;
        d.npatch = H.npatch;
        const int ns = d.nsim, nt = d.ntot;

        // ---- vertex state ----
        std::vector<V4<TC>> X(nt);
        for (int i = 0; i < nt; ++i) X[i] = V4<TC>{(TC)H.X[3 * i], (TC)H.X[3 * i + 1], (TC)H.X[3 * i + 2], TC(0)};
        PD_CK(up(d.P, X));
        PD_CK(up(d.Xrest, X));
        PD_CK(up(d.Pold, X));
        if (kCorrection) {
            PD_CK(zeros(d.Ph, nt));
            PD_CK(zeros(d.Pl, nt));
            PD_CK(zeros(d.Poh, nt));
            PD_CK(zeros(d.Pol, nt));
            PD_CK(zeros(d.Dh, nt));
            PD_CK(zeros(sh_, nt));
            PD_CK(zeros(sl_, nt));
            launch_split(d, d.P, d.Ph, d.Pl, nt, s_);
            launch_split(d, d.Pold, d.Poh, d.Pol, nt, s_);
        }
        PD_CK(zeros(d.X0, ns));
        PD_CK(zeros(d.Vel, ns));
        PD_CK(zeros(d.Dir, nt));
        // iterates: row order on the per-sweep path, slot order (a multiple of
        // 64 slots) on the persistent one
        const int nslot = (ns + 63) / 64 * 64;
        PD_CK(zeros(d.Y, nslot));
        PD_CK(zeros(d.B, nslot));
        PD_CK(zeros(d.Aq, ns));
        PD_CK(zeros(d.Rhs, ns));
        PD_CK(zeros(d.Rhs0, ns));
        PD_CK(zeros(d.Dinert, ns));
        PD_CK(zeros(d.InvD, ns));
        PD_CK(zeros(d.CollDiag, nt));
        PD_CK(zeros(d.CollRhs, nt));
        PD_CK(zeros(scratch_, nt));
        PD_CK(up(vModel_, H.vertexModel));
        std::vector<V4<T>> grav(ns), pinr(ns);
        std::vector<T> invm(ns), de(ns), cn(ns), st(ns);
        std::vector<int> pinf(ns);
        const T g = (T)p.gravity;
        for (int i = 0; i < ns; ++i) {
            grav[i] = V4<T>{T(0), g * (T)H.mass[i], T(0), T(0)};
            invm[i] = (T)(1.0 / H.mass[i]);
            de[i] = (T)H.Delastic[i];
            cn[i] = (T)H.curvNorm[i];
            st[i] = (T)H.strain[i];
            pinf[i] = H.pinSlot[i];
            if (H.pinSlot[i] >= 0) {
                const T k = (T)H.pinK[H.pinSlot[i]];
                pinr[i] = V4<T>{k * (T)X[i].x, k * (T)X[i].y, k * (T)X[i].z, T(0)};
            } else {
                pinr[i] = V4<T>{T(0), T(0), T(0), T(0)};
            }
        }
        PD_CK(up(d.Grav, grav));
        PD_CK(up(d.PinRhs, pinr));
        PD_CK(up(d.InvMass, invm));
        PD_CK(up(d.Delastic, de));
        PD_CK(up(d.CurvNorm, cn));
        PD_CK(up(d.Strain, st));
        PD_CK(up(d.PinFlag, pinf));
        PD_CK(up(d.PinK, conv(H.pinK)));
        PD_CK(zeros(d.C, nslot));
        std::vector<TC> cm(nt, (TC)p.static_mass);
        for (int i = 0; i < ns; ++i) cm[i] = (TC)(T)H.collMassSim[i];
        PD_CK(up(d.CollMass, cm));

        // ---- tetrahedral strain constraints ----
        d.ntet = H.ntet;
        if (d.ntet > 0) {
            std::vector<int4> tets(d.ntet);
            for (int e = 0; e < d.ntet; ++e)
                tets[e] = make_int4(H.tets[4 * e], H.tets[4 * e + 1], H.tets[4 * e + 2], H.tets[4 * e + 3]);
            PD_CK(up(d.Tets, tets));
            PD_CK(up(d.TetIdm, conv(H.tetIdm)));
            PD_CK(up(d.TetW, conv(H.tetW)));
            PD_CK(zeros(d.TetOut, 4 * (size_t)d.ntet));
            PD_CK(up(d.vtPtr, H.vtPtr));
            PD_CK(up(d.vtIdx, H.vtIdx));
        }

        // ---- local-step stencils ----
        PD_CK(up(d.lPtr, H.lPtr));
        PD_CK(up(d.lNbr, H.lNbr));
        PD_CK(up(d.lRest, conv(H.lRest)));
        PD_CK(up(d.lLbo, conv(H.lLbo)));
        PD_CK(up(d.lBend, conv(H.lBend)));
        PD_CK(up(d.lBendT, conv(H.lBendT)));
        {   // and in SELL-32 order (padding: the row itself, zero weights, never read)
            const int nsl = (ns + kSlice - 1) / kSlice;
            std::vector<int> toff(nsl + 1, 0);
            for (int sl = 0; sl < nsl; ++sl) {
                int w = 0;
                for (int r = sl * kSlice; r < std::min(ns, (sl + 1) * kSlice); ++r)
                    w = std::max(w, H.lPtr[r + 1] - H.lPtr[r] - 1);
                toff[sl + 1] = toff[sl] + kSlice * w;
            }
            const size_t tsz = (size_t)std::max(toff[nsl], 1);
            std::vector<int> tn(tsz, 0);
            std::vector<T> tr(tsz, T(0)), tl(tsz, T(0)), tb(tsz, T(0)), b0(ns), l0(ns);
            for (int r = 0; r < ns; ++r) {
                const int sl = r / kSlice, b = H.lPtr[r], e = H.lPtr[r + 1], at = toff[sl] + r % kSlice;
                const int w = (toff[sl + 1] - toff[sl]) / kSlice;
                b0[r] = (T)H.lBend[b];
                l0[r] = (T)H.lLbo[b];
                for (int k = 0; k < w; ++k) {
                    const size_t q = (size_t)at + (size_t)kSlice * k;
                    const int s = b + 1 + k;
                    const bool live = s < e;
                    tn[q] = live ? H.lNbr[s] : r;
                    tr[q] = live ? (T)H.lRest[s] : T(0);
                    tl[q] = live ? (T)H.lLbo[s] : T(0);
                    tb[q] = live ? (T)H.lBendT[s] : T(0);
                }
            }
            PD_CK(up(d.tOff, toff));
            PD_CK(up(d.tNbr, tn));
            PD_CK(up(d.tRest, tr));
            PD_CK(up(d.tLbo, tl));
            PD_CK(up(d.tBendT, tb));
            PD_CK(up(d.tBend0, b0));
            PD_CK(up(d.tLbo0, l0));
        }

        // ---- system matrix in SELL-32 ----
        d.nslice = (ns + kSlice - 1) / kSlice;
        std::vector<int> soff(d.nslice + 1, 0), slen(d.nslice, 0);
        for (int sl = 0; sl < d.nslice; ++sl) {
            int w = 0;
            for (int r = sl * kSlice; r < std::min(ns, (sl + 1) * kSlice); ++r) w = std::max(w, H.nPtr[r + 1] - H.nPtr[r]);
            slen[sl] = w;
            soff[sl + 1] = soff[sl] + kSlice * w;
        }
        std::vector<int> scol(soff[d.nslice], 0);
        std::vector<T> sval(soff[d.nslice], T(0));
        for (int sl = 0; sl < d.nslice; ++sl)
            for (int lane = 0; lane < kSlice; ++lane) {
                const int r = sl * kSlice + lane;
                const int len = r < ns ? H.nPtr[r + 1] - H.nPtr[r] : 0;
                for (int k = 0; k < slen[sl]; ++k) {
                    const size_t at = (size_t)soff[sl] + (size_t)kSlice * k + lane;
                    if (k < len) {
                        scol[at] = H.nCol[H.nPtr[r] + k];
                        sval[at] = (T)H.nVal[H.nPtr[r] + k];
                    } else {
                        scol[at] = r < ns ? r : 0;  // padding: own row, zero weight
                        sval[at] = T(0);
                    }
                }
            }
        sell_entries_ = (int64_t)H.nPtr[ns];
        {   // algorithmic bytes of one PD solve (the stats field pd_solve_bytes)
            const double V = sizeof(T);
            double b = 0.0, lb = 0.0;
            for (int i = 0; i < ns; ++i) {
                const double d1 = H.lPtr[i + 1] - H.lPtr[i];  // self + stencil neighbours
                const double n = H.nPtr[i + 1] - H.nPtr[i];   // matrix off-diagonals
                const double local = d1 * (4.0 + 3.0 * V) + 2.0 * V + 8.0 + 9.0 * V;
                const double sweep = n * (4.0 + V) + 7.0 * V;
                b += local + 2.0 * c_.cheby * sweep + (c_.cheby - 1) * 3.0 * V;
                lb += local + sweep;
            }
            pd_bytes_ = b * c_.lg;
            local_bytes_ = lb;
        }
        sell_padded_ = (int64_t)soff[d.nslice];
        PD_CK(up(d.sOff, soff));
        PD_CK(up(d.sLen, slen));
        PD_CK(up(d.sCol, scol));
        PD_CK(up(d.sVal, sval));
        {   // column-offset patterns for the per-row kernels, kept only when
            // rows share them (a table at most an eighth of the rows' count)
            int patW = 0;
            for (int w : slen) patW = std::max(patW, w);
            std::map<std::vector<int16_t>, int> pats;
            std::vector<int> rp(std::max(ns, 1), 0);
            bool share = patW > 0;
            std::vector<int16_t> o(patW);
            for (int i = 0; i < ns && share; ++i) {
                std::fill(o.begin(), o.end(), (int16_t)0);
                for (int e = H.nPtr[i]; e < H.nPtr[i + 1]; ++e) {
                    const int off = H.nCol[e] - i;
                    if (off < -32768 || off > 32767) {
                        share = false;
                        break;
                    }
                    o[e - H.nPtr[i]] = (int16_t)off;
                }
                rp[i] = pats.emplace(o, (int)pats.size()).first->second;
                if ((int64_t)pats.size() * 8 > (int64_t)ns + 64) share = false;
            }
            if (share) {
                std::vector<int16_t> tab(pats.size() * (size_t)patW);
                for (auto& kv : pats) std::copy(kv.first.begin(), kv.first.end(), tab.begin() + (size_t)kv.second * patW);
                PD_CK(up(d.rowPat, rp));
                PD_CK(up(d.patOff, tab));
                d.patW = patW;
            }
        }

        // ---- collision topology ----
        std::vector<int4> faces(d.nface);
        for (int f = 0; f < d.nface; ++f) faces[f] = make_int4(H.faces[3 * f], H.faces[3 * f + 1], H.faces[3 * f + 2], 0);
        std::vector<int2> edges(d.nedge);
        for (int e = 0; e < d.nedge; ++e) edges[e] = make_int2(H.edges[2 * e], H.edges[2 * e + 1]);
        PD_CK(up(d.Faces, faces));
        PD_CK(up(d.Edges, edges));
        PD_CK(up(d.pfPtr, H.pfPtr));
        PD_CK(up(d.pfIdx, H.pfIdx));
        PD_CK(up(d.ppPtr, H.ppPtr));
        PD_CK(up(d.ppIdx, H.ppIdx));
        PD_CK(up(d.pePtr, H.pePtr));
        PD_CK(up(d.peIdx, H.peIdx));
        PD_CK(up(d.pxPtr, H.pxPtr));
        PD_CK(up(d.pxIdx, H.pxIdx));
        PD_CK(up(d.pStatic, H.pStatic));
        const int np = std::max(1, d.npatch);
        PD_CK(zeros(d.PatchBox, np));
        PD_CK(zeros(d.NodeBox, 2 * np));
        PD_CK(zeros(d.NodeChild, np));
        PD_CK(zeros(d.NodeParent, 2 * np));
        PD_CK(zeros(d.NodeEscape, 2 * np));
        PD_CK(zeros(d.PairCount, 1));
        PD_CK(zeros(d.LeafPatch, np));
        PD_CK(zeros(d.RefitFlag, np));
        PD_CK(zeros(d.Morton, np));

        // ---- scalars ----
        PD_CK(zeros(d.ToiMin, 1));
        const TC one = TC(1);
        PD_CK(cudaMemcpyAsync(d.ToiMin, &one, sizeof(TC), cudaMemcpyHostToDevice, s_));
        PD_CK(zeros(d.Toi, 1));
        PD_CK(zeros(d.ResidPart, direction_blocks(ns)));
        PD_CK(zeros(d.Resid, 1));
        PD_CK(zeros(d.ErrFlags, 1));
        PD_CK(zeros(d.ActiveCount, 1));
        PD_CK(zeros(gate_, 1));
        if (prm_.instance_stop) {
            // the instances: simulated models, each a contiguous run of vertices
            std::vector<int> vinst(nt, -1), beg(1, 0);
            for (int i = 0; i < ns; ++i) {
                if (i > 0 && H.vertexModel[i] != H.vertexModel[i - 1]) beg.push_back(i);
                vinst[i] = (int)beg.size() - 1;
            }
            beg.push_back(ns);
            d.ninst = ns > 0 ? (int)beg.size() - 1 : 0;
            std::vector<TC> ones(std::max(d.ninst, 1), TC(1));
            PD_CK(up(d.VInst, vinst));
            PD_CK(up(d.InstBeg, beg));
            PD_CK(zeros(d.InstStop, std::max(d.ninst, 1)));
            PD_CK(zeros(d.InstResid, std::max(d.ninst, 1)));
            PD_CK(up(d.InstToiMin, ones));
            PD_CK(up(d.InstToi, ones));
            PD_CK(zeros(d.InstIters, std::max(d.ninst, 1)));
            instIters_.assign(std::max(d.ninst, 1), 0);
        }
        PD_CK(cudaMallocHost(&pin_, sizeof(Pinned)));
        std::memset(pin_, 0, sizeof(Pinned));
        PD_CK(cudaMallocHost(&stage_, sizeof(V4<TC>) * (size_t)std::max(nt, 1)));

        // ---- persistent PD solve plan (needs every buffer above) ----
        pdipc_status pr = plan_persistent(H, err);
        if (pr != PDIPC_OK) return pr;

        // ---- patch tree at the rest positions (AipcBvhs::init at initialization) ----
        pdipc_status r = build_tree(true, err);
        if (r != PDIPC_OK) return r;
        PD_CK(cudaStreamSynchronize(s_));
        fill_tuning_record();
        if (prm_.autotune) {
            r = autotune(H, err);
            if (r != PDIPC_OK) return r;
        }
        inited_ = true;
        return PDIPC_OK;
    }

    void tuning(pdipc_tuning* out) override { *out = tuning_; }

private:
    // ---------------- autotuner ----------------
    struct Tuned {
        PlanChoice pd;
        int cand_grid, trav_block, expand_block;
    };

    void fill_tuning_record() {
        tuning_.pd_rows_per_thread = plan_.enabled ? plan_.rows_per_thread : 0;
        tuning_.pd_ctas = plan_.enabled ? plan_.ctas : 0;
        tuning_.pd_launches = plan_.enabled ? (int)groups_.size() : 0;
        tuning_.pd_band = plan_.enabled && plan_.own_max > 0;
        tuning_.pd_l1_gather = plan_.enabled && plan_.l1_gather;
        tuning_.pd_local_sync = plan_.enabled && plan_.local_sync;
        tuning_.cand_grid = c_.cand_grid;
        tuning_.traverse_block = c_.trav_block;
        tuning_.expand_block = c_.expand_block;
    }

    PlanChoice current_choice() const {
        PlanChoice ch;
        if (!plan_.enabled) return ch;
        ch.rows_per_thread = plan_.rows_per_thread;
        ch.band = plan_.own_max > 0;
        ch.l1_gather = plan_.l1_gather;
        ch.local_sync = plan_.local_sync;
        return ch;
    }

    // One outer iteration's PD solve from the predicted state in `start`
    // (positions and, in the correction form, their float-float mirror), timed
    // with CUDA events on the context's stream; mean of `reps` after one warm-up.
    pdipc_status time_pd_solve(const V4<TC>* start, const V4<T>* sh, const V4<T>* sl, int reps, float* ms_out,
                               std::string& err) {
        auto restore = [&]() -> cudaError_t {
            cudaError_t e = cudaMemcpyAsync(d_.P, start, sizeof(V4<TC>) * d_.nsim, cudaMemcpyDeviceToDevice, s_);
            if (e == cudaSuccess && sh)
                e = cudaMemcpyAsync(d_.Ph, sh, sizeof(V4<T>) * d_.nsim, cudaMemcpyDeviceToDevice, s_);
            if (e == cudaSuccess && sl)
                e = cudaMemcpyAsync(d_.Pl, sl, sizeof(V4<T>) * d_.nsim, cudaMemcpyDeviceToDevice, s_);
            return e;
        };
        auto solve = [&]() -> cudaError_t {
            if (plan_.enabled) return launch_persistent();
            enqueue_pd();
            return cudaGetLastError();
        };
        float total = 0.f;
        for (int k = -1; k < reps; ++k) {
            PD_CK(restore());
            PD_CK(cudaEventRecord(ev0_, s_));
            PD_CK(solve());
            PD_CK(cudaEventRecord(ev1_, s_));
            PD_CK(cudaEventSynchronize(ev1_));
            float ms = 0.f;
            PD_CK(cudaEventElapsedTime(&ms, ev0_, ev1_));
            if (k >= 0) total += ms;
        }
        pin_->err = 0;
        PD_CK(cudaMemcpyAsync(&pin_->err, d_.ErrFlags, sizeof(unsigned int), cudaMemcpyDeviceToHost, s_));
        PD_CK(cudaStreamSynchronize(s_));
        if (pin_->err) {  // a device wait gave up: this configuration is not usable here
            PD_CK(cudaMemsetAsync(d_.ErrFlags, 0, sizeof(unsigned int), s_));
            PD_CK(cudaMemsetAsync(pBar_ + 1, 0, sizeof(unsigned), s_));
            *ms_out = -1.f;
            return PDIPC_OK;
        }
        *ms_out = total / (float)reps;
        return PDIPC_OK;
    }

    // The broad phase, the time-of-impact pass and the contact pass over the
    // candidates of the current positions, timed with CUDA events.
    pdipc_status time_collision(int reps, float* ms_out, std::string& err) {
        float total = 0.f;
        for (int k = -1; k < reps; ++k) {
            PD_CK(cudaEventRecord(ev0_, s_));
            pdipc_status r = broadphase(err);
            if (r != PDIPC_OK) return r;
            launch_toi(d_, pos_old(), pos(), c_, (TC*)nullptr, (TC*)nullptr, s_);
            launch_toi_finalize(d_, c_, s_);
            launch_contact(d_, pos(), c_, s_);
            PD_CK(cudaEventRecord(ev1_, s_));
            PD_CK(cudaEventSynchronize(ev1_));
            float ms = 0.f;
            PD_CK(cudaEventElapsedTime(&ms, ev0_, ev1_));
            if (k >= 0) total += ms;
        }
        *ms_out = total / (float)reps;
        return PDIPC_OK;
    }

    // Chooses, per mesh and precision, the persistent solve's configuration
    // (rows per thread and so CTA count, band, gathers, synchronisation, or
    // one launch per sweep) and the collision kernels' launch shapes (grid of
    // the candidate kernels, block sizes of the traversal and the expansion)
    // by timing every candidate with CUDA events at initialize, on the
    // predicted first step of the current state (restored afterwards).  The
    // choice is cached by shape for the process: later contexts of the same
    // shape take it without timing.  Every candidate computes the same
    // iteration; they differ in launch shape and, on the band path, in where a
    // row's sum splits between own and halo entries.
    pdipc_status autotune(const HostTables& H, std::string& err) {
        static std::mutex mu;
        static std::map<std::string, Tuned> cache;
        const std::string key = std::to_string(sizeof(T)) + "/" + std::to_string(sizeof(TC)) + "/" +
                                std::to_string(d_.nsim) + "/" + std::to_string(d_.ntot) + "/" +
                                std::to_string(d_.npatch) + "/" + std::to_string(sell_entries_) + "/" +
                                std::to_string(c_.lg) + "/" + std::to_string(c_.cheby) + "/" +
                                std::to_string(prm_.persistent) + "/" + std::to_string(d_.ntet);
        Tuned best{current_choice(), c_.cand_grid, c_.trav_block, c_.expand_block};
        bool cached = false;
        {
            std::lock_guard<std::mutex> g(mu);
            auto it = cache.find(key);
            if (it != cache.end()) {
                best = it->second;
                cached = true;
            }
        }
        if (cached) {
            pdipc_status r = plan_persistent(H, err, best.pd.rows_per_thread ? &best.pd : nullptr);
            if (r != PDIPC_OK) return r;
            if (best.pd.rows_per_thread == 0) plan_ = PersistPlan();
            c_.cand_grid = best.cand_grid;
            c_.trav_block = best.trav_block;
            c_.expand_block = best.expand_block;
            fill_tuning_record();
            tuning_.autotuned = 1;
            tuning_.from_cache = 1;
            return PDIPC_OK;
        }
        // ---- the PD solve: every configuration that fits, and one launch per sweep ----
        const int ns = d_.nsim;
        V4<TC>*saveP = nullptr, *saveV = nullptr, *start = nullptr;
        V4<T>*saveH = nullptr, *saveL = nullptr, *startH = nullptr, *startL = nullptr;
        PD_CK(alloc(saveP, ns));
        PD_CK(alloc(saveV, ns));
        PD_CK(alloc(start, ns));
        PD_CK(cudaMemcpyAsync(saveP, d_.P, sizeof(V4<TC>) * ns, cudaMemcpyDeviceToDevice, s_));
        PD_CK(cudaMemcpyAsync(saveV, d_.Vel, sizeof(V4<TC>) * ns, cudaMemcpyDeviceToDevice, s_));
        if (d_.Ph) {
            PD_CK(alloc(saveH, ns));
            PD_CK(alloc(saveL, ns));
            PD_CK(alloc(startH, ns));
            PD_CK(alloc(startL, ns));
            PD_CK(cudaMemcpyAsync(saveH, d_.Ph, sizeof(V4<T>) * ns, cudaMemcpyDeviceToDevice, s_));
            PD_CK(cudaMemcpyAsync(saveL, d_.Pl, sizeof(V4<T>) * ns, cudaMemcpyDeviceToDevice, s_));
        }
        launch_predict(d_, (TC)c_.dt, s_);
        PD_CK(cudaMemcpyAsync(start, d_.P, sizeof(V4<TC>) * ns, cudaMemcpyDeviceToDevice, s_));
        if (d_.Ph) {
            PD_CK(cudaMemcpyAsync(startH, d_.Ph, sizeof(V4<T>) * ns, cudaMemcpyDeviceToDevice, s_));
            PD_CK(cudaMemcpyAsync(startL, d_.Pl, sizeof(V4<T>) * ns, cudaMemcpyDeviceToDevice, s_));
        }
        std::vector<PlanChoice> pds;
        pds.push_back(current_choice());  // the default first
        for (const PlanChoice& c : plan_choices_)
            if (!(c.rows_per_thread == pds[0].rows_per_thread && c.band == pds[0].band &&
                  c.l1_gather == pds[0].l1_gather && c.local_sync == pds[0].local_sync))
                pds.push_back(c);
        if (pds[0].rows_per_thread != 0) pds.push_back(PlanChoice{});  // one launch per sweep
        float bestMs = -1.f;
        for (size_t k = 0; k < pds.size(); ++k) {
            pdipc_status r = plan_persistent(H, err, pds[k].rows_per_thread ? &pds[k] : nullptr);
            if (r != PDIPC_OK) return r;
            if (pds[k].rows_per_thread == 0) plan_ = PersistPlan();
            else if (!plan_.enabled) continue;
            float ms = -1.f;
            r = time_pd_solve(start, startH, startL, 3, &ms, err);
            if (r != PDIPC_OK) return r;
            ++tuning_.candidates_timed;
            if (std::getenv("PDIPC_AUTOTUNE_LOG"))  // every timed PD configuration, on stderr
                std::fprintf(stderr, "pdipc autotune: PD rows/thread %d band %d l1 %d nbr-sync %d ctas %d launches %d: %.4f ms\n",
                             plan_.enabled ? plan_.rows_per_thread : 0, plan_.enabled && plan_.own_max > 0,
                             plan_.enabled && plan_.l1_gather, plan_.enabled && plan_.local_sync,
                             plan_.enabled ? plan_.ctas : 0, plan_.enabled ? (int)groups_.size() : 0, ms);
            if (k == 0) tuning_.pd_default_ms = ms;
            if (ms > 0.f && (bestMs < 0.f || ms < bestMs)) {
                bestMs = ms;
                best.pd = pds[k];
            }
        }
        pdipc_status r = plan_persistent(H, err, best.pd.rows_per_thread ? &best.pd : nullptr);
        if (r != PDIPC_OK) return r;
        if (best.pd.rows_per_thread == 0) plan_ = PersistPlan();
        tuning_.pd_solve_ms = bestMs;
        // ---- the collision kernels' launch shapes, over the current candidates ----
        PD_CK(cudaMemcpyAsync(d_.P, saveP, sizeof(V4<TC>) * ns, cudaMemcpyDeviceToDevice, s_));
        if (d_.Ph) {
            PD_CK(cudaMemcpyAsync(d_.Ph, saveH, sizeof(V4<T>) * ns, cudaMemcpyDeviceToDevice, s_));
            PD_CK(cudaMemcpyAsync(d_.Pl, saveL, sizeof(V4<T>) * ns, cudaMemcpyDeviceToDevice, s_));
        }
        float collBest = -1.f;
        const int grids[] = {152 * 16, 152 * 4, 152 * 8, 152 * 32};
        const int tblocks[] = {128, 64};
        const int eblocks[] = {256, 128};
        for (int g : grids)
            for (int tb : tblocks)
                for (int eb : eblocks) {
                    c_.cand_grid = g;
                    c_.trav_block = tb;
                    c_.expand_block = eb;
                    float ms = 0.f;
                    r = time_collision(2, &ms, err);
                    if (r != PDIPC_OK) return r;
                    ++tuning_.candidates_timed;
                    if (g == grids[0] && tb == tblocks[0] && eb == eblocks[0]) tuning_.collision_default_ms = ms;
                    if (collBest < 0.f || ms < collBest) {
                        collBest = ms;
                        best.cand_grid = g;
                        best.trav_block = tb;
                        best.expand_block = eb;
                    }
                }
        c_.cand_grid = best.cand_grid;
        c_.trav_block = best.trav_block;
        c_.expand_block = best.expand_block;
        tuning_.collision_ms = collBest;
        // ---- the state as it was ----
        PD_CK(cudaMemcpyAsync(d_.P, saveP, sizeof(V4<TC>) * ns, cudaMemcpyDeviceToDevice, s_));
        PD_CK(cudaMemcpyAsync(d_.Vel, saveV, sizeof(V4<TC>) * ns, cudaMemcpyDeviceToDevice, s_));
        if (d_.Ph) {
            PD_CK(cudaMemcpyAsync(d_.Ph, saveH, sizeof(V4<T>) * ns, cudaMemcpyDeviceToDevice, s_));
            PD_CK(cudaMemcpyAsync(d_.Pl, saveL, sizeof(V4<T>) * ns, cudaMemcpyDeviceToDevice, s_));
        }
        PD_CK(cudaMemsetAsync(d_.CollDiag, 0, sizeof(T) * d_.ntot, s_));
        PD_CK(cudaMemsetAsync(d_.CollRhs, 0, sizeof(V4<T>) * d_.ntot, s_));
        PD_CK(cudaStreamSynchronize(s_));
        for (V4<TC>* p : {saveP, saveV, start}) dfree(p);
        for (V4<T>* p : {saveH, saveL, startH, startL}) dfree(p);
        launches_ = 0;
        fill_tuning_record();
        tuning_.autotuned = 1;
        {
            std::lock_guard<std::mutex> g(mu);
            cache[key] = best;
        }
        return PDIPC_OK;
    }

public:

    pdipc_status step(int n, std::string& err) override {
        if (!inited_) {
            err = "not initialized";
            return PDIPC_ERR_STATE;
        }
        if (n < 0) {
            err = "negative step count";
            return PDIPC_ERR_ARG;
        }
        launches_ = 0;
        device_ms_ = 0.0;
        pd_ms_ = 0.0;
        pd_solves_ = 0;
        ccd_ms_ = 0.0;
        contact_ms_ = 0.0;
        st_.max_outer_iters = 0;
        st_.total_outer_iters = 0;
        inst_outer_ = 0;
        for (int k = 0; k < n; ++k) {
            if (adj_every_ > 0) {
                pdipc_status r = adjoint_checkpoint(err);
                if (r != PDIPC_OK) {
                    adjoint_clear();
                    return r;
                }
            }
            PD_CK(cudaEventRecord(ev0_, s_));
            pdipc_status r = step_once(err);
            if (r != PDIPC_OK) {
                // a failed step has no well-defined end state to differentiate:
                // the recording ends here rather than count a step that never finished
                if (adj_every_ > 0) {
                    adjoint_clear();
                    err += " (the adjoint recording was dropped)";
                }
                return r;
            }
            if (adj_every_ > 0) ++adj_steps_;
            PD_CK(cudaEventRecord(ev1_, s_));
            PD_CK(cudaEventSynchronize(ev1_));
            float ms = 0.f;
            PD_CK(cudaEventElapsedTime(&ms, ev0_, ev1_));
            device_ms_ += ms;
        }
        return PDIPC_OK;
    }

    pdipc_status get_positions(double* out, std::string& err) override {
        PD_CK(cudaMemcpyAsync(stage_, d_.P, sizeof(V4<TC>) * d_.ntot, cudaMemcpyDeviceToHost, s_));
        PD_CK(cudaStreamSynchronize(s_));
        for (int i = 0; i < d_.ntot; ++i) {
            out[3 * (size_t)i] = (double)stage_[i].x;
            out[3 * (size_t)i + 1] = (double)stage_[i].y;
            out[3 * (size_t)i + 2] = (double)stage_[i].z;
        }
        return PDIPC_OK;
    }
    pdipc_status get_velocities(double* out, std::string& err) override {
        PD_CK(cudaMemcpyAsync(stage_, d_.Vel, sizeof(V4<TC>) * d_.nsim, cudaMemcpyDeviceToHost, s_));
        PD_CK(cudaStreamSynchronize(s_));
        for (int i = 0; i < d_.nsim; ++i) {
            out[3 * (size_t)i] = (double)stage_[i].x;
            out[3 * (size_t)i + 1] = (double)stage_[i].y;
            out[3 * (size_t)i + 2] = (double)stage_[i].z;
        }
        return PDIPC_OK;
    }
    pdipc_status upload_vec(V4<TC>* dst, const double* src, int n, std::string& err) {
        PD_CK(cudaStreamSynchronize(s_));
        for (int i = 0; i < n; ++i)
            stage_[i] = V4<TC>{(TC)src[3 * (size_t)i], (TC)src[3 * (size_t)i + 1], (TC)src[3 * (size_t)i + 2], TC(0)};
        PD_CK(cudaMemcpyAsync(dst, stage_, sizeof(V4<TC>) * n, cudaMemcpyHostToDevice, s_));
        PD_CK(cudaStreamSynchronize(s_));
        return PDIPC_OK;
    }
    pdipc_status set_state(const double* X, const double* V, std::string& err) override {
        adjoint_clear();  // the recorded trajectory no longer leads here
        return put_state(X, V, err);
    }
    // positions (and velocities) to the device without touching a recording
    pdipc_status put_state(const double* X, const double* V, std::string& err) {
        pdipc_status r = upload_vec(d_.P, X, d_.ntot, err);
        if (r != PDIPC_OK) return r;
        launch_split(d_, d_.P, d_.Ph, d_.Pl, d_.ntot, s_);
        if (V) return upload_vec(d_.Vel, V, d_.nsim, err);
        return PDIPC_OK;
    }
    pdipc_status reset(std::string& err) override {
        adjoint_clear();
        PD_CK(cudaMemcpyAsync(d_.P, d_.Xrest, sizeof(V4<TC>) * d_.ntot, cudaMemcpyDeviceToDevice, s_));
        launch_split(d_, d_.P, d_.Ph, d_.Pl, d_.ntot, s_);
        PD_CK(cudaMemsetAsync(d_.Vel, 0, sizeof(V4<TC>) * d_.nsim, s_));
        PD_CK(cudaStreamSynchronize(s_));
        st_.steps_done = 0;
        return PDIPC_OK;
    }
    void stats(pdipc_stats* s) override {
        *s = st_;
        s->n_sim = d_.nsim;
        s->n_total = d_.ntot;
        s->n_patches = d_.npatch;
        s->precision = prm_.precision;
        s->device_bytes = bytes_;
        s->kernel_launches = launches_;
        s->device_ms = device_ms_;
        s->pd_path = plan_.enabled ? (plan_.own_max > 0 ? 3 : plan_.matrix_in_smem ? 2 : 1) : 0;
        s->pd_ctas = plan_.enabled ? plan_.ctas : 0;
        s->pd_solves = pd_solves_;
        s->pd_solve_ms = pd_ms_;
        s->pd_solve_bytes = pd_bytes_;
        s->ccd_ms = ccd_ms_;
        s->contact_ms = contact_ms_;
        s->instances = d_.ninst > 0 ? d_.ninst : num_sim_models_;
        s->instance_outer_iters = prm_.instance_stop ? inst_outer_ : (int64_t)s->instances * st_.total_outer_iters;
    }

    // ---------------- stages ----------------
    pdipc_status stage_broadphase(const double* xo, const double* dx, int* pairs, int64_t cap_pairs,
                                  int64_t* n_pairs, int* pt, int64_t cap_pt, int64_t* n_pt, int* ee, int64_t cap_ee,
                                  int64_t* n_ee, std::string& err) override {
        pdipc_status r = upload_vec(d_.Pold, xo, d_.ntot, err);
        if (r == PDIPC_OK) r = upload_vec(d_.Dir, dx, d_.ntot, err);
        if (r != PDIPC_OK) return r;
        launch_split(d_, d_.Pold, d_.Poh, d_.Pol, d_.ntot, s_);
        launch_split(d_, d_.Dir, d_.Dh, (V4<T>*)nullptr, d_.ntot, s_);
        r = broadphase(err);
        if (r != PDIPC_OK) return r;
        PD_CK(cudaMemsetAsync(d_.Dir, 0, sizeof(V4<TC>) * d_.ntot, s_));
        if (d_.Dh) PD_CK(cudaMemsetAsync(d_.Dh, 0, sizeof(V4<T>) * d_.ntot, s_));
        *n_pairs = d_.nPairs;
        *n_pt = d_.nPT;
        *n_ee = d_.nEE;
        if (d_.nPairs > cap_pairs || d_.nPT > cap_pt || d_.nEE > cap_ee) {
            PD_CK(cudaStreamSynchronize(s_));
            return PDIPC_ERR_OVERFLOW;
        }
        if (d_.nPairs) PD_CK(cudaMemcpyAsync(pairs, d_.Pairs, sizeof(int2) * d_.nPairs, cudaMemcpyDeviceToHost, s_));
        if (d_.nPT) PD_CK(cudaMemcpyAsync(pt, d_.PT, sizeof(int4) * d_.nPT, cudaMemcpyDeviceToHost, s_));
        if (d_.nEE) PD_CK(cudaMemcpyAsync(ee, d_.EE, sizeof(int4) * d_.nEE, cudaMemcpyDeviceToHost, s_));
        PD_CK(cudaStreamSynchronize(s_));
        return PDIPC_OK;
    }
    pdipc_status stage_morton(uint64_t* codes, int* order, int cap, std::string& err) override {
        if (cap < d_.npatch) return PDIPC_ERR_OVERFLOW;
        if (d_.npatch == 0) return PDIPC_OK;
        PD_CK(cudaMemcpyAsync(codes, d_.Morton, sizeof(uint64_t) * d_.npatch, cudaMemcpyDeviceToHost, s_));
        PD_CK(cudaMemcpyAsync(order, d_.LeafPatch, sizeof(int) * d_.npatch, cudaMemcpyDeviceToHost, s_));
        PD_CK(cudaStreamSynchronize(s_));
        return PDIPC_OK;
    }
    pdipc_status stage_toi(const double* x0, const double* x1, double* tpt, double* tee, double* tg,
                           std::string& err) override {
        pdipc_status r = upload_vec(d_.Pold, x0, d_.ntot, err);
        if (r == PDIPC_OK) r = upload_vec(scratch_, x1, d_.ntot, err);
        if (r != PDIPC_OK) return r;
        launch_split(d_, d_.Pold, d_.Poh, d_.Pol, d_.ntot, s_);
        launch_split(d_, scratch_, sh_, sl_, d_.ntot, s_);
        TC *ppt = nullptr, *pee = nullptr;
        if (d_.nPT) PD_CK(cudaMalloc(&ppt, sizeof(TC) * d_.nPT));
        if (d_.nEE) PD_CK(cudaMalloc(&pee, sizeof(TC) * d_.nEE));
        launch_toi(d_, pos_old(), Pos<T, TC>{scratch_, sh_, sl_}, c_, ppt, pee, s_);
        launch_toi_finalize(d_, c_, s_);
        TC toi;
        PD_CK(cudaMemcpyAsync(&toi, d_.Toi, sizeof(TC), cudaMemcpyDeviceToHost, s_));
        std::vector<TC> hp(d_.nPT), he(d_.nEE);
        if (d_.nPT) PD_CK(cudaMemcpyAsync(hp.data(), ppt, sizeof(TC) * d_.nPT, cudaMemcpyDeviceToHost, s_));
        if (d_.nEE) PD_CK(cudaMemcpyAsync(he.data(), pee, sizeof(TC) * d_.nEE, cudaMemcpyDeviceToHost, s_));
        PD_CK(cudaStreamSynchronize(s_));
        cudaFree(ppt);
        cudaFree(pee);
        if (tpt) for (int64_t i = 0; i < d_.nPT; ++i) tpt[i] = (double)hp[i];
        if (tee) for (int64_t i = 0; i < d_.nEE; ++i) tee[i] = (double)he[i];
        if (tg) *tg = (double)toi;
        return PDIPC_OK;
    }
    // stage_toi without any allocation: the per-candidate results go to the
    // library's static device scratch and from there straight to the caller's
    // arrays.  Needs a double CCD scalar (FP64 and mixed modes).
    pdipc_status stage_toi_noalloc(const double* x0, const double* x1, double* tpt, double* tee, double* tg,
                                   std::string& err) override {
        if constexpr (!std::is_same<TC, double>::value) {
            err = "pdipc_stage_toi_noalloc: needs the FP64 or mixed precision mode";
            return PDIPC_ERR_ARG;
        } else {
            ToiScratch sc;
            PD_CK(toi_scratch(&sc));
            const int64_t n = d_.nPT + d_.nEE;
            if (n > sc.entries) {
                err = "pdipc_stage_toi_noalloc: " + std::to_string(n) + " candidates exceed the " +
                      std::to_string(sc.entries) + "-entry scratch";
                return PDIPC_ERR_OVERFLOW;
            }
            std::lock_guard<std::mutex> hold(*sc.lock);
            // Declared after the lock, so destroyed before it: on every return
            // path, including the error returns of PD_CK below, the stream
            // has drained (no kernel or copy still uses the shared array)
            // before another context may take the lock.
            struct Drain {
                cudaStream_t s;
                ~Drain() { cudaStreamSynchronize(s); }
            } drain{s_};
            pdipc_status r = upload_vec(d_.Pold, x0, d_.ntot, err);
            if (r == PDIPC_OK) r = upload_vec(scratch_, x1, d_.ntot, err);
            if (r != PDIPC_OK) return r;
            launch_split(d_, d_.Pold, d_.Poh, d_.Pol, d_.ntot, s_);
            launch_split(d_, scratch_, sh_, sl_, d_.ntot, s_);
            launch_toi(d_, pos_old(), Pos<T, TC>{scratch_, sh_, sl_}, c_, sc.ptr, sc.ptr + d_.nPT, s_);
            launch_toi_finalize(d_, c_, s_);
            TC toi = TC(1);
            PD_CK(cudaMemcpyAsync(&toi, d_.Toi, sizeof(TC), cudaMemcpyDeviceToHost, s_));
            if (tpt && d_.nPT)
                PD_CK(cudaMemcpyAsync(tpt, sc.ptr, sizeof(double) * d_.nPT, cudaMemcpyDeviceToHost, s_));
            if (tee && d_.nEE)
                PD_CK(cudaMemcpyAsync(tee, sc.ptr + d_.nPT, sizeof(double) * d_.nEE, cudaMemcpyDeviceToHost, s_));
            PD_CK(cudaStreamSynchronize(s_));
            if (tg) *tg = (double)toi;
            return PDIPC_OK;
        }
    }
    pdipc_status stage_contact(const double* x, double* diag, double* rhs, int64_t* n_active,
                               std::string& err) override {
        pdipc_status r = upload_vec(scratch_, x, d_.ntot, err);
        if (r != PDIPC_OK) return r;
        launch_split(d_, scratch_, sh_, sl_, d_.ntot, s_);
        launch_contact(d_, Pos<T, TC>{scratch_, sh_, sl_}, c_, s_);
        std::vector<T> hd(d_.ntot);
        std::vector<V4<T>> hr(d_.ntot);
        PD_CK(cudaMemcpyAsync(hd.data(), d_.CollDiag, sizeof(T) * d_.ntot, cudaMemcpyDeviceToHost, s_));
        PD_CK(cudaMemcpyAsync(hr.data(), d_.CollRhs, sizeof(V4<T>) * d_.ntot, cudaMemcpyDeviceToHost, s_));
        PD_CK(cudaMemcpyAsync(&pin_->active, d_.ActiveCount, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s_));
        PD_CK(cudaStreamSynchronize(s_));
        for (int i = 0; i < d_.ntot; ++i) {
            diag[i] = (double)hd[i];
            rhs[3 * (size_t)i] = (double)hr[i].x;
            rhs[3 * (size_t)i + 1] = (double)hr[i].y;
            rhs[3 * (size_t)i + 2] = (double)hr[i].z;
            if (kCorrection)  // the correction form accumulates w (target - x); report sum w target
                for (int k = 0; k < 3; ++k) rhs[3 * (size_t)i + k] += diag[i] * (double)(TC)x[3 * (size_t)i + k];
        }
        if (n_active) *n_active = (int64_t)pin_->active;
        PD_CK(cudaMemsetAsync(d_.CollDiag, 0, sizeof(T) * d_.ntot, s_));
        PD_CK(cudaMemsetAsync(d_.CollRhs, 0, sizeof(V4<T>) * d_.ntot, s_));
        PD_CK(cudaStreamSynchronize(s_));
        return PDIPC_OK;
    }
    pdipc_status stage_pd(const double* X, const double* V, double* out, std::string& err) override {
        std::vector<double> saveX(3 * (size_t)d_.ntot), saveV(3 * (size_t)d_.nsim);
        pdipc_status r = get_positions(saveX.data(), err);
        if (r == PDIPC_OK) r = get_velocities(saveV.data(), err);
        // put_state, not set_state: the state is restored below, so a
        // recording in progress stays valid across this diagnostic call
        if (r == PDIPC_OK) r = put_state(X, V, err);
        if (r != PDIPC_OK) return r;
        launch_predict(d_, (TC)c_.dt, s_);
        if (plan_.enabled) PD_CK(launch_persistent());
        else enqueue_pd();
        r = get_positions(out, err);
        pdipc_status r2 = put_state(saveX.data(), saveV.data(), err);
        return r != PDIPC_OK ? r : r2;
    }

    // ---------------- penalty / discrete-collision stages ----------------
    pdipc_status ensure_pen(std::string& err) {
        if (!pen_f_) {
            PD_CK(zeros(pen_d_, d_.ntot));
            PD_CK(zeros(pen_f_, d_.ntot));
            PD_CK(zeros(pen_v_, d_.nsim));
            PD_CK(zeros(pen_t_, d_.ntot));
        }
        return PDIPC_OK;
    }
    pdipc_status download_vec(const V4<TC>* src, double* dst, int n, std::string& err) {
        PD_CK(cudaMemcpyAsync(stage_, src, sizeof(V4<TC>) * n, cudaMemcpyDeviceToHost, s_));
        PD_CK(cudaStreamSynchronize(s_));
        for (int i = 0; i < n; ++i) {
            dst[3 * (size_t)i] = (double)stage_[i].x;
            dst[3 * (size_t)i + 1] = (double)stage_[i].y;
            dst[3 * (size_t)i + 2] = (double)stage_[i].z;
        }
        return PDIPC_OK;
    }
    pdipc_status stage_penalty_predict(const double* X, double* V, double* sn, std::string& err) override {
        pdipc_status r = ensure_pen(err);
        if (r == PDIPC_OK) r = upload_vec(scratch_, X, d_.nsim, err);
        if (r == PDIPC_OK) r = upload_vec(pen_v_, V, d_.nsim, err);
        if (r != PDIPC_OK) return r;
        launch_pen_predict(d_, scratch_, pen_v_, (TC)c_.dt, pen_f_, s_);
        PD_CK(cudaGetLastError());
        r = download_vec(pen_f_, sn, d_.nsim, err);
        if (r == PDIPC_OK) r = download_vec(pen_v_, V, d_.nsim, err);
        return r;
    }
    pdipc_status stage_penalty(int kind, const double* x, const double* dir, const int* fp, int64_t np, double k,
                               double ks, double damping, double* V, double* force, int* times,
                               std::string& err) override {
        pdipc_status r = ensure_pen(err);
        if (r != PDIPC_OK) return r;
        if (kind == 2) {
            for (int64_t i = 0; i < 2 * np; ++i)
                if (fp[i] < 0 || fp[i] >= d_.nface) {
                    err = "face index out of range";
                    return PDIPC_ERR_ARG;
                }
            if (np > penPairCap_) {
                dfree(penPairs_);
                PD_CK(alloc(penPairs_, (size_t)np));
                penPairCap_ = np;
            }
            if (np > 0) {
                PD_CK(cudaMemcpyAsync(penPairs_, fp, sizeof(int2) * np, cudaMemcpyHostToDevice, s_));
                PD_CK(cudaStreamSynchronize(s_));
            }
        }
        r = upload_vec(scratch_, x, d_.ntot, err);
        if (r == PDIPC_OK) r = upload_vec(pen_v_, V, d_.nsim, err);
        if (r == PDIPC_OK && kind == 0) r = upload_vec(pen_d_, dir, d_.ntot, err);
        if (r != PDIPC_OK) return r;
        PD_CK(cudaMemsetAsync(pen_f_, 0, sizeof(V4<TC>) * d_.ntot, s_));
        PD_CK(cudaMemsetAsync(pen_t_, 0, sizeof(int) * d_.ntot, s_));
        if (kind == 0)
            launch_pen_ccd(d_, scratch_, pen_d_, (TC)k, (TC)c_.ccd_eta, c_.ccd_max_iter, pen_f_, pen_t_, s_);
        else if (kind == 1)
            launch_pen_floor(d_, scratch_, (TC)k, pen_f_, pen_t_, s_);
        else
            launch_pen_dcd(d_, penPairs_, np, vModel_, scratch_, (TC)k, (TC)ks, pen_f_, pen_t_, s_);
        launch_pen_uniform(d_, pen_f_, pen_t_, (TC)damping, pen_v_, s_);
        PD_CK(cudaGetLastError());
        r = download_vec(pen_f_, force, d_.ntot, err);
        if (r == PDIPC_OK) r = download_vec(pen_v_, V, d_.nsim, err);
        if (r != PDIPC_OK) return r;
        PD_CK(cudaMemcpyAsync(times, pen_t_, sizeof(int) * d_.ntot, cudaMemcpyDeviceToHost, s_));
        PD_CK(cudaStreamSynchronize(s_));
        return PDIPC_OK;
    }

    pdipc_status sweep_timing(int launches, double* avg_ms, double* bytes, std::string& err) override {
        // one plain sweep of the solve's own kind (on the correction in the mixed form)
        const T w = (T)c_.relax;
        auto sweep = [&]() {
            if (kCorrection) launch_sweep_delta<T, TC>(d_, 0, d_.Y, nullptr, d_.B, w, T(0), s_);
            else launch_sweep<T, TC>(d_, d_.Y, nullptr, d_.B, w, T(0), s_);
        };
        launch_diag(d_, s_);
        sweep();  // warm
        PD_CK(cudaEventRecord(ev0_, s_));
        for (int k = 0; k < launches; ++k) sweep();
        PD_CK(cudaEventRecord(ev1_, s_));
        PD_CK(cudaEventSynchronize(ev1_));
        float ms = 0.f;
        PD_CK(cudaEventElapsedTime(&ms, ev0_, ev1_));
        *avg_ms = (double)ms / launches;
        const double vec = 3.0 * sizeof(T);
        *bytes = (double)sell_entries_ * (sizeof(int) + sizeof(T)) + (double)d_.nsim * (3.0 * vec + sizeof(T));
        return PDIPC_OK;
    }

    // The local step of the per-sweep path timed alone: the curvature kernel
    // and the right-hand-side kernel (residual in the correction form) with
    // the first Jacobi sweep fused, `launches` times back to back.  Positions
    // are read, never written.
    pdipc_status local_timing(int launches, double* avg_ms, double* bytes, std::string& err) override {
        const T w = (T)c_.relax;
        auto once = [&]() {
            launch_local_aq(d_, s_);
            if constexpr (kCorrection) launch_local_residual(d_, w, s_);
            else launch_local_rhs_sweep(d_, w, s_);
        };
        launch_diag(d_, s_);
        once();  // warm
        PD_CK(cudaEventRecord(ev0_, s_));
        for (int k = 0; k < launches; ++k) once();
        PD_CK(cudaEventRecord(ev1_, s_));
        PD_CK(cudaEventSynchronize(ev1_));
        float ms = 0.f;
        PD_CK(cudaEventElapsedTime(&ms, ev0_, ev1_));
        *avg_ms = (double)ms / launches;
        *bytes = local_bytes_;
        return PDIPC_OK;
    }

private:
    Pos<T, TC> pos() const { return Pos<T, TC>{d_.P, d_.Ph, d_.Pl}; }
    Pos<T, TC> pos_old() const { return Pos<T, TC>{d_.Pold, d_.Poh, d_.Pol}; }

    // ---------------- discrete adjoint (FP64 form, contact-free steps) ----------------
    // Recording keeps the state (positions and velocities of the simulated
    // vertices) at the start of every `every`-th step.  The backward pass walks
    // the checkpoint segments from the last: it replays a segment's steps to
    // regain each step's start state, then for each step from the last replays
    // it once more with the positions at the start of every local-global
    // iteration taped, and runs the step's adjoint (adjoint_kernels.cu) over
    // the tape, last iteration first.  A replayed outer iteration with a
    // clamped step or active contacts ends the pass with PDIPC_ERR_STATE: the
    // adjoint covers contact-free steps.
    static constexpr bool kAdjoint = std::is_same<T, double>::value && std::is_same<TC, double>::value;

    void adjoint_clear() {
        for (V4<TC>*& c : adj_ckpt_) dfree(c);
        adj_ckpt_.clear();
        adj_every_ = 0;
        adj_steps_ = 0;
    }

    pdipc_status adjoint_checkpoint(std::string& err) {
        if (adj_steps_ % adj_every_ == 0) {
            V4<TC>* c = nullptr;
            PD_CK(alloc(c, 2 * (size_t)d_.nsim));
            adj_ckpt_.push_back(c);
            PD_CK(cudaMemcpyAsync(c, d_.P, sizeof(V4<TC>) * d_.nsim, cudaMemcpyDeviceToDevice, s_));
            PD_CK(cudaMemcpyAsync(c + d_.nsim, d_.Vel, sizeof(V4<TC>) * d_.nsim, cudaMemcpyDeviceToDevice, s_));
        }
        return PDIPC_OK;  // step() counts the step once it has completed
    }

    pdipc_status adjoint_record(int every, std::string& err) override {
        if (every < 0) {
            err = "adjoint_record: negative checkpoint interval";
            return PDIPC_ERR_ARG;
        }
        adjoint_clear();
        if (every == 0) return PDIPC_OK;
        if (prm_.instance_stop) {
            err = "adjoint: not with per-instance stopping (params.instance_stop)";
            return PDIPC_ERR_STATE;
        }
        if (!kAdjoint) {
            err = "adjoint: the plain FP64 form only (precision PDIPC_PREC_FP64)";
            return PDIPC_ERR_STATE;
        }
        adj_every_ = every;
        return PDIPC_OK;
    }

    // copy a saved state (P then Vel, nsim each) into the context, or out of it
    pdipc_status adj_load(const V4<TC>* st, std::string& err) {
        PD_CK(cudaMemcpyAsync(d_.P, st, sizeof(V4<TC>) * d_.nsim, cudaMemcpyDeviceToDevice, s_));
        PD_CK(cudaMemcpyAsync(d_.Vel, st + d_.nsim, sizeof(V4<TC>) * d_.nsim, cudaMemcpyDeviceToDevice, s_));
        return PDIPC_OK;
    }
    pdipc_status adj_save(V4<TC>* st, std::string& err) {
        PD_CK(cudaMemcpyAsync(st, d_.P, sizeof(V4<TC>) * d_.nsim, cudaMemcpyDeviceToDevice, s_));
        PD_CK(cudaMemcpyAsync(st + d_.nsim, d_.Vel, sizeof(V4<TC>) * d_.nsim, cudaMemcpyDeviceToDevice, s_));
        return PDIPC_OK;
    }

    pdipc_status adj_buffers(std::string& err) {
        const int ns = d_.nsim, cb = c_.cheby;
        const int max_outer = prm_.fixed_outer > 0 ? prm_.fixed_outer : prm_.max_outer;
        const int tape = max_outer * c_.lg;
        if (adj_tape_cap_ < tape) {
            dfree(adj_tape_);
            PD_CK(alloc(adj_tape_, (size_t)tape * ns));
            adj_tape_cap_ = tape;
        }
        if ((int)adj_seg_.size() < adj_every_) {
            for (V4<TC>*& c : adj_seg_) dfree(c);
            adj_seg_.assign(adj_every_, nullptr);
            for (V4<TC>*& c : adj_seg_) PD_CK(alloc(c, 2 * (size_t)ns));
        }
        if (adj_ready_) return PDIPC_OK;
        int nslot = 0;
        PD_CK(cudaMemcpyAsync(&nslot, d_.lPtr + ns, sizeof(int), cudaMemcpyDeviceToHost, s_));
        PD_CK(cudaStreamSynchronize(s_));
        PD_CK(alloc(adj_lboT_, (size_t)nslot));
        PD_CK(alloc(adj_ntval_, (size_t)sell_padded_));
        PD_CK(alloc(adj_final_, 2 * (size_t)ns));
        PD_CK(alloc(adj_kb_, (size_t)ns));
        if (d_.ntet > 0) PD_CK(alloc(adj_eb_, 4 * (size_t)d_.ntet));
        for (V4<TC>** b : {&adj_pb_, &adj_vb_, &adj_r0b_, &adj_rb_, &adj_qb_, &adj_u_, &adj_rho_})
            PD_CK(alloc(*b, (size_t)ns));
        adj_xb_.assign(cb + 1, nullptr);
        adj_xs_.assign(cb + 1, nullptr);
        adj_ys_.assign(cb, nullptr);
        for (auto* v : {&adj_xb_, &adj_xs_, &adj_ys_})
            for (V4<TC>*& b : *v) PD_CK(alloc(b, (size_t)ns));
        if constexpr (kAdjoint) launch_adj_tables(d_, adj_lboT_, adj_ntval_, s_);
        PD_CK(cudaGetLastError());
        adj_ready_ = true;
        return PDIPC_OK;
    }

    // the adjoint of one step over its tape; adj_pb_/adj_vb_ hold the adjoints
    // of the step's output positions and velocities on entry and of its input
    // positions and velocities on return
    pdipc_status adjoint_step(std::string& err) {
        if constexpr (kAdjoint) {
            Dev<T, TC>& d = d_;
            const int ns = d.nsim, cb = c_.cheby;
            const T w = (T)c_.relax;
            const TC dt = (TC)c_.dt;
            const TC invt = (TC)((1.0 / (double)dt) * (double)(TC)(1.0 - (double)dt));  // as step_once
            std::vector<T> oms;
            {
                T rho2 = (T)c_.rho;
                rho2 = rho2 * rho2;
                T om = omega_first(rho2);
                for (int it = 1; it < cb; ++it) {
                    oms.push_back(om);
                    om = omega_next(rho2, om);
                }
            }
            launch_adj_step_begin(d, invt, adj_pb_, adj_vb_, adj_r0b_, s_);
            const size_t vb = sizeof(V4<TC>) * ns;
            for (int l = adj_tape_n_ - 1; l >= 0; --l) {
                V4<T>* x = adj_tape_ + (size_t)l * ns;
                // the iteration's forward iterates: X_0 = x, Y_t = S(X_t), X_{t+1} from Y_t
                PD_CK(cudaMemcpyAsync(d.P, x, vb, cudaMemcpyDeviceToDevice, s_));
                launch_local_aq(d, s_);
                launch_local_rhs_sweep(d, w, s_);
                PD_CK(cudaMemcpyAsync(adj_ys_[0], d.Y, vb, cudaMemcpyDeviceToDevice, s_));
                PD_CK(cudaMemcpyAsync(adj_xs_[0], x, vb, cudaMemcpyDeviceToDevice, s_));
                if (cb > 1) launch_sweep<T, TC>(d, adj_ys_[0], nullptr, adj_xs_[1], w, T(0), s_);
                for (int it = 1; it < cb; ++it) {
                    launch_sweep<T, TC>(d, adj_xs_[it], nullptr, adj_ys_[it], w, T(0), s_);
                    if (it + 1 < cb)
                        launch_sweep<T, TC>(d, adj_ys_[it], adj_xs_[it - 1], adj_xs_[it + 1], w, oms[it - 1], s_);
                }
                // reverse: Xb[cb] is the adjoint of the iteration's result
                for (int t = 0; t < cb; ++t) PD_CK(cudaMemsetAsync(adj_xb_[t], 0, vb, s_));
                PD_CK(cudaMemsetAsync(adj_rho_, 0, vb, s_));
                std::swap(adj_xb_[cb], adj_pb_);
                for (int it = cb - 1; it >= 1; --it) {
                    launch_adj_sweep(d, adj_ntval_, w, oms[it - 1], adj_xb_[it + 1], adj_xb_[it - 1], adj_ys_[it],
                                     adj_u_, false, adj_rho_, adj_kb_, s_);
                    launch_adj_sweep(d, adj_ntval_, w, T(1), adj_u_, (V4<T>*)nullptr, adj_xs_[it], adj_xb_[it], true,
                                     adj_rho_, adj_kb_, s_);
                }
                launch_adj_sweep(d, adj_ntval_, w, T(1), adj_xb_[1], (V4<T>*)nullptr, adj_ys_[0], adj_u_, false,
                                 adj_rho_, adj_kb_, s_);
                launch_adj_sweep(d, adj_ntval_, w, T(1), adj_u_, (V4<T>*)nullptr, adj_xs_[0], adj_xb_[0], true,
                                 adj_rho_, adj_kb_, s_);
                launch_adj_local(d, adj_lboT_, w, x, adj_rho_, adj_rb_, adj_qb_, adj_r0b_, adj_xb_[0], adj_kb_,
                                 adj_eb_, s_);
                std::swap(adj_xb_[0], adj_pb_);  // the adjoint of the previous iteration's result
            }
            launch_adj_step_end(d, (T)dt, adj_pb_, adj_vb_, adj_r0b_, s_);
            PD_CK(cudaGetLastError());
            return PDIPC_OK;
        } else {
            err = "adjoint: the plain FP64 form only";
            return PDIPC_ERR_STATE;
        }
    }

    pdipc_status adjoint_backward(const double* gx, const double* gv, double* gx0, double* gv0, double* gk,
                                  std::string& err) override {
        if (!kAdjoint) {
            err = "adjoint: the plain FP64 form only (precision PDIPC_PREC_FP64)";
            return PDIPC_ERR_STATE;
        }
        if (adj_every_ <= 0 || adj_steps_ == 0) {
            err = "adjoint_backward: no recorded steps (pdipc_adjoint_record, then pdipc_step)";
            return PDIPC_ERR_STATE;
        }
        if (!gx || !gx0 || !gv0) {
            err = "adjoint_backward: null gradient buffer";
            return PDIPC_ERR_ARG;
        }
        pdipc_status r = adj_buffers(err);
        if (r != PDIPC_OK) return r;
        const int ns = d_.nsim;
        const pdipc_stats st_saved = st_;
        const int64_t launches_saved = launches_;
        const double ms_saved = device_ms_, pd_saved = pd_ms_, ccd_saved = ccd_ms_, contact_saved = contact_ms_;
        const int64_t solves_saved = pd_solves_;
        r = adj_save(adj_final_, err);
        if (r != PDIPC_OK) return r;
        r = upload_vec(adj_pb_, gx, ns, err);
        if (r != PDIPC_OK) return r;
        if (gv) {
            r = upload_vec(adj_vb_, gv, ns, err);
            if (r != PDIPC_OK) return r;
        } else {
            PD_CK(cudaMemsetAsync(adj_vb_, 0, sizeof(V4<TC>) * ns, s_));
        }
        PD_CK(cudaMemsetAsync(adj_kb_, 0, sizeof(T) * ns, s_));
        const int nseg = (adj_steps_ + adj_every_ - 1) / adj_every_;
        for (int c = nseg - 1; c >= 0 && r == PDIPC_OK; --c) {
            const int s0 = c * adj_every_, s1 = std::min(s0 + adj_every_, adj_steps_);
            // start states of the segment's steps
            r = adj_load(adj_ckpt_[c], err);
            if (r == PDIPC_OK) r = adj_save(adj_seg_[0], err);
            for (int s = s0 + 1; s < s1 && r == PDIPC_OK; ++s) {
                r = step_once(err);
                if (r == PDIPC_OK) r = adj_save(adj_seg_[s - s0], err);
            }
            for (int s = s1 - 1; s >= s0 && r == PDIPC_OK; --s) {
                r = adj_load(adj_seg_[s - s0], err);
                if (r != PDIPC_OK) break;
                taping_ = true;
                adj_tape_n_ = 0;
                adj_contact_ = false;
                r = step_once(err);
                taping_ = false;
                if (r != PDIPC_OK) break;
                if (adj_contact_) {
                    err = "adjoint_backward: recorded step " + std::to_string(s) +
                          " has an outer iteration with a clamped step or active contacts; the adjoint covers "
                          "contact-free steps";
                    r = PDIPC_ERR_STATE;
                    break;
                }
                if (adj_tape_n_ > adj_tape_cap_) {
                    err = "adjoint_backward: local-global tape overflow";
                    r = PDIPC_ERR_STATE;
                    break;
                }
                r = adjoint_step(err);
            }
        }
        taping_ = false;
        std::string e2;
        const pdipc_status rl = adj_load(adj_final_, e2);
        st_ = st_saved;
        launches_ = launches_saved;
        device_ms_ = ms_saved;
        pd_ms_ = pd_saved;
        ccd_ms_ = ccd_saved;
        contact_ms_ = contact_saved;
        pd_solves_ = solves_saved;
        if (r != PDIPC_OK) return r;
        if (rl != PDIPC_OK) {
            err = e2;
            return rl;
        }
        PD_CK(cudaMemcpyAsync(stage_, adj_pb_, sizeof(V4<TC>) * ns, cudaMemcpyDeviceToHost, s_));
        PD_CK(cudaStreamSynchronize(s_));
        for (int i = 0; i < ns; ++i) {
            gx0[3 * (size_t)i] = (double)stage_[i].x;
            gx0[3 * (size_t)i + 1] = (double)stage_[i].y;
            gx0[3 * (size_t)i + 2] = (double)stage_[i].z;
        }
        PD_CK(cudaMemcpyAsync(stage_, adj_vb_, sizeof(V4<TC>) * ns, cudaMemcpyDeviceToHost, s_));
        PD_CK(cudaStreamSynchronize(s_));
        for (int i = 0; i < ns; ++i) {
            gv0[3 * (size_t)i] = (double)stage_[i].x;
            gv0[3 * (size_t)i + 1] = (double)stage_[i].y;
            gv0[3 * (size_t)i + 2] = (double)stage_[i].z;
        }
        if (gk) {
            PD_CK(cudaMemcpyAsync(gk, adj_kb_, sizeof(T) * ns, cudaMemcpyDeviceToHost, s_));
            PD_CK(cudaStreamSynchronize(s_));
        }
        return PDIPC_OK;
    }

    // ---------------- allocation helpers ----------------
    // Initialisation and uploads are ordered on the context's stream (created
    // non-blocking, so the legacy default stream gives no ordering with it);
    // uploads come from pageable memory, staged before the call returns.
    template <typename X>
    cudaError_t alloc(X*& p, size_t n) {
        n = std::max<size_t>(n, 1);
        cudaError_t e = cudaMalloc(&p, sizeof(X) * n);
        if (e == cudaSuccess) {
            ptrs_.push_back({(void*)p, sizeof(X) * n});
            bytes_ += (int64_t)(sizeof(X) * n);
        }
        return e;
    }
    template <typename X>
    cudaError_t zeros(X*& p, size_t n) {
        cudaError_t e = alloc(p, n);
        if (e != cudaSuccess) return e;
        return cudaMemsetAsync(p, 0, sizeof(X) * std::max<size_t>(n, 1), s_);
    }
    template <typename X>
    cudaError_t up(X*& p, const std::vector<X>& v) {
        cudaError_t e = alloc(p, v.size());
        if (e != cudaSuccess || v.empty()) return e;
        return cudaMemcpyAsync(p, v.data(), sizeof(X) * v.size(), cudaMemcpyHostToDevice, s_);
    }
    template <typename X>
    void dfree(X*& p) {
        if (!p) return;
        for (size_t i = 0; i < ptrs_.size(); ++i)
            if (ptrs_[i].first == (void*)p) {
                bytes_ -= (int64_t)ptrs_[i].second;
                ptrs_.erase(ptrs_.begin() + i);
                break;
            }
        cudaFree(p);
        p = nullptr;
    }
    template <typename X>
    cudaError_t grow(X*& p, int64_t& cap, int64_t need) {
        if (need <= cap && p) return cudaSuccess;
        const int64_t nc = std::max<int64_t>(need + need / 4, 1024);
        dfree(p);
        cudaError_t e = alloc(p, (size_t)nc);
        cap = (e == cudaSuccess) ? nc : 0;
        return e;
    }
    static std::vector<T> conv(const std::vector<double>& v) {
        std::vector<T> o(v.size());
        for (size_t i = 0; i < v.size(); ++i) o[i] = (T)v[i];
        return o;
    }
    void release() {
        for (int p = 0; p < 2; ++p) {
            if (coll_exec_[p]) cudaGraphExecDestroy(coll_exec_[p]);
            if (coll_graph_[p]) cudaGraphDestroy(coll_graph_[p]);
            coll_exec_[p] = nullptr;
            coll_graph_[p] = nullptr;
        }
        if (graph_exec_) cudaGraphExecDestroy(graph_exec_);
        if (graph_) cudaGraphDestroy(graph_);
        graph_exec_ = nullptr;
        graph_ = nullptr;
        for (auto& pr : ptrs_) cudaFree(pr.first);
        ptrs_.clear();
        if (pin_) cudaFreeHost(pin_);
        if (stage_) cudaFreeHost(stage_);
        pin_ = nullptr;
        stage_ = nullptr;
        if (ev0_) cudaEventDestroy(ev0_);
        if (ev1_) cudaEventDestroy(ev1_);
        for (auto& ring : evo_)
            for (cudaEvent_t& e : ring) {
                if (e) cudaEventDestroy(e);
                e = nullptr;
            }
        ev0_ = ev1_ = nullptr;
        if (s_) cudaStreamDestroy(s_);
        s_ = nullptr;
    }

    // ---------------- persistent PD solve ----------------
    // Partition of the SELL slices over co-resident CTAs (one per SM), with the
    // matrix values in shared memory when they fit, and the argument block.
    // The launch plan of the persistent solve: the default configuration, or
    // `force` when given (disabled if that configuration does not fit).  May
    // run again (the autotuner): the previous plan's tables are freed first.
    pdipc_status plan_persistent(const HostTables& H, std::string& err, const PlanChoice* force = nullptr) {
        plan_ = PersistPlan();
        dfree(pNbr_);
        dfree(pCtaTetPtr_);
        dfree(pCtaTetIdx_);
        dfree(pBand_);
        dfree(pFlags_);
        dfree(pCtaSlice_);
        dfree(pCtaEntry_);
        dfree(pRowPat_);
        dfree(pRowPatLoc_);
        dfree(pCtaPat_);
        dfree(pPatLoc_);
        dfree(pBar_);
        dfree(pSOff_);
        dfree(pSLen_);
        dfree(pSCol_);
        dfree(pSVal_);
        groups_.clear();
        if (!std::is_same<T, float>::value || !prm_.persistent || c_.cheby >= kMaxCheby) return PDIPC_OK;
        Dev<T, TC>& d = d_;
        const int ns = d.nsim;
        int dev = 0, nsm = 0, smem_optin = 0, coop = 0;
        PD_CK(cudaGetDevice(&dev));
        PD_CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
        PD_CK(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
        PD_CK(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
        if (!coop || ns == 0) return PDIPC_OK;
        // the matrix in SELL-32 over slots (slot_of: in every 64-row window the
        // even rows, then the odd ones); columns stay rows, padding repeats a
        // row's last column with value 0 (so its columns stay in order: low
        // halo, own rows, high halo)
        const int nslot = (ns + 63) / 64 * 64, nsl = nslot / kSlice;
        std::vector<int> soff(nsl + 1, 0), slen(nsl, 0);
        auto row_len = [&](int r) { return r < ns ? H.nPtr[r + 1] - H.nPtr[r] : 0; };
        for (int sl = 0; sl < nsl; ++sl) {
            for (int lane = 0; lane < kSlice; ++lane) slen[sl] = std::max(slen[sl], row_len(row_of(sl * kSlice + lane)));
            soff[sl + 1] = soff[sl] + kSlice * slen[sl];
        }
        {
            std::vector<int> pcol((size_t)std::max(soff[nsl], 1), 0);
            std::vector<T> pval((size_t)std::max(soff[nsl], 1), T(0));
            for (int sl = 0; sl < nsl; ++sl)
                for (int lane = 0; lane < kSlice; ++lane) {
                    const int r = row_of(sl * kSlice + lane), len = row_len(r);
                    for (int k = 0; k < slen[sl]; ++k) {
                        const size_t at = (size_t)soff[sl] + (size_t)kSlice * k + lane;
                        const int e = r < ns ? H.nPtr[r] + std::min(k, std::max(len - 1, 0)) : 0;
                        pcol[at] = len > 0 ? H.nCol[e] : std::min(r, ns - 1);
                        pval[at] = k < len ? (T)H.nVal[e] : T(0);
                    }
                }
            PD_CK(up(pSOff_, soff));
            PD_CK(up(pSLen_, slen));
            PD_CK(up(pSCol_, pcol));
            PD_CK(up(pSVal_, pval));
        }
        // distinct column-offset patterns of the rows
        int patW = 0;
        for (int w : slen) patW = std::max(patW, w);
        std::map<std::vector<int16_t>, int> pats;
        std::vector<int> rowPat(ns, 0);
        bool fits16 = true;
        for (int i = 0; i < ns && fits16; ++i) {
            std::vector<int16_t> o(patW, 0);
            for (int e = H.nPtr[i]; e < H.nPtr[i + 1]; ++e) {
                const int off = H.nCol[e] - i;
                if (off < -32768 || off > 32767) {
                    fits16 = false;
                    break;
                }
                o[e - H.nPtr[i]] = (int16_t)off;
            }
            // padding (value 0) repeats the last column, so a row's columns stay
            // in order: low halo, own rows, high halo
            const int len = H.nPtr[i + 1] - H.nPtr[i];
            for (int k = len; k < patW && len > 0; ++k) o[k] = o[len - 1];
            auto it = pats.emplace(o, (int)pats.size()).first;
            rowPat[i] = it->second;
            if (pats.size() > (size_t)1 << 20) fits16 = false;
        }
        auto a16 = [](size_t b) { return (b + 15) / 16 * 16; };
        // Each CTA's own pattern table (the patterns of its rows, in order of
        // first use): ctaPat[c] .. ctaPat[c + 1] of the concatenated tables,
        // and every row's id in its CTA's table.  A batch of many mesh sizes
        // has thousands of patterns, a CTA's rows a few dozen.
        auto local_pats = [&](int spc, std::vector<int>& ctaPat, std::vector<int16_t>* table,
                              std::vector<int>* rowLoc) {
            const int ctas = (nsl + spc - 1) / spc;
            ctaPat.assign(ctas + 1, 0);
            std::vector<int> stamp(pats.size(), -1), loc(pats.size(), 0);
            std::vector<const std::vector<int16_t>*> byId(table ? pats.size() : 0, nullptr);
            if (table) {
                for (auto& kv : pats) byId[kv.second] = &kv.first;
                table->clear();
            }
            if (rowLoc) rowLoc->assign(ns, 0);
            for (int c = 0; c < ctas; ++c) {
                int n = 0;
                for (int r = c * spc * kSlice; r < std::min(ns, (c + 1) * spc * kSlice); ++r) {
                    const int p = rowPat[r];
                    if (stamp[p] != c) {
                        stamp[p] = c;
                        loc[p] = n++;
                        if (table) table->insert(table->end(), byId[p]->begin(), byId[p]->end());
                    }
                    if (rowLoc) (*rowLoc)[r] = loc[p];
                }
                ctaPat[c + 1] = ctaPat[c] + n;
            }
        };
        // matrix values + the CTA's pattern table (unless the band path reads
        // the whole table from parameter space) + the band
        auto cta_smem = [&](int spc, bool smem_mat, size_t band_bytes, bool param_pats) -> size_t {
            if (!smem_mat) return 0;
            std::vector<int> cp;
            if (!param_pats) local_pats(spc, cp, nullptr, nullptr);
            size_t mx = 0;
            for (int c = 0; c * spc < nsl; ++c) {
                const int s0 = c * spc, s1 = std::min(nsl, s0 + spc);
                const size_t E = (size_t)(soff[s1] - soff[s0]);
                const size_t pb = param_pats ? 0 : a16((size_t)(cp[c + 1] - cp[c]) * patW * sizeof(int16_t));
                mx = std::max(mx, a16(E * sizeof(T)) + pb + band_bytes);
            }
            return mx;
        };
        // columns each CTA's matrix rows read, as a range: the band of the
        // iterate a CTA keeps in shared memory; returns the largest halo (the
        // columns outside the CTA's own rows)
        auto col_ranges = [&](int spc, std::vector<int2>& rg) -> int {
            const int ctas = (nsl + spc - 1) / spc;
            rg.assign(ctas, make_int2(0, 0));
            int mx = 0;
            for (int c = 0; c < ctas; ++c) {
                // own slots [r0, r1): the rows of whole 64-row windows
                const int r0 = c * spc * kSlice, r1 = std::min(nslot, (c + 1) * spc * kSlice);
                int lo = r0, hi = r1 - 1;
                for (int r = r0; r < std::min(ns, r1); ++r)
                    for (int e = H.nPtr[r]; e < H.nPtr[r + 1]; ++e) {
                        lo = std::min(lo, H.nCol[e]);
                        hi = std::max(hi, H.nCol[e]);
                    }
                lo &= ~63;                                    // whole windows of slots
                const int hs = std::min(nslot, (hi + 64) & ~63);
                rg[c] = make_int2(lo, hs);
                mx = std::max(mx, (r0 - lo) + (hs - r1));
            }
            return mx;
        };
        const size_t limit = (size_t)smem_optin - 1024;
        // Every configuration that fits: rows per thread R (slices per warp),
        // the band of the iterate in shared memory (correction form: own rows
        // and halo as three planar float arrays, the copies' mbarrier, one more warp
        // without rows for the neighbour flags and the copies), L1 or L2-only
        // gathers, neighbour waits or grid barriers.  The direct form keeps the
        // reference's summation order (gathers, no band).  The default is the
        // first R that fits, with the band when it fits, and the gathers and
        // synchronisation `persistent` names; with persistent = 1 the others
        // are listed in plan_choices_ for the autotuner.
        struct Cand {
            PlanChoice ch;
            bool smem_mat;
            int spc, ctas, threads;
            size_t sm;
            int ownMax, haloMax;
            std::vector<int2> band;
            std::vector<PersistGroup> groups;
            bool band_param = true;  // band path: the whole pattern table in parameter space
        };
        // Launch groups.  A plan whose CTAs are not all co-resident (or more
        // than params.pd_group_ctas) runs as several launches, each over whole
        // instances (runs of rows of one simulated model, which share no
        // matrix entry or stencil with other models): group g holds the
        // instances whose rows lie in at most maxc consecutive CTAs.  False
        // when one instance needs more CTAs than a launch holds.
        std::vector<int> instEnd;  // end row of every instance, ascending
        for (int i = 1; i <= ns; ++i)
            if (i == ns || H.vertexModel[i] != H.vertexModel[i - 1]) instEnd.push_back(i);
        auto form_groups = [&](int spc, int ctas, int maxc, std::vector<PersistGroup>& out) -> bool {
            out.clear();
            if (ctas <= maxc) {
                out.push_back(PersistGroup{0, ctas - 1, 0, ns});
                return true;
            }
            if (H.ntet > 0) return false;  // tets: one launch (a CTA projects tets of its own rows only)
            const int rpc = spc * kSlice;  // rows of a CTA
            size_t k = 0;
            for (int g0 = 0; g0 < ns;) {
                int end = g0;
                while (k < instEnd.size() && (instEnd[k] - 1) / rpc - g0 / rpc + 1 <= maxc) end = instEnd[k++];
                if (end == g0) return false;
                out.push_back(PersistGroup{g0 / rpc, (end - 1) / rpc, g0, end});
                g0 = end;
            }
            return true;
        };
        const int group_cap = prm_.pd_group_ctas > 0 ? prm_.pd_group_ctas : INT_MAX;
        std::vector<Cand> cands;
        const bool dflt_l1 = prm_.persistent != 2, dflt_ls = prm_.persistent != 3;
        for (int pass = 0; pass < 2; ++pass) {
            const bool smem_mat = pass == 0 && fits16;
            if (pass == 0 && !fits16) continue;
            if (pass == 1 && !cands.empty()) break;  // the L2-streamed matrix only when no slice fits
            for (int R = 1; R <= 4; ++R) {
                int W = std::max(1, (nsl + nsm * R - 1) / (nsm * R));
                if ((W * R) & 1) ++W;  // CTAs own whole windows (pairs of slices)
                if (W > kMaxPersistWarps) {
                    // more rows than one launch holds: the widest CTAs that
                    // leave a warp for the band path, in launch groups
                    if (H.ntet > 0 || instEnd.size() < 2) continue;
                    W = kMaxPersistWarps - 1;
                    if ((W * R) & 1) --W;
                }
                const int spc = W * R;
                const int ctas = (nsl + spc - 1) / spc;
                const size_t sm0 = cta_smem(spc, smem_mat, 0, false);
                if (sm0 > limit) continue;
                std::vector<Cand> vs;
                if (kCorrection && smem_mat && prm_.persistent == 1 && W + 1 <= kMaxPersistWarps) {
                    // the whole pattern table in parameter space when it fits
                    // (uniform offsets read through the constant cache), else
                    // each CTA's own table in shared memory
                    const bool param = pats.size() * (size_t)patW <= (size_t)kParamPatterns;
                    std::vector<int2> rg;
                    const int hx = col_ranges(spc, rg);
                    const int om = spc * kSlice;
                    const size_t smb = cta_smem(spc, smem_mat, a16(3 * (size_t)(om + hx) * sizeof(T)) + 16, param);
                    if (smb <= limit)
                        vs.push_back(Cand{PlanChoice{R, true, true, true}, smem_mat, spc, ctas, (W + 1) * 32, smb, om,
                                          hx, std::move(rg), {}, param});
                }
                for (int v = 0; v < 4 && (v == 0 || prm_.persistent == 1); ++v) {
                    const bool l1 = (v & 1) ? !dflt_l1 : dflt_l1, ls = (v & 2) ? !dflt_ls : dflt_ls;
                    vs.push_back(Cand{PlanChoice{R, false, l1, ls}, smem_mat, spc, ctas, W * 32, sm0, 0, 0, {}});
                }
                for (Cand& c : vs) {
                    const void* f =
                        persistent_kernel(kCorrection, smem_mat, c.ch.band, c.band_param, c.ch.l1_gather, R, H.ntet > 0);
                    if (!f) continue;
                    PD_CK(cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)std::max<size_t>(c.sm, 1)));
                    int per_sm = 0;
                    PD_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, f, c.threads, c.sm));
                    if (per_sm < 1 || !form_groups(c.spc, c.ctas, std::min(per_sm * nsm, group_cap), c.groups)) continue;
                    cands.push_back(std::move(c));
                }
            }
        }
        if (!force) {
            plan_choices_.clear();
            for (const Cand& c : cands) plan_choices_.push_back(c.ch);
        }
        const Cand* pick = nullptr;
        for (const Cand& c : cands) {
            const bool match = force ? (c.ch.rows_per_thread == force->rows_per_thread && c.ch.band == force->band &&
                                        c.ch.l1_gather == force->l1_gather && c.ch.local_sync == force->local_sync)
                                     : (c.ch.l1_gather == dflt_l1 && c.ch.local_sync == dflt_ls);
            if (match) {
                pick = &c;
                break;
            }
        }
        if (!pick) return PDIPC_OK;
        plan_.enabled = true;
        plan_.matrix_in_smem = pick->smem_mat;
        plan_.l1_gather = pick->ch.l1_gather;
        plan_.local_sync = pick->ch.local_sync;
        plan_.ctas = pick->ctas;
        plan_.threads = pick->threads;
        plan_.rows_per_thread = pick->ch.rows_per_thread;
        plan_.slices_per_cta = pick->spc;
        plan_.smem_bytes = pick->sm;
        plan_.patterns = pick->smem_mat ? (int)pats.size() : 0;
        plan_.pattern_width = patW;
        plan_.own_max = pick->ownMax;
        plan_.halo_max = pick->haloMax;
        groups_ = pick->groups;
        plan_.band_param = pick->band_param;
        const std::vector<int2> bandRange = pick->band;
        std::vector<int> ctaSlice(plan_.ctas + 1), ctaEntry(plan_.ctas + 1);
        for (int c = 0; c <= plan_.ctas; ++c) {
            ctaSlice[c] = std::min(nsl, c * plan_.slices_per_cta);
            ctaEntry[c] = soff[ctaSlice[c]];
        }
        std::vector<int16_t> patOff(std::max<size_t>(1, pats.size() * (size_t)patW), 0);
        for (auto& kv : pats) std::copy(kv.first.begin(), kv.first.end(), patOff.begin() + (size_t)kv.second * patW);
        // CTAs each CTA exchanges rows with: the CTAs owning the columns of its
        // matrix rows and stencils, closed under "is read by", as one range
        // (a CTA's slots are the rows of whole windows: the same range of rows)
        std::vector<int> ctaOfRow(ns, 0);
        for (int c = 0; c < plan_.ctas; ++c)
            for (int r = ctaSlice[c] * kSlice; r < std::min(ns, ctaSlice[c + 1] * kSlice); ++r) ctaOfRow[r] = c;
        std::vector<int2> rng(plan_.ctas);
        for (int c = 0; c < plan_.ctas; ++c) {
            int lo = c, hi = c;
            for (int r = ctaSlice[c] * kSlice; r < std::min(ns, ctaSlice[c + 1] * kSlice); ++r) {
                for (int e = H.nPtr[r]; e < H.nPtr[r + 1]; ++e) {
                    lo = std::min(lo, ctaOfRow[H.nCol[e]]);
                    hi = std::max(hi, ctaOfRow[H.nCol[e]]);
                }
                for (int e = H.lPtr[r]; e < H.lPtr[r + 1]; ++e) {
                    lo = std::min(lo, ctaOfRow[H.lNbr[e]]);
                    hi = std::max(hi, ctaOfRow[H.lNbr[e]]);
                }
            }
            rng[c] = make_int2(lo, hi);
        }
        // tets: the CTA owning a tet's first vertex projects it (curvature phase);
        // it reads the tet's vertex positions and the CTAs owning them read its
        // projection (residual phase)
        std::vector<int> ctaTetPtr(plan_.ctas + 1, 0), ctaTetIdx(std::max(1, H.ntet), 0);
        if (H.ntet > 0) {
            std::vector<int> owner(H.ntet);
            for (int e = 0; e < H.ntet; ++e) {
                const int c = ctaOfRow[H.tets[4 * (size_t)e]];
                owner[e] = c;
                ++ctaTetPtr[c + 1];
                for (int k = 0; k < 4; ++k) {
                    if (H.tets[4 * (size_t)e + k] < 0) continue;  // a triangle element has three vertices
                    const int c2 = ctaOfRow[H.tets[4 * (size_t)e + k]];
                    rng[c].x = std::min(rng[c].x, c2);
                    rng[c].y = std::max(rng[c].y, c2);
                    rng[c2].x = std::min(rng[c2].x, c);
                    rng[c2].y = std::max(rng[c2].y, c);
                }
            }
            for (int c = 0; c < plan_.ctas; ++c) ctaTetPtr[c + 1] += ctaTetPtr[c];
            std::vector<int> fill(ctaTetPtr.begin(), ctaTetPtr.end() - 1);
            for (int e = 0; e < H.ntet; ++e) ctaTetIdx[fill[owner[e]]++] = e;
        }
        std::vector<int2> nbr = rng;
        for (int c = 0; c < plan_.ctas; ++c)
            for (int d2 = rng[c].x; d2 <= rng[c].y; ++d2) {
                nbr[d2].x = std::min(nbr[d2].x, c);
                nbr[d2].y = std::max(nbr[d2].y, c);
            }
        // An irregular numbering (a tet mesh from a mesher) can make a CTA's
        // neighbour range span most of the grid: every phase then waits on most
        // CTAs, and the per-sweep launches measured faster (the reference's
        // ClothArmadillo example: 54.9 against 50.1 steps/s with grid barriers).
        int widest = 0;
        for (const int2& r : nbr) widest = std::max(widest, r.y - r.x + 1);
        if (widest > 32 && plan_.own_max == 0 && prm_.persistent == 1) {
            plan_ = PersistPlan();
            return PDIPC_OK;
        }
        PD_CK(up(pNbr_, nbr));
        PD_CK(up(pCtaTetPtr_, ctaTetPtr));
        PD_CK(up(pCtaTetIdx_, ctaTetIdx));
        if (plan_.own_max > 0) PD_CK(up(pBand_, bandRange));
        PD_CK(zeros(pFlags_, plan_.ctas));
        PD_CK(up(pCtaSlice_, ctaSlice));
        PD_CK(up(pCtaEntry_, ctaEntry));
        PD_CK(up(pRowPat_, rowPat));
        {
            std::vector<int> ctaPat, rowLoc;
            std::vector<int16_t> table;
            local_pats(plan_.slices_per_cta, ctaPat, &table, &rowLoc);
            if (table.empty()) table.push_back(0);
            PD_CK(up(pRowPatLoc_, rowLoc));
            PD_CK(up(pCtaPat_, ctaPat));
            PD_CK(up(pPatLoc_, table));
        }
        PD_CK(zeros(pBar_, 2));
        if constexpr (std::is_same<T, float>::value) {
            PersistArgs<float, TC>& a = pargs_;
            a.nsim = ns;
            a.nslot = nslot;
            a.lg = c_.lg;
            a.cheby = c_.cheby;
            a.relax = (T)c_.relax;
            T rho2 = (T)c_.rho;
            rho2 = rho2 * rho2;
            T om = omega_first(rho2);
            for (int it = 0; it < kMaxCheby; ++it) a.omega[it] = T(0);
            for (int it = 1; it < c_.cheby; ++it) {
                a.omega[it] = om;
                om = omega_next(rho2, om);
            }
            a.timeout = wait_cycles_;
            a.P = d.P;
            a.Ph = d.Ph;
            a.Pl = d.Pl;
            a.Pold = d.Pold;
            a.Xrest = d.Xrest;
            a.Rhs0 = d.Rhs0;
            a.CollRhs = d.CollRhs;
            a.PinRhs = d.PinRhs;
            a.Aq = d.Aq;
            a.GX = d.B;
            a.GX2 = d.C;
            a.GY = d.Y;
            a.Delastic = d.Delastic;
            a.Dinert = d.Dinert;
            a.CollDiag = d.CollDiag;
            a.PinFlag = d.PinFlag;
            a.PinK = d.PinK;
            a.lPtr = d.lPtr;
            a.tOff = d.tOff;
            a.tNbr = d.tNbr;
            a.tRest = d.tRest;
            a.tLbo = d.tLbo;
            a.tBendT = d.tBendT;
            a.tBend0 = d.tBend0;
            a.tLbo0 = d.tLbo0;
            a.Strain = d.Strain;
            a.CurvNorm = d.CurvNorm;
            a.ntet = d.ntet;
            a.Tets = d.Tets;
            a.TetIdm = d.TetIdm;
            a.TetW = d.TetW;
            a.TetOut = d.TetOut;
            a.vtPtr = d.vtPtr;
            a.vtIdx = d.vtIdx;
            a.ctaTetPtr = pCtaTetPtr_;
            a.ctaTetIdx = pCtaTetIdx_;
            a.sliceEntry = pSOff_;
            a.sliceLen = pSLen_;
            a.sCol = pSCol_;
            a.sVal = pSVal_;
            a.ctaSlice = pCtaSlice_;
            a.ctaEntry = pCtaEntry_;
            a.rowPattern = pRowPat_;
            a.rowPatLocal = pRowPatLoc_;
            a.ctaPat = pCtaPat_;
            a.patLocal = pPatLoc_;
            std::fill(a.patc, a.patc + kParamPatterns, (int16_t)0);
            if (plan_.own_max > 0 && plan_.band_param) std::copy(patOff.begin(), patOff.end(), a.patc);
            a.patW = patW;
            a.bar = pBar_;
            a.err = d.ErrFlags;
            a.flags = pFlags_;
            a.nbr = plan_.local_sync ? pNbr_ : nullptr;
            a.band = plan_.own_max > 0 ? pBand_ : nullptr;
            a.ownMax = plan_.own_max;
            a.haloMax = plan_.halo_max;
            a.epoch0 = 0;
            a.nphases = (unsigned)(c_.lg * (2 * c_.cheby + 1) + 1);
            a.ctaLo = 0;
            a.ctaHi = plan_.ctas - 1;
            a.row0 = 0;
            a.row1 = ns;
            a.vInst = prm_.instance_stop ? d.VInst : nullptr;
            a.instStop = prm_.instance_stop ? d.InstStop : nullptr;
            if (prm_.instance_stop && (!a.vInst || !a.instStop)) {
                plan_.enabled = false;
                err = "persistent solve: unallocated instance table";
                return PDIPC_ERR_STATE;
            }
            const void* ptrs[] = {a.P, a.Pold, a.Xrest, a.Rhs0, a.CollRhs, a.PinRhs, a.Aq, a.GX, a.GX2, a.GY, a.Delastic,
                                  a.Dinert, a.CollDiag, a.PinFlag, a.PinK, a.lPtr, a.tOff, a.tNbr, a.tRest,
                                  a.tLbo, a.tBendT, a.tBend0, a.tLbo0, a.Strain, a.CurvNorm, a.sliceEntry, a.sliceLen, a.sCol,
                                  a.sVal, a.ctaSlice, a.ctaEntry, a.rowPattern, a.rowPatLocal, a.ctaPat, a.patLocal,
                                  a.bar, a.err};
            if (a.ntet > 0 && (!a.Tets || !a.TetIdm || !a.TetW || !a.TetOut || !a.vtPtr || !a.vtIdx)) {
                plan_.enabled = false;
                err = "persistent solve: unallocated tet table";
                return PDIPC_ERR_STATE;
            }
            if (kCorrection && (!a.Ph || !a.Pl)) {
                plan_.enabled = false;
                err = "persistent solve: unallocated position mirror";
                return PDIPC_ERR_STATE;
            }
            for (const void* q : ptrs)
                if (!q) {
                    plan_.enabled = false;
                    err = "persistent solve: unallocated buffer";
                    return PDIPC_ERR_STATE;
                }
        }
        return PDIPC_OK;
    }

    // one PD solve: a launch per group, in order on the stream; returns the launches made
    cudaError_t launch_persistent(int* launched = nullptr) {
        if constexpr (std::is_same<T, float>::value) {
            pargs_.gate = d_.Gate;
            for (const PersistGroup& g : groups_) {
                // fresh phase numbers for this launch: every flag from earlier launches is below them
                pargs_.epoch0 = epoch_;
                epoch_ += pargs_.nphases;
                pargs_.ctaLo = g.cta_lo;
                pargs_.ctaHi = g.cta_hi;
                pargs_.row0 = g.row0;
                pargs_.row1 = g.row1;
                const cudaError_t e = launch_pd_persistent(plan_, pargs_, s_);
                if (e != cudaSuccess) return e;
                if (launched) ++*launched;
            }
            return cudaSuccess;
        }
        return cudaErrorNotSupported;
    }

    // ---------------- patch tree ----------------
    pdipc_status build_tree(bool from_rest, std::string& err) {
        Dev<T, TC>& d = d_;
        if (d.npatch == 0) return PDIPC_OK;
        const T infl = (T)c_.infl;
        if (from_rest) {
            launch_patch_init_boxes(d, infl, s_);
            ++launches_;
        }
        T* cs = nullptr;
        unsigned long long* keys = nullptr;
        int* vals = nullptr;
        void* tmp = nullptr;
        PD_CK(cudaMalloc(&cs, sizeof(T) * 4));
        PD_CK(cudaMalloc(&keys, sizeof(unsigned long long) * d.npatch));
        PD_CK(cudaMalloc(&vals, sizeof(int) * d.npatch));
        PD_CK(cudaMalloc(&tmp, sort_tmp_bytes(d.npatch)));
        launch_morton(d, cs, keys, vals, s_);
        radix_sort_u64(keys, vals, d.npatch, tmp, d.ErrFlags, s_);
        PD_CK(cudaMemcpyAsync(d.LeafPatch, vals, sizeof(int) * d.npatch, cudaMemcpyDeviceToDevice, s_));
        launch_karras(d, keys, s_);
        launches_ += 3 + 2 + 8 + 1;
        pin_->err = 0;
        PD_CK(cudaMemcpyAsync(&pin_->err, d.ErrFlags, sizeof(unsigned int), cudaMemcpyDeviceToHost, s_));
        PD_CK(cudaStreamSynchronize(s_));
        cudaFree(cs);
        cudaFree(keys);
        cudaFree(vals);
        cudaFree(tmp);
        PD_CK(cudaGetLastError());
        if (pin_->err & kErrSort) {
            PD_CK(cudaMemsetAsync(d.ErrFlags, 0, sizeof(unsigned int), s_));
            err = "patch tree: a look-back wait of the radix sort timed out";
            return PDIPC_ERR_CUDA;
        }
        return PDIPC_OK;
    }

    pdipc_status ensure_scan_tmp(int64_t n, std::string& err) {
        const int64_t need = (int64_t)scan_tmp_bytes(n);
        if (need <= scan_tmp_cap_ && scan_tmp_) return PDIPC_OK;
        if (scan_tmp_) dfree(scan_tmp_);
        scan_tmp_cap_ = need * 2;
        PD_CK(alloc(scan_tmp_, (size_t)scan_tmp_cap_));
        return PDIPC_OK;
    }

    // gpuCcdCulling (cpp:1799-1869) from Pold and Dir.
    pdipc_status broadphase(std::string& err) {
        Dev<T, TC>& d = d_;
        d.nPairs = d.nPT = d.nEE = 0;
        if (d.npatch == 0) return PDIPC_OK;
        const T infl = (T)c_.infl;
        launch_patch_boxes(d, d.Pold, d.Dir, (const V4<T>*)d.Poh, (const V4<T>*)d.Dh, infl, s_);
        ++launches_;
        if (prm_.rebuild_bvh) {
            pdipc_status r = build_tree(false, err);
            if (r != PDIPC_OK) return r;
        }
        launch_refit(d, s_);
        ++launches_;
        // One traversal writes the pairs and their record counts; the counts
        // are scanned over the whole buffer (entries past the pairs found stay
        // zero), so one read gives the pair and record totals.  When the pairs
        // overflow the buffer it grows and the traversal runs again.
        if (d.capPairs < 1) PD_CK(grow(d.Pairs, d.capPairs, 8 * (int64_t)d.npatch));
        for (;;) {
            if (!cpt_ || cptCap_ != d.capPairs) {
                if (cpt_) { dfree(cpt_); dfree(cee_); dfree(opt_); dfree(oee_); }
                int64_t c1 = 0, c2 = 0, c3 = 0, c4 = 0;
                PD_CK(grow(cpt_, c1, d.capPairs));
                PD_CK(grow(cee_, c2, d.capPairs));
                PD_CK(grow(opt_, c3, d.capPairs + 1));
                PD_CK(grow(oee_, c4, d.capPairs + 1));
                cptCap_ = d.capPairs;
            }
            pdipc_status r = ensure_scan_tmp(d.capPairs + 1, err);
            if (r != PDIPC_OK) return r;
            PD_CK(cudaMemsetAsync(d.PairCount, 0, sizeof(unsigned long long), s_));
            PD_CK(cudaMemsetAsync(cpt_, 0, sizeof(int64_t) * d.capPairs, s_));
            PD_CK(cudaMemsetAsync(cee_, 0, sizeof(int64_t) * d.capPairs, s_));
            launch_traverse(d, cpt_, cee_, d.capPairs, d.PairCount, c_, s_);
            scan_exclusive_i64(cpt_, opt_, d.capPairs, opt_ + d.capPairs, scan_tmp_, s_);
            scan_exclusive_i64(cee_, oee_, d.capPairs, oee_ + d.capPairs, scan_tmp_, s_);
            launches_ += 5;
            PD_CK(cudaMemcpyAsync(&pin_->n_pairs, d.PairCount, sizeof(int64_t), cudaMemcpyDeviceToHost, s_));
            PD_CK(cudaMemcpyAsync(&pin_->n_pt, opt_ + d.capPairs, sizeof(int64_t), cudaMemcpyDeviceToHost, s_));
            PD_CK(cudaMemcpyAsync(&pin_->n_ee, oee_ + d.capPairs, sizeof(int64_t), cudaMemcpyDeviceToHost, s_));
            PD_CK(cudaStreamSynchronize(s_));
            d.nPairs = pin_->n_pairs;
            if (d.nPairs <= d.capPairs) break;
            PD_CK(grow(d.Pairs, d.capPairs, d.nPairs + d.nPairs / 4));
        }
        if (d.nPairs == 0) return PDIPC_OK;
        d.nPT = pin_->n_pt;
        d.nEE = pin_->n_ee;
        PD_CK(grow(d.PT, d.capPT, d.nPT));
        PD_CK(grow(d.EE, d.capEE, d.nEE));
        launch_expand(d, opt_, oee_, c_, s_);
        ++launches_;
        st_.patch_pairs = d.nPairs;
        st_.pt_candidates = d.nPT;
        st_.ee_candidates = d.nEE;
        PD_CK(cudaGetLastError());
        return PDIPC_OK;
    }

    // ---------------- projective dynamics ----------------
    // One outer iteration's solve: diagonal, then lg x (local step + Chebyshev
    // accelerated Jacobi).  R2 x + c is evaluated as two weighted-Jacobi sweeps
    // S(S(x)); the iterates rotate through P and B, the last lands in P.
    static constexpr bool kCorrection = sizeof(T) == 4 && sizeof(TC) == 8;

    // Correction (mixed-precision) form: the same Chebyshev-accelerated Jacobi
    // iteration on delta = x - x_start from delta_0 = 0, with the residual of
    // x_start as right-hand side; the iterates rotate through B and C and the
    // last one is added to P.
    int enqueue_pd_correction() {
        Dev<T, TC>& d = d_;
        const T w = (T)c_.relax;
        T rho2 = (T)c_.rho;
        rho2 = rho2 * rho2;
        int k = 0;
        launch_diag(d, s_);
        ++k;
        for (int lg = 0; lg < c_.lg; ++lg) {
            launch_local_aq(d, s_);
            launch_tet_project(d, s_);
            k += d.ntet > 0;
            launch_local_residual(d, w, s_);
            launch_sweep_delta<T, TC>(d, c_.cheby == 1 ? 4 : 0, d.Y, nullptr, d.B, w, T(0), s_);
            k += 3;
            T om = omega_first(rho2);
            for (int it = 1; it < c_.cheby; ++it) {
                V4<T>* cur = (it & 1) ? d.B : d.C;
                V4<T>* prv = (it & 1) ? d.C : d.B;
                const bool last = it == c_.cheby - 1;
                const int mode = 1 | (it == 1 ? 2 : 0) | (last ? 4 : 0);
                launch_sweep_delta<T, TC>(d, 0, cur, nullptr, d.Y, w, T(0), s_);
                launch_sweep_delta<T, TC>(d, mode, d.Y, prv, prv, w, om, s_);  // mode 4: into P
                k += 2;
                om = omega_next(rho2, om);
            }
        }
        return k;
    }

    int enqueue_pd() {
        if constexpr (kCorrection) {
            return enqueue_pd_correction();
        } else {
        Dev<T, TC>& d = d_;
        const T w = (T)c_.relax;
        T rho2 = (T)c_.rho;
        rho2 = rho2 * rho2;
        int k = 0;
        launch_diag(d, s_);
        ++k;
        for (int lg = 0; lg < c_.lg; ++lg) {
            if (taping_) {  // positions at the start of every local-global iteration
                if (adj_tape_n_ < adj_tape_cap_)
                    cudaMemcpyAsync(adj_tape_ + (size_t)adj_tape_n_ * d.nsim, d.P, sizeof(V4<TC>) * d.nsim,
                                    cudaMemcpyDeviceToDevice, s_);
                ++adj_tape_n_;
            }
            launch_local_aq(d, s_);
            launch_tet_project(d, s_);
            k += d.ntet > 0;
            launch_local_rhs_sweep(d, w, s_);
            launch_sweep<T, TC>(d, d.Y, nullptr, c_.cheby == 1 ? d.P : d.B, w, T(0), s_);
            k += 3;
            T om = omega_first(rho2);
            for (int it = 1; it < c_.cheby; ++it) {
                V4<T>* cur = (it & 1) ? d.B : d.P;
                V4<T>* prv = (it & 1) ? d.P : d.B;
                V4<T>* out = (it == c_.cheby - 1) ? d.P : prv;
                launch_sweep<T, TC>(d, cur, nullptr, d.Y, w, T(0), s_);
                launch_sweep<T, TC>(d, d.Y, prv, out, w, om, s_);
                k += 2;
                om = omega_next(rho2, om);
            }
        }
        return k;
        }
    }

    pdipc_status pd_solve(std::string& err) {
        if (plan_.enabled) {
            int n = 0;
            PD_CK(launch_persistent(&n));
            launches_ += n;
            return PDIPC_OK;
        }
        if (!prm_.use_graphs || taping_) {
            launches_ += enqueue_pd();
            return PDIPC_OK;
        }
        if (!graph_exec_) {
            PD_CK(cudaStreamBeginCapture(s_, cudaStreamCaptureModeThreadLocal));
            graph_nodes_ = enqueue_pd();
            PD_CK(cudaStreamEndCapture(s_, &graph_));
            PD_CK(cudaGraphInstantiate(&graph_exec_, graph_, 0));
        }
        PD_CK(cudaGraphLaunch(graph_exec_, s_));
        launches_ += graph_nodes_;
        return PDIPC_OK;
    }

    // One outer iteration of the step, enqueued without waiting: PD solve,
    // direction, the broad phase (first iteration only), toi pass, clamp,
    // contact pass, the stopping test on the device with its 16-byte record
    // copied to pinned memory, then the copy of the positions into Pold,
    // which the test skips when it stops the loop.
    pdipc_status enqueue_outer(int outer, std::string& err) {
        Dev<T, TC>& d = d_;
        cudaEvent_t* ev = evo_[outer & 1];
        PD_CK(cudaEventRecord(ev[kEvP0], s_));
        pdipc_status r = pd_solve(err);
        if (r != PDIPC_OK) return r;
        PD_CK(cudaEventRecord(ev[kEvP1], s_));
        if (outer > 0 && prm_.use_graphs) {
            // the collision pass as one graph launch (captured once per step,
            // after the first iteration's broad phase fixed the candidate lists)
            r = collision_graph(err);
            if (r != PDIPC_OK) return r;
            PD_CK(cudaGraphLaunch(coll_exec_[outer & 1], s_));
            launches_ += coll_nodes_;
            return PDIPC_OK;
        }
        launches_ += coll_head();
        if (outer == 0) {
            r = broadphase(err);
            if (r != PDIPC_OK) return r;
            if (d.ninst > 0) {  // per-candidate times of impact, reduced per instance
                PD_CK(grow(instPT_, instPTCap_, std::max<int64_t>(d.nPT, 1)));
                PD_CK(grow(instEE_, instEECap_, std::max<int64_t>(d.nEE, 1)));
            }
        }
        int n = 0;
        r = coll_tail(outer & 1, n, err);
        launches_ += n;
        return r;
    }

    // The collision pass of an outer iteration after its PD solve, in two
    // parts around the first iteration's broad phase.  Head: the direction
    // and its residual (per instance too).  Tail: toi pass, clamp, contact
    // pass, the stopping test on the device with its 16-byte record copied to
    // pinned memory (slot `parity`), then the copy of the positions into Pold,
    // which the test skips when it stops the loop.  Nothing in them depends on
    // the iteration's index beyond its parity (the test reads the index from
    // the device), so both can be captured in a graph.  Return the kernels
    // they launch.
    int coll_head() {
        launch_direction(d_, s_);
        if (d_.ninst > 0) launch_inst_resid(d_, s_);
        return 2 + (d_.ninst > 0);
    }
    pdipc_status coll_tail(int parity, int& n, std::string& err, bool capturing = false) {
        Dev<T, TC>& d = d_;
        cudaEvent_t* ev = evo_[parity];
        const bool inst = d.ninst > 0;
        // in a capture, an event record becomes a graph node only when external
        // (the host synchronises on these events after each launch)
        const unsigned rf = capturing ? cudaEventRecordExternal : cudaEventRecordDefault;
        PD_CK(cudaEventRecordWithFlags(ev[kEvC0], s_, rf));
        launch_toi(d, pos_old(), pos(), c_, inst ? instPT_ : (TC*)nullptr, inst ? instEE_ : (TC*)nullptr, s_);
        launch_toi_finalize(d, c_, s_);
        if (inst) launch_inst_toi(d, instPT_, instEE_, c_, s_);
        PD_CK(cudaEventRecordWithFlags(ev[kEvC1], s_, rf));
        launch_clamp(d, s_);
        PD_CK(cudaEventRecordWithFlags(ev[kEvQ0], s_, rf));
        launch_contact(d, pos(), c_, s_);
        PD_CK(cudaEventRecordWithFlags(ev[kEvQ1], s_, rf));
        if (inst)
            launch_inst_gate(d, prm_.outer_tol, prm_.fixed_outer <= 0, s_);
        else
            launch_outer_gate(d, prm_.outer_tol, prm_.fixed_outer <= 0, s_);
        PD_CK(cudaMemcpyAsync(&pin_->gate[parity], d.Gate, sizeof(OuterGate), cudaMemcpyDeviceToHost, s_));
        PD_CK(cudaEventRecordWithFlags(ev[kEvGate], s_, rf));
        launch_copy_old(d, s_);
        // toi x2 (+ cubic), finalize, clamp, contact clear, contact x2, gate, copy into Pold
        n = (1 + (c_.ccd_mode != 0)) * ((d.nPT > 0) + (d.nEE > 0)) + (d.nPT > 0) + (d.nEE > 0) + 5 +
            (inst ? 1 + (d.nPT > 0) + (d.nEE > 0) : 0);
        return PDIPC_OK;
    }
    // The collision pass (head and tail) captured as a graph per parity of the
    // outer iteration (the events and the pinned record slot alternate), again
    // whenever the candidate lists or the buffers they use changed since the
    // last capture.
    pdipc_status collision_graph(std::string& err) {
        const Dev<T, TC>& d = d_;
        const std::array<const void*, 6> sig{(const void*)d.PT, (const void*)d.EE, (const void*)instPT_,
                                             (const void*)instEE_, (const void*)(intptr_t)d.nPT,
                                             (const void*)(intptr_t)d.nEE};
        if (coll_exec_[0] && sig == coll_sig_) return PDIPC_OK;
        for (int p = 0; p < 2; ++p) {
            if (coll_exec_[p]) cudaGraphExecDestroy(coll_exec_[p]);
            if (coll_graph_[p]) cudaGraphDestroy(coll_graph_[p]);
            coll_exec_[p] = nullptr;
            coll_graph_[p] = nullptr;
            PD_CK(cudaStreamBeginCapture(s_, cudaStreamCaptureModeThreadLocal));
            int n = coll_head();
            int m = 0;
            pdipc_status r = coll_tail(p, m, err, true);
            cudaGraph_t g = nullptr;
            const cudaError_t ce = cudaStreamEndCapture(s_, &g);
            if (r != PDIPC_OK) {
                if (g) cudaGraphDestroy(g);
                return r;
            }
            PD_CK(ce);
            coll_graph_[p] = g;
            PD_CK(cudaGraphInstantiate(&coll_exec_[p], g, 0));
            coll_nodes_ = n + m;
        }
        coll_sig_ = sig;
        return PDIPC_OK;
    }

    // Sets the device stopping test for the kernels of one step; stage entry
    // points outside a step launch the same kernels without it.
    struct GateScope {
        Dev<T, TC>& d;
        GateScope(Dev<T, TC>& dev, OuterGate* g) : d(dev) { d.Gate = g; }
        ~GateScope() { d.Gate = nullptr; }
    };

    // PdIpcSimulator::advance (cpp:1683-1796): predict, then outer iterations
    // until |dir|^2 < outer_tol after the first one (or max_outer), then the
    // velocity update.  With the persistent solve, iteration k+1 is enqueued
    // before the host waits for iteration k's stopping test, so the GPU never
    // idles on the host's round trip; when the test stops the loop at k, every
    // kernel of iteration k+1 returns at entry.  The per-sweep solve (plain
    // launches or a CUDA graph of them) has no entry test, so that path waits
    // for each test before enqueueing the next iteration.
    pdipc_status step_once(std::string& err) {
        Dev<T, TC>& d = d_;
        const TC dt = (TC)c_.dt;
        GateScope scope(d_, gate_);
        PD_CK(cudaMemsetAsync(gate_, 0, sizeof(OuterGate), s_));
        if (d.ninst > 0) {
            PD_CK(cudaMemsetAsync(d.InstStop, 0, sizeof(unsigned) * d.ninst, s_));
            PD_CK(cudaMemsetAsync(d.InstIters, 0, sizeof(int) * d.ninst, s_));
        }
        launch_predict(d, dt, s_);
        ++launches_;
        const int max_outer = prm_.fixed_outer > 0 ? prm_.fixed_outer : prm_.max_outer;
        const int ahead = plan_.enabled ? 1 : 0;
        int enq = 0, outer = 0;
        for (; enq <= ahead && enq < max_outer; ++enq) {
            pdipc_status r = enqueue_outer(enq, err);
            if (r != PDIPC_OK) return r;
        }
        for (int k = 0; k < max_outer; ++k) {
            cudaEvent_t* ev = evo_[k & 1];
            PD_CK(cudaEventSynchronize(ev[kEvGate]));
            float pms = 0.f;
            PD_CK(cudaEventElapsedTime(&pms, ev[kEvP0], ev[kEvP1]));
            pd_ms_ += pms;
            PD_CK(cudaEventElapsedTime(&pms, ev[kEvC0], ev[kEvC1]));
            ccd_ms_ += pms;
            PD_CK(cudaEventElapsedTime(&pms, ev[kEvQ0], ev[kEvQ1]));
            contact_ms_ += pms;
            ++pd_solves_;
            const OuterGate g = pin_->gate[k & 1];
            if (g.iters != k + 1) {
                err = "outer-loop stopping test out of step with the host";
                return PDIPC_ERR_STATE;
            }
            st_.last_residual = g.resid;
            if (taping_ && (g.toi != 1.0 || g.active != 0)) adj_contact_ = true;
            outer = k + 1;
            if (g.stop) break;
            if (enq < max_outer) {
                pdipc_status r = enqueue_outer(enq, err);
                if (r != PDIPC_OK) return r;
                ++enq;
            }
        }
        const TC damping = (TC)(1.0 - (double)dt);
        const TC invt = (TC)((1.0 / (double)dt) * (double)damping);
        launch_velocity(d, invt, s_);
        ++launches_;
        PD_CK(cudaMemcpyAsync(&pin_->err, d.ErrFlags, sizeof(unsigned int), cudaMemcpyDeviceToHost, s_));
        PD_CK(cudaMemcpyAsync(&pin_->active, d.ActiveCount, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s_));
        TC toi;
        PD_CK(cudaMemcpyAsync(&toi, d.Toi, sizeof(TC), cudaMemcpyDeviceToHost, s_));
        if (d.ninst > 0) {
            // the instances' outer-iteration counts; outside a step no row is skipped
            PD_CK(cudaMemcpyAsync(instIters_.data(), d.InstIters, sizeof(int) * d.ninst, cudaMemcpyDeviceToHost, s_));
            PD_CK(cudaMemsetAsync(d.InstStop, 0, sizeof(unsigned) * d.ninst, s_));
        }
        PD_CK(cudaStreamSynchronize(s_));
        PD_CK(cudaGetLastError());
        for (int k = 0; k < d.ninst; ++k) inst_outer_ += instIters_[k];
        st_.last_toi = (double)toi;
        st_.active_contacts = (int64_t)pin_->active;
        st_.last_outer_iters = outer;
        st_.total_outer_iters += outer;
        st_.max_outer_iters = std::max(st_.max_outer_iters, outer);
        st_.steps_done++;
        if (pin_->err) {
            const unsigned int e = pin_->err;
            pin_->err = 0;
            cudaMemsetAsync(d.ErrFlags, 0, sizeof(unsigned int), s_);
            if (e & kErrBarrier) {
                cudaMemsetAsync(pBar_ + 1, 0, sizeof(unsigned), s_);
                err = "grid barrier of the persistent solve timed out";
                return PDIPC_ERR_CUDA;
            }
            if (e & kErrNonFinite) {
                err = "non-finite position after the step";
                return PDIPC_ERR_NONFINITE;
            }
            err = "broad-phase traversal ran past its node budget (malformed patch tree)";
            return PDIPC_ERR_OVERFLOW;
        }
        return PDIPC_OK;
    }

    Dev<T, TC> d_;
    pdipc_params prm_{};
    SolverConsts c_{};
    cudaStream_t s_ = nullptr;
    cudaEvent_t ev0_ = nullptr, ev1_ = nullptr;
    // per outer iteration (two in flight): around the PD solve, the toi pass
    // and the contact pass, and after the stopping test's copy to the host
    enum { kEvP0, kEvP1, kEvC0, kEvC1, kEvQ0, kEvQ1, kEvGate, kEvPerOuter };
    cudaEvent_t evo_[2][kEvPerOuter] = {};
    OuterGate* gate_ = nullptr;  // the device's stopping test of the outer loop
    double ccd_ms_ = 0.0, contact_ms_ = 0.0;
    double device_ms_ = 0.0;
    double pd_ms_ = 0.0, pd_bytes_ = 0.0, local_bytes_ = 0.0;
    int64_t pd_solves_ = 0;
    std::vector<std::pair<void*, size_t>> ptrs_;
    int64_t bytes_ = 0;
    int64_t launches_ = 0;
    int64_t sell_entries_ = 0, sell_padded_ = 0;
    V4<TC>* scratch_ = nullptr;
    // penalty stages: direction, force, velocity, hit counts, face pairs; per-vertex model index
    V4<TC>* pen_d_ = nullptr;
    V4<TC>* pen_f_ = nullptr;
    V4<TC>* pen_v_ = nullptr;
    int* pen_t_ = nullptr;
    int2* penPairs_ = nullptr;
    int64_t penPairCap_ = 0;
    int* vModel_ = nullptr;
    V4<T>* sh_ = nullptr;  // float-float mirror of scratch_ (correction form)
    V4<T>* sl_ = nullptr;
    int64_t cptCap_ = 0;  // pair capacity the record-count buffers below were sized for
    int64_t* cpt_ = nullptr;
    int64_t* cee_ = nullptr;
    int64_t* opt_ = nullptr;
    int64_t* oee_ = nullptr;
    char* scan_tmp_ = nullptr;
    int64_t scan_tmp_cap_ = 0;
    Pinned* pin_ = nullptr;
    // discrete adjoint: checkpoints, tape and work vectors (FP64 form)
    int adj_every_ = 0, adj_steps_ = 0;
    int clock_khz_ = 2000000;
    long long wait_cycles_ = 4000000000ll;
    std::vector<V4<TC>*> adj_ckpt_, adj_seg_;
    V4<TC>* adj_tape_ = nullptr;
    int adj_tape_cap_ = 0, adj_tape_n_ = 0;
    bool taping_ = false, adj_contact_ = false, adj_ready_ = false;
    T* adj_lboT_ = nullptr;
    T* adj_ntval_ = nullptr;
    T* adj_kb_ = nullptr;
    V4<TC>* adj_eb_ = nullptr;  // strain-limit elements' adjoints (4 per element)
    V4<TC>* adj_final_ = nullptr;
    V4<TC>*adj_pb_ = nullptr, *adj_vb_ = nullptr, *adj_r0b_ = nullptr, *adj_rb_ = nullptr, *adj_qb_ = nullptr,
           *adj_u_ = nullptr, *adj_rho_ = nullptr;
    std::vector<V4<TC>*> adj_xb_, adj_xs_, adj_ys_;
    PersistPlan plan_;
    std::vector<PlanChoice> plan_choices_;  // every persistent configuration that fits (default planning)
    pdipc_tuning tuning_{};
    PersistArgs<float, TC> pargs_{};
    std::vector<PersistGroup> groups_;  // launches of one persistent PD solve
    // the matrix in SELL-32 over slots (slot_of) for the persistent solve
    int* pSOff_ = nullptr;
    int* pSLen_ = nullptr;
    int* pSCol_ = nullptr;
    T* pSVal_ = nullptr;
    int* pCtaSlice_ = nullptr;
    int* pCtaEntry_ = nullptr;
    int* pRowPat_ = nullptr;
    int* pRowPatLoc_ = nullptr;  // persistent plan: every row's id in its CTA's pattern table
    int* pCtaPat_ = nullptr;
    int16_t* pPatLoc_ = nullptr;
    unsigned* pBar_ = nullptr;
    unsigned* pFlags_ = nullptr;  // per-CTA phase counts of the neighbour synchronisation
    int2* pNbr_ = nullptr;        // per-CTA range of CTAs to wait for
    int2* pBand_ = nullptr;       // per-CTA [first, last + 1) slot its rows read (band path)
    int* pCtaTetPtr_ = nullptr;   // per-CTA range of the tets it projects
    int* pCtaTetIdx_ = nullptr;
    unsigned epoch_ = 1;
    V4<TC>* stage_ = nullptr;  // pinned host staging of one state vector
    cudaGraph_t graph_ = nullptr;
    cudaGraphExec_t graph_exec_ = nullptr;
    int graph_nodes_ = 0;
    // the collision pass of outer iterations 1, 2, ... as a graph per parity
    cudaGraph_t coll_graph_[2] = {};
    cudaGraphExec_t coll_exec_[2] = {};
    std::array<const void*, 6> coll_sig_{};
    int coll_nodes_ = 0;
    bool inited_ = false;
    pdipc_stats st_{};
    // per-instance stopping: per-candidate times of impact and the instances' counts
    TC* instPT_ = nullptr;
    TC* instEE_ = nullptr;
    int64_t instPTCap_ = 0, instEECap_ = 0;
    std::vector<int> instIters_;
    int64_t inst_outer_ = 0;
    int num_sim_models_ = 0;
};

std::unique_ptr<SolverBase> make_solver(int precision) {
    if (precision == PDIPC_PREC_FP64) return std::unique_ptr<SolverBase>(new Solver<double, double>());
    if (precision == PDIPC_PREC_MIXED) return std::unique_ptr<SolverBase>(new Solver<float, double>());
    return std::unique_ptr<SolverBase>(new Solver<float, float>());
}

}  // namespace pdipc
