// pdipc_simulator.hpp — header-only C++ class with the reference's simulator
// interface, implemented on the C ABI of libpdipc.so (pdipc.h).
//
// Mirrors, member for member, what callers of the reference use:
//   BaseSimulator            Simulator/BaseSimulator.h:32-136
//   PD_IPC::PdIpcSimulator   Simulator/PD-IPC/PdIpcSimulator.h:441-642, 879-916
//   createSimulator          Simulator/SimulatorFactor.h:13-57
// The reference reads meshes through Qt/tinyxml config files; here models are
// added from vertex/face arrays (addClothModel / addStaticModel), which is what
// addModelFromConfigFile ends up passing to the model.  Errors do not abort the
// process (the reference's CUDA_CALL calls assert(0)): every member records the
// status of its C call, readable through status() and lastError().
#ifndef PDIPC_SIMULATOR_HPP
#define PDIPC_SIMULATOR_HPP

#include <cstdio>
#include <memory>
#include <string>
#include <vector>

#include "pdipc.h"

namespace PD_IPC_GB300 {

typedef float qeal;  // the reference's scalar (DataCore.h:19)

enum RunPlatform { CPU, OPEMMP, CUDA };  // BaseSimulator.h:13-18 (only CUDA exists for PD-IPC)

class BaseSimulator {
public:
    virtual ~BaseSimulator() = default;
    virtual std::string getSimulatorName() { return name_; }
    virtual void initialization() {}
    virtual void animate(int frame = 0) {
        run(frame);
        postRun();
    }
    virtual void run(int frame = 0) { (void)frame; }
    virtual void postRun() {}
    virtual void reset() {}
    virtual void saveSimulator(int frame) { (void)frame; }
    virtual qeal getTimeStep() { return timeStep_; }
    virtual void setTimeStep(qeal t) { timeStep_ = t; }
    virtual qeal getGraviry() { return gravity_; }
    virtual void setGraviry(qeal g) { gravity_ = g; }

protected:
    explicit BaseSimulator(std::string name) : name_(std::move(name)) {}
    std::string name_;
    qeal timeStep_ = 0.01f;  // BaseSimulator.h:37
    qeal gravity_ = -9.8f;   // BaseSimulator.h:38
};

class PdIpcSimulator : public BaseSimulator {
public:
    explicit PdIpcSimulator(std::string simName = "pd_ipc_simulator", RunPlatform platform = CUDA,
                            pdipc_precision precision = PDIPC_PREC_MIXED)
        : BaseSimulator(std::move(simName)) {
        pdipc_default_params(&params_);
        params_.precision = precision;
        if (platform != CUDA) status_ = PDIPC_ERR_ARG;  // no CPU platform for this path, as in the reference
    }
    ~PdIpcSimulator() override {
        if (ctx_) pdipc_destroy(ctx_);
    }
    PdIpcSimulator(const PdIpcSimulator&) = delete;
    PdIpcSimulator& operator=(const PdIpcSimulator&) = delete;

    // config attributes read by readExtraAttributeFromConfigFile (PdIpcSimulator.h:602-642);
    // they take effect at initialization()
    void setDHat(double d) { params_.dhat = d; }
    void setKappa(double k) { params_.kappa = k; }
    void setLocalGlobalIterations(int n) { params_.lg_iterations = n; }
    pdipc_params& params() { return params_; }

    // <object> with <type> 0 k_stretch k_bend k_pin, <density>, <patchDim>
    // (addModelFromConfigFile, PdIpcSimulator.h:462-534); fixed points as in fixed_points.txt
    bool addClothModel(const std::vector<double>& X, const std::vector<int>& F, const std::vector<int>& fixedIds,
                       double density, double strainStiffness, double bendingStiffness, double positionStiffness,
                       int patchDim = 10) {
        Model m{X, F, fixedIds, false, density, strainStiffness, bendingStiffness, positionStiffness, patchDim};
        models_.push_back(std::move(m));
        return true;
    }
    // <object volumetric_mesh="tet"> with <type> 1 k_strain k_volume k_pin
    // (PdIpcVolumetricModel(s0, s1, s2)); X, T from the tetgen .node/.ele pair
    bool addVolumetricModel(const std::vector<double>& X, const std::vector<int>& T, const std::vector<int>& fixedIds,
                            double density, double strainStiffness, double volumeStiffness, double positionStiffness,
                            int patchDim = 10) {
        Model m{X, {}, fixedIds, false, density, strainStiffness, 0.0, positionStiffness, patchDim};
        m.T = T;
        m.k_volume = volumeStiffness;
        models_.push_back(std::move(m));
        return true;
    }
    // <static_object> (addStaticModelFromConfigFile, PdIpcSimulator.h:536-600)
    bool addStaticModel(const std::vector<double>& X, const std::vector<int>& F, int patchDim = 10) {
        Model m{X, F, {}, true, 0.0, 0.0, 0.0, 0.0, patchDim};
        models_.push_back(std::move(m));
        return true;
    }

    void initialization() override {
        if (status_ != PDIPC_OK) return;
        params_.time_step = timeStep_;
        params_.gravity = gravity_;
        if ((status_ = pdipc_create(&params_, &ctx_)) != PDIPC_OK) return;
        for (const Model& m : models_) {
            const int nv = (int)m.X.size() / 3, nf = (int)m.F.size() / 3;
            const int* pins = m.pins.empty() ? nullptr : m.pins.data();
            if (m.is_static)
                status_ = pdipc_add_static(ctx_, m.X.data(), nv, m.F.data(), nf, m.patch_dim);
            else if (!m.T.empty())
                status_ = pdipc_add_volumetric(ctx_, m.X.data(), nv, m.T.data(), (int)m.T.size() / 4, m.density,
                                               m.k_stretch, m.k_volume, pins, (int)m.pins.size(), m.k_pin,
                                               m.patch_dim);
            else
                status_ = pdipc_add_cloth(ctx_, m.X.data(), nv, m.F.data(), nf, m.density, m.k_stretch, m.k_bend,
                                          pins, (int)m.pins.size(), m.k_pin, m.patch_dim);
            if (status_ != PDIPC_OK) return;
        }
        if ((status_ = pdipc_initialize(ctx_)) != PDIPC_OK) return;
        pdipc_stats st;
        pdipc_get_stats(ctx_, &st);
        points_.assign(3 * (size_t)st.n_total, 0.0);
    }
    // PdIpcSimulator::run(frame) -> doTime -> advance (PdIpcSimulator.cpp:18-21, 1538-1796)
    void run(int frame = 0) override {
        (void)frame;
        if (ready()) status_ = pdipc_step(ctx_, 1);
    }
    // postRun: device positions to the host buffer (PdIpcSimulator.cpp:23-32)
    void postRun() override {
        if (ready()) status_ = pdipc_get_positions(ctx_, points_.data());
    }
    void reset() override {
        if (ready()) status_ = pdipc_reset(ctx_);
    }
    // saveDat/frame_XXXX.dat in EigenMatrixIO layout (PdIpcSimulator.h:879-916), with velocities appended
    void saveSimulator(int frame) override {
        if (!ready()) return;
        char name[64];
        std::snprintf(name, sizeof(name), "frame_%04d.dat", frame);
        status_ = pdipc_save(ctx_, (saveDir_ + name).c_str());
    }
    void setSaveDirectory(const std::string& dir) { saveDir_ = dir; }

    const std::vector<double>& points() const { return points_; }  // headless render buffer
    pdipc_status status() const { return status_; }
    std::string lastError() const {
        return ctx_ ? std::string(pdipc_last_error(ctx_)) : std::string(pdipc_status_string(status_));
    }
    pdipc_ctx* context() { return ctx_; }

private:
    struct Model {
        std::vector<double> X;
        std::vector<int> F;
        std::vector<int> pins;
        bool is_static;
        double density, k_stretch, k_bend, k_pin;  // k_stretch: the strain stiffness of a volumetric model
        int patch_dim;
        std::vector<int> T;  // tets of a volumetric model
        double k_volume = 0.0;
    };
    bool ready() { return ctx_ && status_ == PDIPC_OK; }

    pdipc_params params_{};
    pdipc_ctx* ctx_ = nullptr;
    pdipc_status status_ = PDIPC_OK;
    std::vector<Model> models_;
    std::vector<double> points_;
    std::string saveDir_;
};

// createSimulator (SimulatorFactor.h:13-57): this library provides "pd_ipc_simulator".
inline std::unique_ptr<BaseSimulator> createSimulator(const std::string& simName, RunPlatform platform) {
    if (simName == "pd_ipc_simulator") return std::unique_ptr<BaseSimulator>(new PdIpcSimulator(simName, platform));
    return nullptr;
}

}  // namespace PD_IPC_GB300

#endif  // PDIPC_SIMULATOR_HPP
