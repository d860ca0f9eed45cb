// Uses the reference-style C++ interface on top of the C ABI: a 3x3 cloth
// above a static triangle.  Prints the status of initialization and, when a
// device is present, of a few animate() calls.
#include <cstdio>

#include "pdipc_simulator.hpp"

using namespace PD_IPC_GB300;

int main() {
    std::vector<double> X = {0, 0, 0, 0.5, 0, 0, 1, 0, 0, 0, 0, 0.5, 0.5, 0, 0.5, 1, 0, 0.5, 0, 0, 1, 0.5, 0, 1, 1, 0, 1};
    std::vector<int> F = {0, 3, 4, 0, 4, 1, 1, 4, 2, 2, 4, 5, 3, 6, 4, 4, 6, 7, 4, 7, 8, 4, 8, 5};
    std::vector<double> S = {-1, -0.5, -1, 2, -0.5, -1, -1, -0.5, 2};
    std::vector<int> SF = {0, 1, 2};
    auto sim = createSimulator("pd_ipc_simulator", CUDA);
    if (!sim || createSimulator("fem_simulator", CUDA)) return 2;
    auto* pd = static_cast<PdIpcSimulator*>(sim.get());
    pd->setTimeStep(1.0f / 240);
    pd->addClothModel(X, F, {0, 2}, 0.1, 1e4, 1e-3, 1e6, 3);
    pd->addStaticModel(S, SF, 1);
    pd->initialization();
    std::printf("init %s\n", pdipc_status_string(pd->status()));
    if (pd->status() != PDIPC_OK) return 0;
    for (int f = 0; f < 5; ++f) pd->animate(f);
    std::printf("animate %s y4=%.6f\n", pdipc_status_string(pd->status()), pd->points()[3 * 4 + 1]);
    return pd->status() == PDIPC_OK ? 0 : 1;
}
