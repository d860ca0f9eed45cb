// pd_persistent.cu — kernels of the persistent PD solve without the band
// (matrix streamed from L2, or values and offset patterns in shared memory),
// the tet variants, the dispatch over every variant and the launch.  The
// band variants are compiled in pd_persistent_band.cu.
#include "pd_persistent.cuh"

namespace pdipc {
namespace {

template <bool kL1>
const void* kernel_for_l1(bool correction, int mode, int R) {
    if (correction) return mode == 1 ? kernel_for<float, true, 1, kL1>(R) : kernel_for<float, true, 0, kL1>(R);
    return mode == 1 ? kernel_for<float, false, 1, kL1>(R) : kernel_for<float, false, 0, kL1>(R);
}

}  // namespace

const void* persistent_kernel(bool correction, bool matrix_in_smem, bool band, bool band_param, bool l1_gather,
                              int rows_per_thread, bool tets) {
    if (band) return correction ? persistent_band_kernel(band_param, l1_gather, rows_per_thread, tets) : nullptr;
    const int mode = matrix_in_smem ? 1 : 0;
    if (tets) {
        if (!l1_gather || rows_per_thread > 2) return nullptr;
        if (correction)
            return mode == 1 ? kernel_for_tets<float, true, 1>(rows_per_thread)
                             : kernel_for_tets<float, true, 0>(rows_per_thread);
        return mode == 1 ? kernel_for_tets<float, false, 1>(rows_per_thread)
                         : kernel_for_tets<float, false, 0>(rows_per_thread);
    }
    return l1_gather ? kernel_for_l1<true>(correction, mode, rows_per_thread)
                     : kernel_for_l1<false>(correction, mode, rows_per_thread);
}

template <typename S>
cudaError_t launch_args(const PersistPlan& plan, const PersistArgs<float, S>& args, cudaStream_t s) {
    const bool correction = std::is_same<S, double>::value;
    const void* f = persistent_kernel(correction, plan.matrix_in_smem, plan.own_max > 0, plan.band_param,
                                      plan.l1_gather, plan.rows_per_thread, args.ntet > 0);
    if (!f) return cudaErrorInvalidConfiguration;
    void* params[] = {(void*)&args};
    const int grid = args.ctaHi - args.ctaLo + 1;
    if (grid < 1 || args.ctaLo < 0 || args.ctaHi >= plan.ctas) return cudaErrorInvalidConfiguration;
    return cudaLaunchCooperativeKernel(f, dim3(grid), dim3(plan.threads), params, plan.smem_bytes, s);
}

cudaError_t launch_pd_persistent(const PersistPlan& plan, const PersistArgs<float, float>& args, cudaStream_t s) {
    return launch_args(plan, args, s);
}
cudaError_t launch_pd_persistent(const PersistPlan& plan, const PersistArgs<float, double>& args, cudaStream_t s) {
    return launch_args(plan, args, s);
}

}  // namespace pdipc
