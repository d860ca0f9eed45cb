// pd_persistent_band.cu — the band variants of the persistent PD solve
// (correction form: the iterate's band in shared memory), in their own
// translation unit so that they compile beside the others.  kMode 2 reads
// the rows' column-offset patterns from parameter space (the whole table fits
// there); kMode 3 keeps each CTA's own patterns in shared memory (a batch of
// many mesh sizes has more patterns than parameter space holds).
#include "pd_persistent.cuh"

namespace pdipc {

const void* persistent_band_kernel(bool param_patterns, bool l1_gather, int rows_per_thread, bool tets) {
    if (tets) {
        if (!l1_gather || rows_per_thread > 2) return nullptr;
        return param_patterns ? kernel_for_tets<float, true, 2>(rows_per_thread)
                              : kernel_for_tets<float, true, 3>(rows_per_thread);
    }
    if (param_patterns)
        return l1_gather ? kernel_for<float, true, 2, true>(rows_per_thread)
                         : kernel_for<float, true, 2, false>(rows_per_thread);
    return l1_gather ? kernel_for<float, true, 3, true>(rows_per_thread)
                     : kernel_for<float, true, 3, false>(rows_per_thread);
}

}  // namespace pdipc
