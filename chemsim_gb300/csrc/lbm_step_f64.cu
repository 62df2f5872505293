// lbm_step_f64.cu — fused-step launches for f64 storage.
#include "lbm_step.cuh"

namespace lbmk {

template <>
cudaError_t launch_step<double>(const StepArgs<double>& a, int frame, bool fast,
                            int cells_per_thread, int rows, cudaStream_t stream) {
    switch (cells_per_thread) {
        case 2: return launch_step_v<double, 2>(a, frame, fast, rows, stream);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace lbmk
