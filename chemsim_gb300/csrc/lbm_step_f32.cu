// lbm_step_f32.cu — fused-step launches for f32 storage.
#include "lbm_step.cuh"

namespace lbmk {

template <>
cudaError_t launch_step<float>(const StepArgs<float>& a, int frame, bool fast,
                            int cells_per_thread, int rows, cudaStream_t stream) {
    switch (cells_per_thread) {
        case 2: return launch_step_v<float, 2>(a, frame, fast, rows, stream);
        case 4: return launch_step_v<float, 4>(a, frame, fast, rows, stream);
        case 8: return launch_step_v<float, 8>(a, frame, fast, rows, stream);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace lbmk
