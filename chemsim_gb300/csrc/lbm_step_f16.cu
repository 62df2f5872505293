// lbm_step_f16.cu — fused-step launches for IEEE-half deviation storage.
#include "lbm_step.cuh"

namespace lbmk {

template <>
cudaError_t launch_step<__half>(const StepArgs<float>& a, int frame, bool fast,
                            int cells_per_thread, int rows, cudaStream_t stream) {
    switch (cells_per_thread) {
        case 4: return launch_step_v<__half, 4>(a, frame, fast, rows, stream);
        case 8: return launch_step_v<__half, 8>(a, frame, fast, rows, stream);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace lbmk
