// spawn_fp64.cu -- the spawn kernels with FP64 amplitudes, and the step's
// spawn launch.
#include "spawn.cuh"

namespace neci {

template void launch_spawn_real<double>(Engine &e, cudaStream_t s);
extern template void launch_spawn_real<float>(Engine &e, cudaStream_t s);

void launch_spawn(Engine &e, cudaStream_t s) {
    if (e.h_params->precision == NECI_PREC_MIXED) launch_spawn_real<float>(e, s);
    else launch_spawn_real<double>(e, s);
}

}  // namespace neci
