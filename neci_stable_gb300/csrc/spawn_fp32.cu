// spawn_fp32.cu -- the spawn kernels with FP32 H_ij, p_gen and amplitudes
// (the mixed-precision step).
#include "spawn.cuh"

namespace neci {

template void launch_spawn_real<float>(Engine &e, cudaStream_t s);

}  // namespace neci
