// Instantiations of the specialised stage kernels (fast_stage.cuh) for one arithmetic; split
// per arithmetic so that the three translation units compile in parallel.
#include "fast_stage.cuh"

namespace p3d {
int launch_fast_df(const FastArgs &a, cudaStream_t st) { return fk_dispatch<DF>(a, st); }
}  // namespace p3d
