// Instantiations of the specialised stage kernels (fast_stage.cuh) for one (arithmetic, kind)
// pair, selected at compile time: P3D_FAST_ARITH 0 float-float, 1 native FP64, 2 FP32, and
// P3D_FAST_KIND a FastKind.  The build compiles this file once per pair, in parallel.
#include "fast_stage.cuh"

#if !defined(P3D_FAST_ARITH) || !defined(P3D_FAST_KIND)
#error "compile with -DP3D_FAST_ARITH=<0|1|2> -DP3D_FAST_KIND=<0|1|2|3|4>"
#endif

namespace p3d {
#if P3D_FAST_ARITH == 0
using FastArith = DFP;
#elif P3D_FAST_ARITH == 1
using FastArith = Native<double>;
#else
using FastArith = Native<float>;
#endif

template <>
int fast_launch_kind<FastArith, P3D_FAST_KIND>(int n, const FParams &p, const FGroup *g, int ctas, cudaStream_t st) {
  return fk_dispatch_n<FastArith, P3D_FAST_KIND>(n, p, g, ctas, st);
}
}  // namespace p3d
