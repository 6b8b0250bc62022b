// Instantiations of the specialised stage kernels (fast_stage.cuh) for one (arithmetic, kind,
// part), selected at compile time: P3D_FAST_ARITH 0 float-float, 1 native FP64, 2 FP32, 3 FP32
// with split twiddles (lengths 512, 1024, 2048), P3D_FAST_KIND a FastKind, and P3D_FAST_PART the
// half of the lengths (float-float only; fast_part_of).  The build compiles this file once per
// triple, in parallel.
#include "fast_stage.cuh"

#if !defined(P3D_FAST_ARITH) || !defined(P3D_FAST_KIND)
#error "compile with -DP3D_FAST_ARITH=<0|1|2|3> -DP3D_FAST_KIND=<0..4> [-DP3D_FAST_PART=<0|1>]"
#endif
#ifndef P3D_FAST_PART
#define P3D_FAST_PART 0
#endif

namespace p3d {
#if P3D_FAST_ARITH == 0
using FastArith = DFP;
#elif P3D_FAST_ARITH == 1
using FastArith = Native<double>;
#elif P3D_FAST_ARITH == 2
using FastArith = Native<float>;
#else
using FastArith = FSplit;  // FP32 with split twiddles, long lines only
#endif

static_assert(P3D_FAST_PART < fast_nparts<FastArith>(), "part out of range for this arithmetic");

template <>
int fast_launch_part<FastArith, P3D_FAST_KIND, P3D_FAST_PART>(int n, const FParams &p, const FGroup *g, int ctas,
                                                              cudaStream_t st, const CUtensorMap *tm) {
  return fk_dispatch_n<FastArith, P3D_FAST_KIND, P3D_FAST_PART>(n, p, g, ctas, st, tm);
}
}  // namespace p3d
