// Internal interface between the stage executor (core.cpp) and the runtimes built on it: the
// batch executor (batch.cpp) and the serving loop (serve.cpp).  Not exported.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <vector>

#include "kernels.h"

namespace p3d {

// A scratch set holds the two ping-pong intermediate fields of a plan's stage chain.  Plans that
// run one after another on the same stream can share a set.
void *scratch_set_create();
void scratch_set_destroy(void *set);
size_t scratch_set_bytes(const void *set);
// allocates both slots at `bytes` each (no-op when already that large)
int scratch_set_reserve(void *set, size_t bytes);
// a set over two caller-owned device buffers of `bytes` each (not freed by scratch_set_destroy)
void *scratch_set_wrap(void *s0, void *s1, size_t bytes);

// field sizes of a 3D plan, and the size of each scratch slot its stage chain needs
int plan3d_sizes(int plan, size_t *in_bytes, size_t *out_bytes, size_t *scratch_bytes, int *prec);

// Runs a 3D plan on device pointers, on stream `st`, with the intermediates in `scratch_set`,
// without synchronising.  With `capturing` set no allocation or synchronising call is made, so the
// launches can be recorded into a CUDA graph.
int exec_plan_on(int plan, const void *in, void *out, int idir, cudaStream_t st, void *scratch_set, bool capturing);

// Runs the executor's buffer assignment for a 3D plan (device pointers, intermediates in
// `scratch_set`, allocated here if needed) and appends its stages to *rec instead of launching them.
int record_plan(int plan, const void *in, void *out, int idir, void *scratch_set, std::vector<StageLaunch> *rec);
DeviceTables *device_tables();

bool device_ready();
cudaStream_t library_stream();
bool library_sync();
int current_arith();
void add_kernel_count(long long n);
long long kernel_count_now();
void record_error(int code, const char *msg);

}  // namespace p3d
