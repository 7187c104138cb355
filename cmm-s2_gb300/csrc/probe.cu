// FP64 issue-rate calibration kernel: eight independent FMA chains per
// thread, enough warps to fill every SM.  Used to report the FP64 roofline
// of the kernels above on the GPU they run on.
#include <cuda_runtime.h>

#include "cmm_internal.h"

namespace cmm {

namespace {

__global__ void fp64_probe_kernel(double* __restrict__ sink, int iters, double a, double b) {
  double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5,
         x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  sink[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

}  // namespace

int launch_fp64_probe(int blocks, int iters, double* sink, cudaStream_t s) {
  fp64_probe_kernel<<<blocks, 256, 0, s>>>(sink, iters, 0.999, 0.001);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? CMM_OK : cuda_fail(e, "fp64_probe_kernel");
}

}  // namespace cmm
