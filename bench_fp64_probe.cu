// FP64 issue-rate calibration for bench.py (not part of the library):
// eight independent FMA chains per thread, enough warps to fill every SM.
// bench.py times it with CUDA events to report the FP64 roofline of the
// map kernels on the GPU they run on.  Built by __graft_entry__.build()
// into cmm-s2_gb300/lib/libcmmprobe.so.
#include <cuda_runtime.h>

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

// blocks x 256 threads, `iters` rounds of 8 FMAs each; sink: blocks*256
// doubles.  Returns 0 or the CUDA error code.
extern "C" int bench_fp64_probe(int blocks, int iters, double* sink, void* stream) {
  if (blocks < 1 || iters < 1 || !sink) return -1;
  fp64_probe_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(sink, iters, 0.999, 0.001);
  return (int)cudaGetLastError();
}
