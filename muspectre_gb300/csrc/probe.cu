// FP64 FMA throughput probe (instrumentation; no counterpart in the reference).
//
// The FP64 plain method and the FP64 Newton level of the mixed path run FFT and
// pixel-local passes whose arithmetic intensity (about 1 flop per byte) puts them on
// the FP64 FMA pipe rather than on HBM bandwidth on this GPU.  Their roofline needs a
// measured FP64 peak: this kernel keeps every SM's FP64 pipe busy with independent
// fused multiply-add chains (eight per thread, so that the pipe's latency is covered
// by the chains of one warp and the warps of a block) and reports FLOP/s = 2 x FMAs /
// CUDA-event time.
#include "musg_internal.h"

namespace musg {
namespace {

constexpr int kChains = 8;

__global__ void k_fp64_fma(double *sink, int iters, double a, double b) {
  double v[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) v[c] = (double)(threadIdx.x + c) * 1e-3;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) v[c] = fma(v[c], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += v[c];
  if (s == 12345.678) sink[0] = s;  // keeps the chains live; never true for these inputs
}

}  // namespace

double fp64_fma_tflops(cudaStream_t s) {
  int dev = 0, nsm = 0;
  MUSG_CUDA(cudaGetDevice(&dev));
  MUSG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  double *sink = nullptr;
  MUSG_CUDA(cudaMalloc(&sink, sizeof(double)));
  cudaEvent_t e0, e1;
  MUSG_CUDA(cudaEventCreate(&e0));
  MUSG_CUDA(cudaEventCreate(&e1));
  const int threads = 256, blocks = nsm * 8, iters = 4096;
  float best = 1e30f;
  for (int rep = 0; rep < 4; ++rep) {
    MUSG_CUDA(cudaEventRecord(e0, s));
    k_fp64_fma<<<blocks, threads, 0, s>>>(sink, iters, 0.999999, 1e-9);
    MUSG_CHECK_LAUNCH();
    MUSG_CUDA(cudaEventRecord(e1, s));
    MUSG_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    MUSG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    if (rep > 0 && ms < best) best = ms;  // the first launch warms up
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(sink);
  const double flops = 2.0 * kChains * (double)iters * threads * (double)blocks;
  return flops / (best * 1e-3) / 1e12;
}

}  // namespace musg
