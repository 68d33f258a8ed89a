// probe.cu -- the bandwidth denominators of the roofline figures, measured on the running GPU.
//
// The tracker re-reads every pair's points and frame level across ~26 passes; those re-reads are
// served by L2, so its "achieved" bytes are set against the L2 read bandwidth of an L2-resident
// working set as well as against the HBM copy peak.  This file measures the former: a persistent
// grid re-reads a buffer that fits in L2 (but in no SM's L1) with L2-only float4 loads.
#include <cuda_runtime.h>

#include "lsdg_host.h"

namespace {

lsdg_status check(lsdg_ctx* ctx, cudaError_t e) { return e == cudaSuccess ? LSDG_OK : ctx_cuda(ctx, e, "cudaSetDevice"); }

__global__ void __launch_bounds__(512) l2_read_kernel(const float4* __restrict__ buf, long n4, int reps,
                                                      float* __restrict__ sink) {
  const long stride = (long)gridDim.x * blockDim.x;
  float acc = 0.f;
  for (int r = 0; r < reps; ++r) {
    float4 a = make_float4(0.f, 0.f, 0.f, 0.f), b = a;
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + stride < n4; i += 2 * stride) {  // two loads in flight per thread
      const float4 x = __ldcg(&buf[i]);
      const float4 y = __ldcg(&buf[i + stride]);
      a.x += x.x; a.y += x.y; a.z += x.z; a.w += x.w;
      b.x += y.x; b.y += y.y; b.z += y.z; b.w += y.w;
    }
    if (i < n4) {
      const float4 x = __ldcg(&buf[i]);
      a.x += x.x; a.y += x.y; a.z += x.z; a.w += x.w;
    }
    acc += (a.x + a.y) + (a.z + a.w) + (b.x + b.y) + (b.z + b.w);
  }
  sink[(long)blockIdx.x * blockDim.x + threadIdx.x] = acc;  // keeps the loads
}

// Non-zero contents (a buffer of zeros could be served by the memory system's compression of
// constant data rather than read).
__global__ void fill_kernel(float4* __restrict__ buf, long n4) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += (long)gridDim.x * blockDim.x) {
    const float v = (float)(i & 1023) * 0.25f + 1.0f;
    buf[i] = make_float4(v, v + 1.f, v + 2.f, v + 3.f);
  }
}

}  // namespace

extern "C" lsdg_status lsdg_measure_l2_read(lsdg_ctx* ctx, long bytes, int reps, double* gbps) {
  if (!ctx || !gbps || bytes < (1L << 20) || reps < 1) return ctx_fail(ctx, LSDG_INVALID_ARG, "bad argument");
  if (check(ctx, cudaSetDevice(ctx->device)) != LSDG_OK) return LSDG_CUDA_ERROR;
  const long n4 = bytes / 16;
  const int blocks = 4 * (ctx->sm_count > 0 ? ctx->sm_count : 1), threads = 512;
  float4* buf = nullptr;
  float* sink = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaMalloc(&buf, n4 * 16);
  if (e == cudaSuccess) e = cudaMalloc(&sink, sizeof(float) * blocks * threads);
  if (e == cudaSuccess) {
    fill_kernel<<<blocks, threads, 0, ctx->stream>>>(buf, n4);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  float ms = 0.f;
  if (e == cudaSuccess) {
    l2_read_kernel<<<blocks, threads, 0, ctx->stream>>>(buf, n4, 2, sink);  // brings the buffer into L2
    cudaEventRecord(e0, ctx->stream);
    l2_read_kernel<<<blocks, threads, 0, ctx->stream>>>(buf, n4, reps, sink);
    cudaEventRecord(e1, ctx->stream);
    e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (buf) cudaFree(buf);
  if (sink) cudaFree(sink);
  if (e != cudaSuccess) return ctx_cuda(ctx, e, "L2 read probe");
  ctx->launches += 3;
  *gbps = (double)n4 * 16.0 * reps / (ms * 1e-3) / 1e9;
  return LSDG_OK;
}
