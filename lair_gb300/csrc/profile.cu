// Optional per-launch CUDA-event profile of the luhot kernels.
//
// When enabled (luhot_profile_enable), every kernel launch is bracketed by a
// pair of events recorded on the stream the kernel runs on; luhot_profile_read
// synchronises and sums the elapsed times, algorithmic flops and bytes per
// kernel class.  Off by default; the bracketing costs two event records per
// launch.
#include <algorithm>

#include "common.cuh"
#include "luhot_internal.h"

namespace luhot {

static cudaEvent_t take_event(luhot_ctx* ctx) {
  if (!ctx->prof_event_pool.empty()) {
    cudaEvent_t e = ctx->prof_event_pool.back();
    ctx->prof_event_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  if (cudaEventCreate(&e) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return e;
}

void prof_begin(luhot_ctx* ctx, int cls) {
  (void)cls;
  if (!ctx->prof_on) return;
  ctx->prof_pending = take_event(ctx);
  if (ctx->prof_pending) cudaEventRecord(ctx->prof_pending, ctx->stream);
}

void prof_end(luhot_ctx* ctx, int cls, double flops, double bytes) {
  count_launch(ctx);
  if (!ctx->prof_on || !ctx->prof_pending) return;
  cudaEvent_t stop = take_event(ctx);
  if (!stop) return;
  cudaEventRecord(stop, ctx->stream);
  ctx->prof_records.push_back(ProfRecord{cls, ctx->prof_pending, stop, flops, bytes});
  ctx->prof_pending = nullptr;
}

static void recycle(luhot_ctx* ctx) {
  for (auto& r : ctx->prof_records) {
    ctx->prof_event_pool.push_back(r.start);
    ctx->prof_event_pool.push_back(r.stop);
  }
  ctx->prof_records.clear();
}

}  // namespace luhot

using namespace luhot;

extern "C" {

int luhot_profile_enable(luhot_ctx* ctx, int on) {
  if (!ctx) return LUHOT_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  recycle(ctx);
  ctx->prof_on = on != 0;
  return LUHOT_OK;
}

int luhot_profile_read(luhot_ctx* ctx, luhot_profile* out) {
  if (!ctx || !out) return LUHOT_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  cudaSetDevice(ctx->device);
  LUHOT_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  *out = luhot_profile{};
  for (auto& r : ctx->prof_records) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, r.start, r.stop) != cudaSuccess) {
      cudaGetLastError();
      continue;
    }
    out->ms[r.cls] += ms;
    out->flops[r.cls] += r.flops;
    out->bytes[r.cls] += r.bytes;
    out->launches[r.cls] += 1;
  }
  recycle(ctx);
  return LUHOT_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// FP64 tensor peak probe: every warp keeps 8 independent m8n8k4 DMMA chains
// in registers (no shared or global traffic inside the loop) and writes one
// value per thread at the end.
// ---------------------------------------------------------------------------
namespace luhot {

__device__ __forceinline__ void peak_dmma(double& d0, double& d1, double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
               : "+d"(d0), "+d"(d1)
               : "d"(a), "d"(b));
}

// Every chain starts from a different accumulator and multiplies different
// operands, so no two chains compute the same values (identical chains can be
// merged by the assembler, which would overstate the rate).
__global__ void dmma_peak_kernel(double* out, double a, double b, int iters) {
  double c[8][2], av[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    c[q][0] = q * 0.25 + threadIdx.x * 1e-6;
    c[q][1] = q * 0.5 - threadIdx.x * 1e-6;
    av[q] = a + q * 1e-3 + threadIdx.x * 1e-9;
  }
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int q = 0; q < 8; ++q) peak_dmma(c[q][0], c[q][1], av[q], b);
  }
  double s = 0.0;
#pragma unroll
  for (int q = 0; q < 8; ++q) s += c[q][0] + c[q][1];
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace luhot

extern "C" int luhot_measure_dmma_peak(luhot_ctx* ctx, double* tflops) {
  if (!ctx || !tflops) return LUHOT_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lock(ctx->mu);
  cudaSetDevice(ctx->device);
  const int iters = 2048;
  double best = 0.0;
  const int launch_shapes[][2] = {{4, 256}, {8, 256}, {2, 512}, {4, 128}};
  double* out = nullptr;
  const size_t max_threads = (size_t)ctx->num_sms * 8 * 256;
  LUHOT_CUDA_TRY(ctx, cudaMalloc(&out, max_threads * sizeof(double)));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  for (int rep = 0; rep < 2; ++rep) {
    for (const auto& cfg : launch_shapes) {
      const int blocks = ctx->num_sms * cfg[0], threads = cfg[1];
      cudaEventRecord(e0, ctx->stream);
      dmma_peak_kernel<<<blocks, threads, 0, ctx->stream>>>(out, 0.999, 1e-3, iters);
      cudaEventRecord(e1, ctx->stream);
      cudaEventSynchronize(e1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      const double flops = (double)blocks * (threads / 32) * iters * 8 * 512.0;
      if (ms > 0) best = std::max(best, flops / (ms * 1e-3) / 1e12);
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  LUHOT_CUDA_TRY(ctx, cudaGetLastError());
  *tflops = best;
  return LUHOT_OK;
}
