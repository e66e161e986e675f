// FP64 throughput probe: the roofline denominators for the FP64 element
// kernels (MEASURED_PEAKS.json holds HBM and bf16 figures only).  Two short
// kernels of independent FP64 work: scalar FMA chains and mma.sync
// m8n8k4 f64 (DMMA) chains, timed with CUDA events.
#include <cuda_runtime.h>

#include "../../include/gb_newton.h"
#include "gb_context.h"

namespace gb {

static constexpr int kProbeIters = 2048;

__global__ void probe_fma64(double *out, double s) {
  double a0 = threadIdx.x * 1e-3, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4,
         a5 = a0 + 5, a6 = a0 + 6, a7 = a0 + 7;
  for (int i = 0; i < kProbeIters; i++) {
    a0 = fma(a0, s, 0.5);
    a1 = fma(a1, s, 0.5);
    a2 = fma(a2, s, 0.5);
    a3 = fma(a3, s, 0.5);
    a4 = fma(a4, s, 0.5);
    a5 = fma(a5, s, 0.5);
    a6 = fma(a6, s, 0.5);
    a7 = fma(a7, s, 0.5);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

__global__ void probe_dmma(double *out, double s) {
  double a = threadIdx.x * 1e-3, b = s;
  double c0 = 0, c1 = 0, d0 = 0, d1 = 0, e0 = 0, e1 = 0, f0 = 0, f1 = 0;
  for (int i = 0; i < kProbeIters / 4; i++) {
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                 : "+d"(c0), "+d"(c1) : "d"(a), "d"(b));
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                 : "+d"(d0), "+d"(d1) : "d"(a), "d"(b));
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                 : "+d"(e0), "+d"(e1) : "d"(a), "d"(b));
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                 : "+d"(f0), "+d"(f1) : "d"(a), "d"(b));
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = c0 + c1 + d0 + d1 + e0 + e1 + f0 + f1;
}

// DMMA chains whose operands change every iteration (integer updates of the
// low mantissa bits, so no FP64 instruction besides the mma itself): the
// loop-invariant operands of probe_dmma can run faster than mma.sync on
// operands that change, as in a real contraction.
__global__ void probe_dmma_varying(double *out, double s) {
  long long a0 = __double_as_longlong(1.0 + threadIdx.x * 1e-3), b0 = __double_as_longlong(s);
  long long a1 = a0 ^ 3, b1 = b0 ^ 5, a2 = a0 ^ 6, b2 = b0 ^ 9, a3 = a0 ^ 12, b3 = b0 ^ 17;
  double c0 = 0, c1 = 0, d0 = 0, d1 = 0, e0 = 0, e1 = 0, f0 = 0, f1 = 0;
  for (int i = 0; i < kProbeIters / 4; i++) {
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                 : "+d"(c0), "+d"(c1) : "d"(__longlong_as_double(a0)), "d"(__longlong_as_double(b0)));
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                 : "+d"(d0), "+d"(d1) : "d"(__longlong_as_double(a1)), "d"(__longlong_as_double(b1)));
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                 : "+d"(e0), "+d"(e1) : "d"(__longlong_as_double(a2)), "d"(__longlong_as_double(b2)));
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                 : "+d"(f0), "+d"(f1) : "d"(__longlong_as_double(a3)), "d"(__longlong_as_double(b3)));
    a0 ^= 0x11; b0 ^= 0x22; a1 ^= 0x33; b1 ^= 0x44; a2 ^= 0x55; b2 ^= 0x66; a3 ^= 0x77; b3 ^= 0x88;
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = c0 + c1 + d0 + d1 + e0 + e1 + f0 + f1;
}

}  // namespace gb

// TFLOP/s of the varying-operand DMMA probe (see probe_dmma_varying)
extern "C" int gb_probe_dmma_varying(double *tflops) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = sms * 8, threads = 256;
  double *out = nullptr;
  cudaError_t e = cudaMalloc(&out, sizeof(double) * blocks * threads);
  if (e != cudaSuccess) return gb::cuda_fail(e, "probe buffer");
  cudaEvent_t t0, t1;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  float best = 1e30f, ms;
  for (int rep = 0; rep < 3; rep++) {
    cudaEventRecord(t0);
    gb::probe_dmma_varying<<<blocks, threads>>>(out, 0.999);
    cudaEventRecord(t1);
    cudaEventSynchronize(t1);
    cudaEventElapsedTime(&ms, t0, t1);
    best = ms < best ? ms : best;
  }
  e = cudaGetLastError();
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  cudaFree(out);
  if (e != cudaSuccess) return gb::cuda_fail(e, "probe");
  if (tflops) *tflops = 512.0 * gb::kProbeIters * (double)blocks * (threads / 32) / (best * 1e-3) / 1e12;
  return 0;
}

extern "C" int gb_probe_fp64_peaks(double *dmma_tflops, double *fma_tflops) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = sms * 8, threads = 256;
  double *out = nullptr;
  cudaError_t e = cudaMalloc(&out, sizeof(double) * blocks * threads);
  if (e != cudaSuccess) return gb::cuda_fail(e, "probe buffer");
  cudaEvent_t t0, t1;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  float best_f = 1e30f, best_d = 1e30f, ms;
  for (int rep = 0; rep < 3; rep++) {
    cudaEventRecord(t0);
    gb::probe_fma64<<<blocks, threads>>>(out, 0.999);
    cudaEventRecord(t1);
    cudaEventSynchronize(t1);
    cudaEventElapsedTime(&ms, t0, t1);
    best_f = ms < best_f ? ms : best_f;
    cudaEventRecord(t0);
    gb::probe_dmma<<<blocks, threads>>>(out, 0.999);
    cudaEventRecord(t1);
    cudaEventSynchronize(t1);
    cudaEventElapsedTime(&ms, t0, t1);
    best_d = ms < best_d ? ms : best_d;
  }
  e = cudaGetLastError();
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  cudaFree(out);
  if (e != cudaSuccess) return gb::cuda_fail(e, "probe");
  const double fma_flops = 2.0 * 8 * gb::kProbeIters * (double)blocks * threads;
  const double mma_flops = 512.0 * gb::kProbeIters * (double)blocks * (threads / 32);
  if (fma_tflops) *fma_tflops = fma_flops / (best_f * 1e-3) / 1e12;
  if (dmma_tflops) *dmma_tflops = mma_flops / (best_d * 1e-3) / 1e12;
  return 0;
}
