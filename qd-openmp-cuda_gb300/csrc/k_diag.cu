// Diagnostics: a register-resident FMA loop to measure the device's FP64 and
// FP32 FMA throughput (the denominators of the FP64 roofline fractions), and a
// self-test of the bounded mbarrier wait used by the pipelined kernels.
#include <string>

#include "qd_internal.h"
#include "qd_mbarrier.cuh"

namespace qd {

template <typename T>
__global__ void k_fma_loop(T *out, int iters, T a, T b) {
  T x0 = (T)threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; i++) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  const T s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == (T)-12345.0) out[threadIdx.x] = s;   // keeps the loop live
}

template <typename T>
static double measure(int iters) {
  int dev = 0, sms = 0;
  QD_CUDA(cudaGetDevice(&dev));
  QD_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  T *out = nullptr;
  QD_CUDA(cudaMalloc(&out, 1024 * sizeof(T)));
  cudaEvent_t e0, e1;
  QD_CUDA(cudaEventCreate(&e0));
  QD_CUDA(cudaEventCreate(&e1));
  const int blocks = sms * 8, threads = 256;
  k_fma_loop<T><<<blocks, threads>>>(out, iters / 10, (T)0.999999, (T)1e-7);   // warm-up
  QD_CUDA(cudaEventRecord(e0));
  k_fma_loop<T><<<blocks, threads>>>(out, iters, (T)0.999999, (T)1e-7);
  QD_CUDA(cudaEventRecord(e1));
  QD_CUDA(cudaEventSynchronize(e1));
  float ms = 0;
  QD_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  const double flops = 2.0 * 8.0 * (double)iters * blocks * threads;
  return flops / (ms * 1e-3) / 1e12;
}

double measure_fp64_tflops() { return measure<double>(20000); }
double measure_fp32_tflops() { return measure<float>(400000); }

// FP64 tensor-core (DMMA) throughput: every warp chains mma.sync m8n8k4 f64
// products into four independent accumulator tiles held in registers
// (8 x 8 x 4 = 256 FMA per instruction per warp).
__global__ void k_dmma_loop(double *out, int iters, double a) {
  double acc[4][2];
#pragma unroll
  for (int t = 0; t < 4; t++) acc[t][0] = acc[t][1] = (double)threadIdx.x * 1e-3 + t;
  const double x = a, y = a * 0.5;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int t = 0; t < 4; t++)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};"
                   : "+d"(acc[t][0]), "+d"(acc[t][1])
                   : "d"(x), "d"(y));
  }
  double s = 0.0;
#pragma unroll
  for (int t = 0; t < 4; t++) s += acc[t][0] + acc[t][1];
  if (s == -12345.0) out[threadIdx.x] = s;   // keeps the loop live
}

double measure_dmma_tflops() {
  int dev = 0, sms = 0;
  QD_CUDA(cudaGetDevice(&dev));
  QD_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  double *out = nullptr;
  QD_CUDA(cudaMalloc(&out, 1024 * sizeof(double)));
  cudaEvent_t e0, e1;
  QD_CUDA(cudaEventCreate(&e0));
  QD_CUDA(cudaEventCreate(&e1));
  const int blocks = sms * 8, threads = 256, iters = 4000;
  k_dmma_loop<<<blocks, threads>>>(out, iters / 10, 0.999);   // warm-up
  QD_CUDA(cudaEventRecord(e0));
  k_dmma_loop<<<blocks, threads>>>(out, iters, 0.999);
  QD_CUDA(cudaEventRecord(e1));
  QD_CUDA(cudaEventSynchronize(e1));
  float ms = 0;
  QD_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  const double flops = 2.0 * 256.0 * 4.0 * (double)iters * blocks * (threads / 32);
  return flops / (ms * 1e-3) / 1e12;
}

// Thread 0 waits (bounded) on a fresh mbarrier of count 1; thread 1 arrives on
// it only when `arrive` is set.  A wait that gives up records QD_ERR_TIMEOUT,
// exactly as the tensor-core kernels do.
__global__ void k_wait_selftest(uint64_t budget_ns, int arrive, int *status, unsigned long long *elapsed_ns) {
  __shared__ uint64_t mb;
  if (threadIdx.x == 0) {
    mbar_init(smem_u32(&mb), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 1 && arrive) mbar_arrive(smem_u32(&mb));
  if (threadIdx.x == 0) {
    const uint64_t t0 = globaltimer();
    const bool ok = mbar_wait_bounded(smem_u32(&mb), 0u, budget_ns);
    *elapsed_ns = globaltimer() - t0;
    if (!ok) atomicCAS(status, 0, QD_ERR_TIMEOUT);
  }
}

void device_wait_selftest(double budget_ms, int arrive) {
  QD_REQUIRE(budget_ms > 0.0 && budget_ms <= 2000.0, "0 < budget_ms <= 2000");
  int *status = nullptr;
  unsigned long long *elapsed = nullptr;
  QD_CUDA(cudaMalloc(&status, sizeof(int)));
  cudaError_t e = cudaMalloc(&elapsed, sizeof(unsigned long long));
  if (e != cudaSuccess) {
    cudaFree(status);
    QD_CUDA(e);
  }
  int st = 0;
  unsigned long long ns = 0;
  e = cudaMemset(status, 0, sizeof(int));
  if (e == cudaSuccess) {
    k_wait_selftest<<<1, 32>>>((uint64_t)(budget_ms * 1e6), arrive ? 1 : 0, status, elapsed);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(&st, status, sizeof(int), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(&ns, elapsed, sizeof(ns), cudaMemcpyDeviceToHost);
  cudaFree(status);
  cudaFree(elapsed);
  QD_CUDA(e);
  if (st)
    throw Error{st, "device wait gave up after " + std::to_string(ns * 1e-6) + " ms (budget " +
                        std::to_string(budget_ms) + " ms)"};
}

}  // namespace qd
