// Throughput probes for the roofline denominators that a copy / GEMM
// measurement does not give: FP32 FMA, FP64 FMA and MUFU ex2 issue rates of
// the whole GPU.  Each thread runs independent dependency chains long enough
// to hide latency; the grid fills every SM several times over.
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/tcw_b200.h"

namespace {

constexpr int kChains = 8;
constexpr int kIters = 2048;

__global__ void __launch_bounds__(256) probe_fp32(float *out, float a, float b) {
  float v[kChains];
#pragma unroll
  for (int c = 0; c < kChains; c++) v[c] = threadIdx.x * 1e-3f + c;
  for (int i = 0; i < kIters; i++) {
#pragma unroll
    for (int c = 0; c < kChains; c++) v[c] = fmaf(v[c], a, b);
  }
  float s = 0.0f;
#pragma unroll
  for (int c = 0; c < kChains; c++) s += v[c];
  if (s == 1234.5f) out[0] = s;  // keeps the chains live
}

__global__ void __launch_bounds__(256) probe_fp64(double *out, double a, double b) {
  double v[kChains];
#pragma unroll
  for (int c = 0; c < kChains; c++) v[c] = threadIdx.x * 1e-3 + c;
  for (int i = 0; i < kIters / 16; i++) {
#pragma unroll
    for (int c = 0; c < kChains; c++) v[c] = fma(v[c], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < kChains; c++) s += v[c];
  if (s == 1234.5) out[0] = s;
}

__global__ void __launch_bounds__(256) probe_fp32x2(float *out, float a, float b) {
  unsigned long long v[kChains], A, B;
  asm("mov.b64 %0, {%1, %2};" : "=l"(A) : "f"(a), "f"(a));
  asm("mov.b64 %0, {%1, %2};" : "=l"(B) : "f"(b), "f"(b));
#pragma unroll
  for (int c = 0; c < kChains; c++) {
    float x = threadIdx.x * 1e-3f + c;
    asm("mov.b64 %0, {%1, %2};" : "=l"(v[c]) : "f"(x), "f"(x + 0.5f));
  }
  for (int i = 0; i < kIters; i++) {
#pragma unroll
    for (int c = 0; c < kChains; c++)
      asm volatile("fma.rn.f32x2 %0, %0, %1, %2;" : "+l"(v[c]) : "l"(A), "l"(B));
  }
  float s = 0.0f;
#pragma unroll
  for (int c = 0; c < kChains; c++) {
    float x, y;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(x), "=f"(y) : "l"(v[c]));
    s += x + y;
  }
  if (s == 1234.5f) out[0] = s;
}

__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm volatile("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__global__ void __launch_bounds__(256) probe_mufu(float *out, float a) {
  float v[kChains];
#pragma unroll
  for (int c = 0; c < kChains; c++) v[c] = -1e-3f * (threadIdx.x + c);
  for (int i = 0; i < kIters / 4; i++) {
#pragma unroll
    for (int c = 0; c < kChains; c++) v[c] = ex2_approx(v[c]) * a;
  }
  float s = 0.0f;
#pragma unroll
  for (int c = 0; c < kChains; c++) s += v[c];
  if (s == 1234.5f) out[0] = s;
}

template <class F>
float time_ms(F launch, cudaStream_t s, int reps) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  launch();  // warm-up
  cudaEventRecord(e0, s);
  for (int r = 0; r < reps; r++) launch();
  cudaEventRecord(e1, s);
  cudaEventSynchronize(e1);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return ms / reps;
}

}  // namespace

extern "C" {

// Measured peaks of `device`: FP32 and FP64 in TFLOP/s (an FMA counts 2),
// MUFU ex2 in tera-operations/s, and FP32 through packed fma.rn.f32x2
// (4 flops per instruction).  Measurement utility with no counterpart in
// the reference; takes well under a second.
int tcw_probe_peaks(int device, double *fp32_tflops, double *fp64_tflops, double *mufu_tops,
                    double *fp32x2_tflops) {
  if (cudaSetDevice(device) != cudaSuccess) {
    cudaGetLastError();
    return TCW_ERR_NO_DEVICE;
  }
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  float *buf = nullptr;
  if (cudaMalloc(&buf, 64) != cudaSuccess) {
    cudaGetLastError();
    return TCW_ERR_ALLOC;
  }
  cudaStream_t s;
  cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  const int blocks = sms * 16, threads = 256;
  const double nthr = (double)blocks * threads;
  float ms32 = time_ms([&] { probe_fp32<<<blocks, threads, 0, s>>>(buf, 0.999f, 1e-3f); }, s, 5);
  float ms64 = time_ms([&] {
    probe_fp64<<<blocks, threads, 0, s>>>(reinterpret_cast<double *>(buf), 0.999, 1e-3);
  }, s, 3);
  float msmu = time_ms([&] { probe_mufu<<<blocks, threads, 0, s>>>(buf, 0.5f); }, s, 5);
  float ms2 = time_ms([&] { probe_fp32x2<<<blocks, threads, 0, s>>>(buf, 0.999f, 1e-3f); }, s, 5);
  cudaError_t e = cudaGetLastError();
  cudaStreamDestroy(s);
  cudaFree(buf);
  if (e != cudaSuccess) return TCW_ERR_CUDA;
  if (fp32_tflops) *fp32_tflops = 2.0 * nthr * kChains * kIters / (ms32 * 1e-3) / 1e12;
  if (fp64_tflops) *fp64_tflops = 2.0 * nthr * kChains * (kIters / 16) / (ms64 * 1e-3) / 1e12;
  if (mufu_tops) *mufu_tops = nthr * kChains * (kIters / 4) / (msmu * 1e-3) / 1e12;
  if (fp32x2_tflops) *fp32x2_tflops = 4.0 * nthr * kChains * kIters / (ms2 * 1e-3) / 1e12;
  return TCW_OK;
}

}  // extern "C"
