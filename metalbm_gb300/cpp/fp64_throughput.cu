// FP64 / FP32 throughput probe for the GPU the library runs on.
//
// The FP64 kernels of this library are bound by the FP64 pipe and by FP64
// log throughput on GB300, not by HBM; this program measures those roofs:
// FP64 FMA, FP32 FMA (8 independent chains per thread), CUDA's FP64 log and
// FP64 division, each over (SMs x 8) blocks of 256 threads, timed with CUDA
// events after a warm-up launch.
//
// Build and run:
//   nvcc -gencode arch=compute_103a,code=sm_103a -O3 -o fp64_throughput \
//        metalbm_gb300/cpp/fp64_throughput.cu && ./fp64_throughput
#include <cstdio>
#include <cuda_runtime.h>
__global__ void dfma(double* out, int iters) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  double x[8];
  for (int k = 0; k < 8; ++k) x[k] = 1e-3 * (t + k);
  const double b = 0.999999, c = 1e-7;
  for (int i = 0; i < iters; ++i)
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = fma(x[k], b, c);
  double s = 0; for (int k = 0; k < 8; ++k) s += x[k];
  out[t] = s;
}
__global__ void ffma(double* out, int iters) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  float x[8];
  for (int k = 0; k < 8; ++k) x[k] = 1e-3f * (t + k);
  const float b = 0.999999f, c = 1e-7f;
  for (int i = 0; i < iters; ++i)
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = fmaf(x[k], b, c);
  float s = 0; for (int k = 0; k < 8; ++k) s += x[k];
  out[t] = s;
}
__global__ void dlog(double* out, int iters) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  double acc = 0.0, x = 1.0 + 1e-9 * t;
  for (int i = 0; i < iters; ++i) { acc += log(x); x += 1e-12; }
  out[t] = acc;
}
__global__ void ddiv(double* out, int iters) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  double acc = 0.0, x = 1.0 + 1e-9 * t;
  for (int i = 0; i < iters; ++i) { acc += 1.0 / x; x += 1e-12; }
  out[t] = acc;
}
int main() {
  int dev; cudaGetDevice(&dev); cudaDeviceProp p; cudaGetDeviceProperties(&p, dev); int clk = 0; cudaDeviceGetAttribute(&clk, cudaDevAttrClockRate, dev);
  const int NB = p.multiProcessorCount * 8, BS = 256;
  double* out; cudaMalloc(&out, sizeof(double) * NB * BS);
  cudaEvent_t a, b; cudaEventCreate(&a); cudaEventCreate(&b);
  auto run = [&](const char* name, void (*k)(double*, int), int iters, double ops_per_iter) {
    k<<<NB, BS>>>(out, 10); cudaDeviceSynchronize();
    cudaEventRecord(a); k<<<NB, BS>>>(out, iters); cudaEventRecord(b); cudaEventSynchronize(b);
    float ms; cudaEventElapsedTime(&ms, a, b);
    double ops = (double)NB * BS * iters * ops_per_iter;
    printf("%s: %.3f ms, %.3f Gop/s (%.2f op/clk/SM at %d MHz)\n", name, ms, ops / ms * 1e-6,
           ops / (ms * 1e-3) / p.multiProcessorCount / (clk * 1e3), clk / 1000);
  };
  printf("%s, %d SMs\n", p.name, p.multiProcessorCount);
  run("dfma (8 chains)", dfma, 2000, 8);
  run("ffma (8 chains)", ffma, 20000, 8);
  run("dlog", dlog, 2000, 1);
  run("ddiv", ddiv, 2000, 1);
  cudaError_t e = cudaGetLastError();
  printf("status: %s\n", cudaGetErrorString(e));
  return e == cudaSuccess ? 0 : 1;
}
