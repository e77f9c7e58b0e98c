// Binary64 issue-rate probe: the denominator of the FP64 roofline, and the measurement behind
// the codelets' fused forms (a*1 + b for a + b, a*b + (-0) for a*b).
//
//   nvcc -gencode arch=compute_103a,code=sm_103a -O3 fp64_issue_probe.cu -o fp64_issue_probe
//   ./fp64_issue_probe
//
// 8 CTAs of 256 threads per SM, 8 independent dependency chains per thread, 4096 iterations,
// CUDA events over 5 launches after one warm-up.  The operands 1.0, -0.0, the addend and the
// multiplier are read from device memory, so the compiler cannot fold a fused form back into
// an add or a multiply.
#include <cstdio>
#include <cuda_runtime.h>
#define CH 8
template <int OP>
__global__ void __launch_bounds__(256) k(double* out, const double* p, int iters) {
  const double one = p[0], c = p[1], m = p[2], nz = p[3];
  double x[CH];
#pragma unroll
  for (int i = 0; i < CH; ++i) x[i] = (double)(threadIdx.x + i) * 1e-3;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < CH; ++i) {
      if (OP == 0) x[i] = __dadd_rn(x[i], c);
      if (OP == 1) x[i] = __fma_rn(x[i], one, c);     // = x + c exactly
      if (OP == 2) x[i] = __fma_rn(x[i], m, c);       // a genuine FMA
      if (OP == 3) x[i] = __dmul_rn(x[i], m);
      if (OP == 4) x[i] = __fma_rn(x[i], m, nz);      // = x * m exactly
      if (OP == 5) x[i] = (i & 1) ? __fma_rn(x[i], one, c) : __fma_rn(x[i], m, c);
    }
  }
  double s = 0;
#pragma unroll
  for (int i = 0; i < CH; ++i) s += x[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
template <int OP>
float run(double* out, const double* p, int grid, int iters) {
  cudaEvent_t a, b; cudaEventCreate(&a); cudaEventCreate(&b);
  k<OP><<<grid, 256>>>(out, p, iters);
  cudaEventRecord(a);
  for (int r = 0; r < 5; ++r) k<OP><<<grid, 256>>>(out, p, iters);
  cudaEventRecord(b); cudaEventSynchronize(b);
  float ms; cudaEventElapsedTime(&ms, a, b);
  return ms / 5;
}
int main() {
  int sms = 0; cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
  const int grid = sms * 8, iters = 4096;
  double *out, *p; cudaMalloc(&out, (size_t)grid * 256 * sizeof(double)); cudaMalloc(&p, 4 * sizeof(double));
  const double h[4] = {1.0, 1e-9, 1.0000001, -0.0};
  cudaMemcpy(p, h, sizeof h, cudaMemcpyHostToDevice);
  const double ops = (double)grid * 256 * CH * iters;
  const char* names[6] = {"DADD", "DFMA(x, one=1.0 runtime, c)", "DFMA(x, m, c)", "DMUL", "DFMA(x, m, nz=-0.0 runtime)", "DFMA one/m interleaved"};
  float t[6] = {run<0>(out, p, grid, iters), run<1>(out, p, grid, iters), run<2>(out, p, grid, iters),
                run<3>(out, p, grid, iters), run<4>(out, p, grid, iters), run<5>(out, p, grid, iters)};
  for (int i = 0; i < 6; ++i) printf("%-32s %.3f ms  %.4f T instr/s\n", names[i], t[i], ops / (t[i] * 1e-3) / 1e12);
  printf("status: %s\n", cudaGetErrorString(cudaGetLastError()));
  return 0;
}
