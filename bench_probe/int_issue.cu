// int_issue.cu -- integer-issue throughput probe of the benchmark (not part
// of the engine library): bench.py loads it as bench_probe/_build/libintissue.so.
//
// The sweeps are bound by the SM's integer pipes (no memory or tensor-core
// work in the inner loop), so their roofline denominator is the rate at
// which the SMs can retire 32-bit integer lane operations.  This kernel
// measures it on the device it runs on: independent chains of LOP3
// (ALU pipe) interleaved with IMAD (FMA pipe) lane operations, the two
// integer pipes the sweep kernels use.  Inline PTX keeps the compiler from
// folding the chains.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>

namespace {

constexpr int kProbeIters = 2048;

// MODE 0: LOP3 only (ALU pipe), 1: IMAD only (FMA pipe), 2: LOP3 and IMAD
// alternating (both integer pipes).  The mode is a template parameter so
// that every mode compiles to straight chains of its own instructions.
template <int MODE>
__global__ void __launch_bounds__(256) int_issue_probe(uint32_t* out, uint32_t k) {
  uint32_t a[8];
  const uint32_t k2 = k * 3u + 1u;
#pragma unroll
  for (int i = 0; i < 8; ++i) a[i] = k * (threadIdx.x + 1) + i;
  // eight independent chains per thread: each instruction depends only on
  // its own chain's previous result
  for (int it = 0; it < kProbeIters; ++it) {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      if (MODE == 0 || (MODE == 2 && (i & 1) == 0))
        asm volatile("lop3.b32 %0, %0, %1, %2, 0x96;" : "+r"(a[i]) : "r"(k), "r"(k2));
      else
        asm volatile("mad.lo.u32 %0, %0, %1, %2;" : "+r"(a[i]) : "r"(k), "r"(k2));
    }
  }
  uint32_t s = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) s ^= a[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

extern "C" {

// lane_ops_per_s[0] = LOP3 only (ALU pipe), [1] = IMAD only (FMA pipe),
// [2] = alternating LOP3 / IMAD (both integer pipes).  Returns 0, or 1 for a
// null argument, 2 for a CUDA error (message on stderr).
__attribute__((visibility("default"))) int probe_int_issue(int device, double* lane_ops_per_s) {
  if (!lane_ops_per_s) return 1;
  cudaError_t e = cudaSetDevice(device);
  int nsm = 0;
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
  const int blocks = nsm * 8, threads = 256;
  uint32_t* buf = nullptr;
  if (e == cudaSuccess) e = cudaMalloc(&buf, (size_t)blocks * threads * sizeof(uint32_t));
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  for (int mode = 0; mode < 3 && e == cudaSuccess; ++mode) {
    float best = 1e30f;
    for (int rep = 0; rep < 3 && e == cudaSuccess; ++rep) {
      cudaEventRecord(e0);
      const uint32_t k = 0x9E3779B9u + rep;
      if (mode == 0) int_issue_probe<0><<<blocks, threads>>>(buf, k);
      else if (mode == 1) int_issue_probe<1><<<blocks, threads>>>(buf, k);
      else int_issue_probe<2><<<blocks, threads>>>(buf, k);
      cudaEventRecord(e1);
      e = cudaEventSynchronize(e1);
      float ms = 0.f;
      if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
      if (ms < best) best = ms;
    }
    lane_ops_per_s[mode] = (double)blocks * threads * kProbeIters * 8 / (best * 1e-3);
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (buf) cudaFree(buf);
  if (e != cudaSuccess) {
    std::fprintf(stderr, "int issue probe: %s\n", cudaGetErrorString(e));
    return 2;
  }
  return 0;
}

}  // extern "C"
