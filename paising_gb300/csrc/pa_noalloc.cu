// pa_noalloc.cu -- pa_resample_plan_noalloc: the resampling plan (Q, lnQ,
// copy numbers, exclusive scan, gather map) for callers that cannot allocate
// device memory.
//
// pa_resample_plan allocates its scratch (the population descriptor and the
// per-block partial sums) with cudaMalloc on every call.  Some callers cannot
// do that: a framework that has reserved the device's memory for its own
// allocator leaves nothing for out-of-band cudaMalloc, and a latency-critical
// loop cannot afford the device-wide synchronisation cudaFree implies.  This
// variant runs the same kernels with the same launch shapes, but its scratch
// is the file-scope device array g_plan_scratch (kNoAllocScratchBytes, held
// by every GPU that loads the library until the process exits).  It calls no
// cudaMalloc, cudaFree or allocating library routine; the caller still
// passes every input and output buffer.
//
// Contract: at most kNoAllocMaxUnits replica slots (SSC: R_prev; MSC:
// 32 * ceil(R_prev / 32)); larger inputs are rejected with PA_ERR_ARG.  Every
// call shares the one array and leaves its contents behind, so calls whose
// GPU work overlaps (other streams, other host threads) race with each other.
// Every call looks up the array's device address on the current device
// (cudaGetSymbolAddress, which allocates nothing), so the address stays right
// after cudaDeviceReset re-creates the context.  The first call on a device
// may load the library's device code (lazy module loading): make that first
// call before any stream capture.
#include <cuda_runtime.h>

#include <cstring>
#include <string>

#include "../../include/paising.h"
#include "pa_device.cuh"
#include "pa_error.h"
#include "pa_kernels.h"

using namespace pa;

namespace {

constexpr size_t kNoAllocScratchBytes = 32768;
constexpr long long kNoAllocMaxUnits = (long long)kResBlocksMax * 256;

// layout of the scratch array
constexpr size_t kOffState = 0;
constexpr size_t kOffBetas = 1024;
constexpr size_t kOffBlkTot = kOffBetas + 256;
constexpr size_t kOffBlkOff = kOffBlkTot + sizeof(uint32_t) * kResBlocksMax;
constexpr size_t kOffQd = kOffBlkOff + sizeof(uint32_t) * kResBlocksMax;
constexpr size_t kOffQf = kOffQd + sizeof(double) * kResBlocksMax;
constexpr size_t kOffEnd = kOffQf + 2 * sizeof(float) * kResBlocksMax;
static_assert(sizeof(PopDev) <= kOffBetas, "descriptor does not fit its slot");
static_assert(kOffEnd <= kNoAllocScratchBytes, "scratch layout exceeds the array");

static __device__ __align__(256) unsigned char g_plan_scratch[kNoAllocScratchBytes];

// Writes the call's descriptor and inverse temperatures into the scratch
// array; the descriptor's ticket and error fields start at zero.
__global__ void noalloc_setup_kernel(PopDev h, double beta_prev, double beta) {
  *reinterpret_cast<PopDev*>(g_plan_scratch + kOffState) = h;
  double* b = reinterpret_cast<double*>(g_plan_scratch + kOffBetas);
  b[0] = beta_prev;
  b[1] = beta;
}

int fail(int code, const std::string& m) {
  pa::g_last_error = "pa_resample_plan_noalloc: " + m;
  return code;
}

}  // namespace

extern "C" {

int pa_resample_plan_noalloc(const int32_t* E, const uint8_t* active, int coding, int R_prev, int Rinit, int Rcap,
                             double beta_prev, double beta, double e_ref, int weights, uint64_t seed, uint64_t iseq,
                             uint32_t* roff, uint32_t* offs, uint32_t* src, double* out, void* stream) {
  if (!E || !roff || !offs || !src || !out || R_prev < 1 || Rinit < 1 || Rcap < 1)
    return fail(PA_ERR_ARG, "null buffer or non-positive size");
  if (coding != PA_CODING_SSC && coding != PA_CODING_MSC) return fail(PA_ERR_ARG, "bad coding");
  if (coding == PA_CODING_MSC && !active) return fail(PA_ERR_ARG, "MSC needs the active flags");
  if (weights != PA_WEIGHTS_FP32 && weights != PA_WEIGHTS_FP64) return fail(PA_ERR_ARG, "bad weights");
  const long long units = coding == PA_CODING_MSC ? ((long long)R_prev + kMsb - 1) / kMsb * kMsb : R_prev;
  if (units > kNoAllocMaxUnits)
    return fail(PA_ERR_ARG, "population of " + std::to_string(units) + " replica slots exceeds the maximum of " +
                                std::to_string(kNoAllocMaxUnits) + " supported without allocation");
  cudaStream_t s = (cudaStream_t)stream;
  // the array's address on the current device; the host-side symbol
  // g_plan_scratch is a stand-in, never a device address
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_plan_scratch);
  if (e != cudaSuccess) return fail(PA_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
  unsigned char* base = static_cast<unsigned char*>(p);

  PopDev h;
  std::memset(&h, 0, sizeof(h));
  h.coding = coding;
  h.L = 8;
  h.N = 64;
  h.step = 1;
  h.nsteps = 1;
  h.Rinit = Rinit;
  h.Rcap = Rcap;
  h.rgcap = (int)(((long long)Rcap + kMsb - 1) / kMsb);
  h.R_prev = R_prev;
  h.R_cur = R_prev;
  h.weights = weights;
  h.seed = seed;
  h.iseq = iseq;
  h.Emean = e_ref;
  h.Emin = (int)e_ref;
  h.E = const_cast<int32_t*>(E);
  h.active[0] = h.active[1] = const_cast<uint8_t*>(active);
  h.roff = roff;
  h.offs = offs;
  h.src = src;
  h.blk_tot = reinterpret_cast<uint32_t*>(base + kOffBlkTot);
  h.blk_off = reinterpret_cast<uint32_t*>(base + kOffBlkOff);
  h.qpart_d = reinterpret_cast<double*>(base + kOffQd);
  h.qpart_f = reinterpret_cast<float*>(base + kOffQf);
  h.betas = reinterpret_cast<double*>(base + kOffBetas);
  PopDev* st = reinterpret_cast<PopDev*>(base + kOffState);

  const int blocks = res_blocks(units);
  noalloc_setup_kernel<<<1, 1, 0, s>>>(h, beta_prev, beta);
  if ((e = cudaGetLastError()) != cudaSuccess) return fail(PA_ERR_CUDA, cudaGetErrorString(e));
  if ((e = launch_q(st, 1, blocks, s)) != cudaSuccess) return fail(PA_ERR_CUDA, cudaGetErrorString(e));
  if ((e = launch_copy_numbers(st, 1, blocks, s)) != cudaSuccess) return fail(PA_ERR_CUDA, cudaGetErrorString(e));
  if ((e = launch_scatter(st, 1, blocks, s)) != cudaSuccess) return fail(PA_ERR_CUDA, cudaGetErrorString(e));
  PopDev back;
  if ((e = cudaMemcpyAsync(&back, st, sizeof(PopDev), cudaMemcpyDeviceToHost, s)) != cudaSuccess)
    return fail(PA_ERR_CUDA, cudaGetErrorString(e));
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return fail(PA_ERR_CUDA, cudaGetErrorString(e));
  out[0] = back.lnQ;
  out[1] = back.q;
  out[2] = back.error ? 0.0 : (double)back.R_cur;
  if (back.error == 1) return fail(PA_ERR_CAPACITY, "new population exceeds Rcap");
  if (back.error == 2) return fail(PA_ERR_EXTINCT, "population became empty");
  return PA_OK;
}

}  // extern "C"
