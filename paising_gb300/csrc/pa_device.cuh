// pa_device.cuh -- device-side building blocks shared by the kernels:
// Philox4x32-10, the reference-coordinate ("injected") stream, warp/block
// reductions and exact 128-bit accumulation helpers.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "pa_kernels.h"
#include "pa_state.h"

namespace pa {

// ----------------------------------------------------------------- Philox
// Philox4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw,
// "Parallel random numbers: as easy as 1, 2, 3", SC'11), written from the
// paper: two 32x32->64 multiplies per round, Weyl-sequence key schedule.
constexpr uint32_t kPhiloxM0 = 0xD2511F53u;
constexpr uint32_t kPhiloxM1 = 0xCD9E8D57u;
constexpr uint32_t kPhiloxW0 = 0x9E3779B9u;
constexpr uint32_t kPhiloxW1 = 0xBB67AE85u;

struct U4 {
  uint32_t x, y, z, w;
};

__host__ __device__ __forceinline__ uint32_t mulhi32(uint32_t a, uint32_t b) {
#ifdef __CUDA_ARCH__
  return __umulhi(a, b);
#else
  return (uint32_t)(((uint64_t)a * b) >> 32);
#endif
}

__host__ __device__ __forceinline__ U4 philox10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                                 uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t hi0 = mulhi32(kPhiloxM0, c0), lo0 = kPhiloxM0 * c0;
    const uint32_t hi1 = mulhi32(kPhiloxM1, c2), lo1 = kPhiloxM1 * c2;
    c0 = hi1 ^ c1 ^ k0;
    c1 = lo1;
    c2 = hi0 ^ c3 ^ k1;
    c3 = lo0;
    k0 += kPhiloxW0;
    k1 += kPhiloxW1;
  }
  return U4{c0, c1, c2, c3};
}

// Philox4x32-10 with the key schedule k + r*W precomputed (k[2r], k[2r+1] =
// round-r key); same output as philox10.  The SSC bit-plane sweep takes it as
// a __grid_constant__ kernel parameter computed on the host (0.5% faster than
// forming it in the kernel); the MSC sweeps form it from the seed (0.6%
// faster that way).
struct PhiloxKeys {
  uint32_t k[20];
  __host__ __device__ __forceinline__ explicit PhiloxKeys(unsigned long long seed) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
      k[2 * r] = (uint32_t)seed + (uint32_t)r * kPhiloxW0;
      k[2 * r + 1] = (uint32_t)(seed >> 32) + (uint32_t)r * kPhiloxW1;
    }
  }
};

__device__ __forceinline__ U4 philox10k(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, const PhiloxKeys& K) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const unsigned long long p0 = (unsigned long long)kPhiloxM0 * c0;
    const unsigned long long p1 = (unsigned long long)kPhiloxM1 * c2;
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    c0 = hi1 ^ c1 ^ K.k[2 * r];
    c1 = lo1;
    c2 = hi0 ^ c3 ^ K.k[2 * r + 1];
    c3 = lo0;
  }
  return U4{c0, c1, c2, c3};
}

// The same generator with each round's two products written as PTX
// mul.wide.u32.  Same output; which form the compiler schedules better
// depends on the kernel around it (measured, 8 populations at L=64: the SSC
// bit-plane sweep 1.7% faster this way, the MSC sweep 1.2% slower), so a
// kernel chooses by the type of its keys.
struct PhiloxKeysWide : PhiloxKeys {
  __host__ __device__ __forceinline__ explicit PhiloxKeysWide(unsigned long long seed) : PhiloxKeys(seed) {}
};

__device__ __forceinline__ unsigned long long mul_wide_u32(uint32_t a, uint32_t b) {
  unsigned long long p;
  asm("mul.wide.u32 %0, %1, %2;" : "=l"(p) : "r"(a), "r"(b));
  return p;
}

__device__ __forceinline__ U4 philox10k(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, const PhiloxKeysWide& K) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const unsigned long long p0 = mul_wide_u32(c0, kPhiloxM0);
    const unsigned long long p1 = mul_wide_u32(c2, kPhiloxM1);
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    c0 = hi1 ^ c1 ^ K.k[2 * r];
    c1 = lo1;
    c2 = hi0 ^ c3 ^ K.k[2 * r + 1];
    c3 = lo0;
  }
  return U4{c0, c1, c2, c3};
}

// The reference draws every random number from a per-thread cuRAND stream
// initialised as curand_init(seed, subsequence, 0) and consumed in order
// (PAisingSSC.cu:152,164,241; PAisingMSC.cu:171,195,355).  "Reference
// coordinates" mode evaluates, for draw number ctr of subsequence subseq,
//   H = word (ctr & 3) of Philox4x32-10(key = seed, counter = (ctr >> 2, subseq))
// so that a kernel with any thread layout can reproduce the draw a reference
// thread would have made.  A uniform double is (H + 1) * 2^-32.
__host__ __device__ __forceinline__ uint32_t ref_word(uint64_t seed, uint64_t subseq, uint64_t ctr) {
  const uint64_t blk = ctr >> 2;
  const U4 o = philox10((uint32_t)blk, (uint32_t)(blk >> 32), (uint32_t)subseq, (uint32_t)(subseq >> 32),
                        (uint32_t)seed, (uint32_t)(seed >> 32));
  const uint32_t j = (uint32_t)ctr & 3u;
  return j == 0 ? o.x : j == 1 ? o.y : j == 2 ? o.z : o.w;
}

__host__ __device__ __forceinline__ double ref_uniform(uint32_t h) {
  return ((double)h + 1.0) * (1.0 / 4294967296.0);
}

// Domain tags for the native sweep streams (counter word 3, top byte).
constexpr uint32_t kTagSscSweep = 0x53u << 24;
constexpr uint32_t kTagMscSweep = 0x4Du << 24;

// Counter word 2 of the native sweep streams: the temperature index (below
// 2^14, since schedules end at nBmax = 10000) and, above it, the population's
// run number, so that repeated runs of a handle draw fresh sweep randomness
// (runs 2^18 apart share it).
__device__ __forceinline__ uint32_t native_step_word(const PopDev* st) {
  return (uint32_t)st->step | ((uint32_t)st->run << 14);
}

// -------------------------------------------------------------- reductions
template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <class T>
__device__ __forceinline__ T warp_min(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    T w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w < v ? w : v;
  }
  return v;
}

// Block-wide sum; every thread must call it; result valid in all threads.
// scratch: >= 32 elements of shared memory.
template <class T>
__device__ __forceinline__ T block_sum(T v, T* scratch) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) scratch[wid] = v;
  __syncthreads();
  v = (lane < nw) ? scratch[lane] : T(0);
  v = warp_sum(v);
  return v;
}

// Block-wide exclusive scan of one uint32 per thread (blockDim multiple of 32,
// <= 1024).  Returns the exclusive prefix; *total receives the block total.
__device__ __forceinline__ uint32_t block_exscan(uint32_t v, uint32_t* scratch, uint32_t* total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  uint32_t inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  __syncthreads();
  if (lane == 31) scratch[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    uint32_t w = lane < nw ? scratch[lane] : 0u, wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t t = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += t;
    }
    if (lane < nw) scratch[lane] = wi - w;
    if (lane == nw - 1) scratch[32] = wi;
  }
  __syncthreads();
  uint32_t ex = scratch[wid] + inc - v;
  *total = scratch[32];
  return ex;
}

// ------------------------------------------------ exact 128-bit accumulation
// Sums of M^4 exceed 64 bits (|M| <= N, N up to 65536).  They are kept as
// (lo, hi) pairs of uint64 and added with carry, so the total does not depend
// on the order in which replicas are accumulated.
struct U128 {
  unsigned long long lo, hi;
};

__device__ __forceinline__ void u128_add(U128& a, unsigned long long lo, unsigned long long hi) {
  const unsigned long long s = a.lo + lo;
  a.hi += hi + (s < a.lo ? 1ull : 0ull);
  a.lo = s;
}

__device__ __forceinline__ void u128_atomic_add(unsigned long long* lo_p, unsigned long long* hi_p,
                                                unsigned long long lo, unsigned long long hi) {
  const unsigned long long old = atomicAdd(lo_p, lo);
  const unsigned long long carry = (old + lo < old) ? 1ull : 0ull;
  if (hi + carry) atomicAdd(hi_p, hi + carry);
}

// m^4 for |m| <= 65536 as (lo, hi)
__device__ __forceinline__ void m4_of(int m, unsigned long long& lo, unsigned long long& hi) {
  const unsigned long long m2 = (unsigned long long)((long long)m * (long long)m);
  lo = m2 * m2;
  hi = __umul64hi(m2, m2);
}

__host__ __device__ __forceinline__ double u128_to_double(unsigned long long lo, unsigned long long hi) {
  return (double)hi * 18446744073709551616.0 + (double)lo;
}

// --------------------------------------------------------- batch work queue
// Population p and its local unit for queue entry u: prefix[p] <= u < prefix[p+1].
__device__ __forceinline__ int queue_pop(const BatchDev* b, int u, int* local) {
  int lo = 0, hi = b->npop;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (b->unit_prefix[mid] <= u) lo = mid;
    else hi = mid;
  }
  *local = u - b->unit_prefix[lo];
  return lo;
}

// Persistent grid: as many CTAs of `block` threads as can be resident.
inline cudaError_t persistent_launch(const void* fn, int block, int smem, SweepLaunch* out) {
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  int dev, nsm, per = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, block, smem)) != cudaSuccess) return e;
  out->grid = nsm * (per > 0 ? per : 1);
  out->block = block;
  out->smem = smem;
  return cudaSuccess;
}

}  // namespace pa
