/*
 * inj_shim.cuh -- force-included (nvcc -include) into the injected-stream
 * build of the reference programs PAisingSSC.cu / PAisingMSC.cu.
 *
 * TEST INFRASTRUCTURE ONLY (oracle).  It replaces the reference's RNG state
 * type  curandStatePhilox4_32_10_t  (typedef'd to RNGState at
 * PAisingSSC.cu:33, PAisingMSC.cu:32) by InjState, whose curand_init / curand
 * / curand_uniform_double overloads draw from the pure function inj_H of
 * inj_stream.h.  Draw order, subsequence numbering and every other line of the
 * reference stay as written, so the reference's own kernels consume
 *     H(seed, subsequence, 0), H(seed, subsequence, 1), ...
 * per thread, exactly like cuRAND's sequential stream would be consumed.
 *
 * curand_kernel.h is included first so that its include guard makes the
 * reference's own #include a no-op and the macro below renames only the
 * reference's use of the type.
 */
#ifndef PAISING_ORACLE_INJ_SHIM_CUH
#define PAISING_ORACLE_INJ_SHIM_CUH

#include <curand_kernel.h>
#include "inj_stream.h"

struct InjState {
    unsigned long long seed;
    unsigned long long subseq;
    unsigned long long ctr;
};

__host__ __device__ inline void curand_init(unsigned long long seed,
                                            unsigned long long subsequence,
                                            unsigned long long offset,
                                            InjState* s) {
    s->seed = seed;
    s->subseq = subsequence;
    s->ctr = offset;
}

__device__ inline unsigned int curand(InjState* s) {
    return inj_H(s->seed, s->subseq, s->ctr++);
}

__device__ inline double curand_uniform_double(InjState* s) {
    return inj_uniform_double(inj_H(s->seed, s->subseq, s->ctr++));
}

#define curandStatePhilox4_32_10_t InjState

#endif
