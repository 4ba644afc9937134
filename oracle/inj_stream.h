/*
 * inj_stream.h -- the injected ("test mode") random stream, oracle side.
 *
 * TEST INFRASTRUCTURE ONLY.  This header is part of the oracle: it is used by
 * the CPU restatement (oracle/pa_oracle.c) and by the injected-stream build of
 * the reference programs (oracle/inj_shim.cuh).  The product library carries
 * its own Philox implementation (paising_gb300/csrc/philox.cuh); the tests
 * check that the two agree word for word.
 *
 * The reference draws every random number from cuRAND's Philox4_32_10 device
 * generator, initialised per thread as curand_init(seed, subsequence, 0)
 * (PAisingSSC.cu:152,164,241; PAisingMSC.cu:171,195,355) and consumed
 * sequentially (curand / curand_uniform_double).  cuRAND's own stream is not
 * pinned by anything in the reference, so bit-exact comparisons replace it by
 * a pure function
 *
 *     H(seed, subsequence, ctr) -> uint32
 *
 * evaluated at the same (subsequence, ctr) coordinates by both sides.  H is
 * the Philox4x32-10 counter-based generator of Salmon, Moraes, Dror and Shaw,
 * "Parallel random numbers: as easy as 1, 2, 3" (SC'11), restated from the
 * paper:
 *     key     = (lo32(seed), hi32(seed))
 *     counter = (lo32(ctr >> 2), hi32(ctr >> 2), lo32(subseq), hi32(subseq))
 *     H       = word (ctr & 3) of Philox4x32-10(key, counter)
 * A uniform double is (H + 1) * 2^-32, in (0, 1].
 */
#ifndef PAISING_ORACLE_INJ_STREAM_H
#define PAISING_ORACLE_INJ_STREAM_H

#include <stdint.h>

#ifdef __CUDACC__
#define INJ_HD __host__ __device__ __forceinline__
#else
#define INJ_HD static inline
#endif

/* Philox4x32 round constants (Salmon et al. 2011, table 2 / section 5). */
#define INJ_PHILOX_M0 0xD2511F53u
#define INJ_PHILOX_M1 0xCD9E8D57u
#define INJ_PHILOX_W0 0x9E3779B9u
#define INJ_PHILOX_W1 0xBB67AE85u

INJ_HD void inj_philox4x32_10(const uint32_t key_in[2], const uint32_t ctr_in[4],
                              uint32_t out[4]) {
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; ++r) {
        if (r) { k0 += INJ_PHILOX_W0; k1 += INJ_PHILOX_W1; }
        uint64_t p0 = (uint64_t)INJ_PHILOX_M0 * c0;
        uint64_t p1 = (uint64_t)INJ_PHILOX_M1 * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

INJ_HD uint32_t inj_H(uint64_t seed, uint64_t subseq, uint64_t ctr) {
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint64_t blk = ctr >> 2;
    uint32_t c[4] = {(uint32_t)blk, (uint32_t)(blk >> 32), (uint32_t)subseq,
                     (uint32_t)(subseq >> 32)};
    uint32_t o[4];
    inj_philox4x32_10(key, c, o);
    return o[ctr & 3u];
}

INJ_HD double inj_uniform_double(uint32_t h) {
    return ((double)h + 1.0) * (1.0 / 4294967296.0);
}

#endif /* PAISING_ORACLE_INJ_STREAM_H */
