/*
 * pa_oracle.c -- CPU restatement of the reference's population-annealing path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links or calls
 * this file; it is built into oracle/_build/libpaoracle.so and used by the
 * tests, by __graft_entry__.smoke() to verify the engine's results, and by
 * bench.py's cpu_baseline leg.
 *
 * It restates, stage by stage and in the reference's own draw order, the two
 * reference programs:
 *   SSC = PAisingSSC.cu (one int8 spin per site, one replica per CUDA block)
 *   MSC = PAisingMSC.cu (32 replicas bit-packed per 32-bit word)
 * with cuRAND's Philox stream replaced by the injected stream H of
 * inj_stream.h (same (subsequence, counter) coordinates).  Lattice size L is a
 * runtime argument here; in the reference it is the compile-time #define at
 * PAisingSSC.cu:27 / PAisingMSC.cu:26.  MSbits is fixed at 32
 * (PAisingMSC.cu:34).
 *
 * Storage (oracle-internal, mirrors the reference structs):
 *   SSC  spins[r*N + i]        i <  N/2 : gA[i], i >= N/2 : gB[i-N/2], int8 +-1
 *        (struct Replica, PAisingSSC.cu:70-77)
 *   MSC  words[g*N + i]        same split, uint32 bit k = replica k of group g
 *        (struct Replica, PAisingMSC.cu:84-92); IE/M/Roff/isActive as
 *        separate arrays indexed g*32 + k.
 *
 * Compile with -ffp-contract=off so that no multiply-add is fused: the result
 * then does not depend on the host architecture.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "inj_stream.h"

#define EQT 128      /* EQthreads, PAisingSSC.cu:62 */
#define NT 1024      /* Nthreads,  PAisingSSC.cu:63 */
#define MSB 32       /* MSbits,    PAisingMSC.cu:34 */
#define LCG_A 1664525u      /* PAisingMSC.cu:53 */
#define LCG_C 1013904223u   /* PAisingMSC.cu:54 */

int or_version(void) { return 1; }

void or_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int or_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

uint32_t or_H(uint64_t seed, uint64_t subseq, uint64_t ctr) { return inj_H(seed, subseq, ctr); }

void or_philox(const uint32_t key[2], const uint32_t ctr[4], uint32_t out[4]) {
    inj_philox4x32_10(key, ctr, out);
}

/* ---------------------------------------------------------------- geometry */
/* Checkerboard neighbours, PAisingSSC.cu:169-172 (A sites) and 181-184 (B
 * sites): idx = ty*L/2 + tx; i1 is the horizontal neighbour that is not at the
 * same idx, i3 the row below, i4 the row above. */
static inline void nbr(int L, int idx, int subl, int* i1, int* i3, int* i4) {
    int h = L / 2, ty = idx / h, tx = idx - ty * h;
    int right_odd = (subl == 0) ? (ty & 1) : !(ty & 1);
    *i1 = ty * h + (right_odd ? (tx + 1) : (tx + h - 1)) % h;
    *i3 = ((ty + L - 1) % L) * h + tx;
    *i4 = ((ty + 1) % L) * h + tx;
}

/* number of idx = t, t+128, ... below N/2 (the per-thread loop count of the
 * reference's `for (idx = t; idx < N/2; idx += EQthreads)`) */
static inline int kt_count(int half_n, int t) { return t < half_n ? (half_n - t + EQT - 1) / EQT : 0; }

/* ------------------------------------------------ reference block reduction */
/* blockReduceSum<double> for a 1024-thread block (PAisingSSC.cu:107-124):
 * __shfl_down tree inside each warp, then the same tree over the 32 warp
 * sums.  v has 1024 entries (zero padded). */
static double warp_tree(const double* v) {
    double a[32];
    for (int i = 0; i < 32; ++i) a[i] = v[i];
    for (int off = 16; off > 0; off >>= 1)
        for (int i = 0; i < off; ++i) a[i] = a[i] + a[i + off];
    return a[0];
}

static double block_tree_1024(const double* v) {
    double w[32];
    for (int k = 0; k < 32; ++k) w[k] = warp_tree(v + 32 * k);
    return warp_tree(w);
}

/* QKer second part (PAisingSSC.cu:225-233): partial sums p[0..nb) reduced in
 * chunks of 1024 with the block tree, accumulated serially. */
static double reduce_partials(const double* p, int nb) {
    double acc = 0.0, buf[NT];
    for (int j = 0; j < nb; j += NT) {
        for (int t = 0; t < NT; ++t) buf[t] = (j + t < nb) ? p[j + t] : 0.0;
        acc += block_tree_1024(buf);
    }
    return acc;
}

/* ====================================================================== SSC */

/* ReplicaInit, PAisingSSC.cu:150-157 */
void or_ssc_init(int8_t* spins, int L, int R, uint64_t seed, uint64_t iseq) {
    int N = L * L, h = N / 2;
#pragma omp parallel for schedule(static)
    for (int B = 0; B < R; ++B) {
        int8_t* g = spins + (size_t)B * N;
        for (int idx = 0; idx < h; ++idx) {
            int t = idx % EQT, k = idx / EQT;
            uint64_t sub = iseq + (uint64_t)t + (uint64_t)EQT * B;
            g[idx] = inj_uniform_double(inj_H(seed, sub, 2ull * k)) >= 0.5 ? 1 : -1;
            g[h + idx] = inj_uniform_double(inj_H(seed, sub, 2ull * k + 1)) >= 0.5 ? 1 : -1;
        }
    }
}

/* Boltzmann table, PAisingSSC.cu:512-516 */
void or_ssc_boltz(double beta, double tab[10]) {
    for (int i0 = 0; i0 <= 1; ++i0)
        for (int i1 = 0; i1 <= 4; ++i1) {
            double e = exp(-2 * (2 * i0 - 1) * (2 * i1 - 4) * beta);
            tab[i0 + 2 * i1] = e < 1.0 ? e : 1.0;
        }
}

/* checkKerALL, PAisingSSC.cu:159-193 */
void or_ssc_sweep(int8_t* spins, int L, int R, int sweeps, const double tab[10], uint64_t seed,
                  uint64_t iseq) {
    int N = L * L, h = N / 2;
#pragma omp parallel for schedule(static)
    for (int B = 0; B < R; ++B) {
        int8_t* gA = spins + (size_t)B * N;
        int8_t* gB = gA + h;
        for (int sw = 0; sw < sweeps; ++sw)
            for (int half = 0; half < 2; ++half) {
                int8_t* s = half ? gB : gA;
                const int8_t* o = half ? gA : gB;
                for (int idx = 0; idx < h; ++idx) {
                    int t = idx % EQT, k = idx / EQT, K = kt_count(h, t);
                    int i1, i3, i4;
                    nbr(L, idx, half, &i1, &i3, &i4);
                    int spin = s[idx];
                    int t0 = (1 + spin) / 2;
                    int t1 = (4 + o[i1] + o[idx] + o[i3] + o[i4]) / 2;
                    uint64_t sub = iseq + (uint64_t)t + (uint64_t)EQT * B;
                    uint64_t ctr = (uint64_t)sw * 2 * K + (uint64_t)half * K + k;
                    if (inj_uniform_double(inj_H(seed, sub, ctr)) < tab[t0 + 2 * t1]) s[idx] = (int8_t)-spin;
                }
            }
    }
}

/* energyKer, PAisingSSC.cu:195-215: left and up bond of every site */
void or_ssc_energy(const int8_t* spins, int L, int R, int32_t* E, int32_t* M) {
    int N = L * L, h = N / 2, hw = L / 2;
#pragma omp parallel for schedule(static)
    for (int B = 0; B < R; ++B) {
        const int8_t* gA = spins + (size_t)B * N;
        const int8_t* gB = gA + h;
        int e = 0, m = 0;
        for (int idx = 0; idx < h; ++idx) {
            int sA = gA[idx], sB = gB[idx], ty = idx / hw, tx = idx - ty * hw;
            int iL = ty * hw + (tx + hw - 1) % hw, iU = ((ty + 1) % L) * hw + tx;
            int Ai2, Bi2;
            if (ty & 1) { Ai2 = sB; Bi2 = gA[iL]; }
            else { Ai2 = gB[iL]; Bi2 = sA; }
            int Ai4 = gB[iU], Bi4 = gA[iU];
            e += -sA * (Ai2 + Ai4) - sB * (Bi2 + Bi4);
            m += sA + sB;
        }
        E[B] = e;
        M[B] = m;
    }
}

/* QKer (PAisingSSC.cu:217-234) in the reference's reduction order:
 * q = sum_i exp(-dB (E_i - Emean)). */
double or_ssc_q(const int32_t* E, int R, double dB, double Emean) {
    int nb = (R + NT - 1) / NT;
    double* part = (double*)malloc(sizeof(double) * (nb ? nb : 1));
    double buf[NT];
    for (int b = 0; b < nb; ++b) {
        for (int t = 0; t < NT; ++t) {
            int idx = t + NT * b;
            buf[t] = (idx < R) ? exp(-dB * (E[idx] - Emean)) : 0.0;
        }
        part[b] = block_tree_1024(buf);
    }
    double q = reduce_partials(part, nb);
    free(part);
    return q;
}

/* nearest-integer resampling of one replica, PAisingSSC.cu:242-247 */
static inline uint32_t copies(int Rinit, int R, int32_t IE, double lnQ, double dB, uint32_t u) {
    double mu = ((double)Rinit) / R * exp(-dB * (double)IE - lnQ);
    double fl = floor(mu);
    return (uint32_t)(inj_uniform_double(u) < (mu - fl) ? fl + 1 : fl);
}

/* CalcTauKer, PAisingSSC.cu:236-254; returns the new population size */
uint32_t or_ssc_copy_numbers(const int32_t* E, int R, int Rinit, double lnQ, double dB, uint64_t seed,
                             uint64_t iseq, uint32_t* roff) {
    uint64_t tot = 0;
#pragma omp parallel for reduction(+ : tot) schedule(static)
    for (int idx = 0; idx < R; ++idx) {
        roff[idx] = copies(Rinit, R, E[idx], lnQ, dB, inj_H(seed, iseq + (uint64_t)idx, 0));
        tot += roff[idx];
    }
    return (uint32_t)tot;
}

/* CalcParSum (PAisingSSC.cu:256-270; PAisingMSC.cu:362-395): exclusive scan */
uint32_t or_scan(const uint32_t* roff, int n, uint32_t* offs) {
    uint32_t s = 0;
    for (int i = 0; i < n; ++i) { offs[i] = s; s += roff[i]; }
    return s;
}

/* resampleKer, PAisingSSC.cu:272-280: replica j is copied to slots
 * [offs_j, offs_j + roff_j) of the new population */
void or_ssc_resample(const int8_t* old, int L, int R_old, const uint32_t* roff, const uint32_t* offs,
                     int8_t* neu) {
    size_t N = (size_t)L * L;
#pragma omp parallel for schedule(dynamic, 64)
    for (int j = 0; j < R_old; ++j)
        for (uint32_t p = 0; p < roff[j]; ++p) memcpy(neu + (offs[j] + p) * N, old + (size_t)j * N, N);
}

/* CalcAverages (PAisingSSC.cu:282-292; PAisingMSC.cu:437-450) as exact sums:
 * avg = {sum E, sum E^2, sum |M|, sum M^2, sum M^4} over active replicas.
 * The first four are integers below 2^53 and so equal the reference's FP64
 * atomics in any order; M^4 is summed in long double. */
void or_averages(const int32_t* E, const int32_t* M, const uint8_t* active, int n, double avg[5]) {
    long long se = 0, se2 = 0, sm = 0, sm2 = 0;
    long double sm4 = 0;
    for (int i = 0; i < n; ++i) {
        if (active && !active[i]) continue;
        long long e = E[i], m = M[i] < 0 ? -(long long)M[i] : M[i];
        se += e; se2 += e * e; sm += m; sm2 += m * m;
        sm4 += (long double)(m * m) * (long double)(m * m);
    }
    avg[0] = (double)se; avg[1] = (double)se2; avg[2] = (double)sm; avg[3] = (double)sm2;
    avg[4] = (double)sm4;
}

/* ====================================================================== MSC */

/* ReplicaInit, PAisingMSC.cu:169-188 (MSbits = 32) */
void or_msc_init(uint32_t* words, uint8_t* active, int L, int R, int rg, uint64_t seed, uint64_t iseq) {
    int N = L * L, h = N / 2;
#pragma omp parallel for schedule(static)
    for (int B = 0; B < rg; ++B) {
        uint32_t* g = words + (size_t)B * N;
        for (int idx = 0; idx < h; ++idx) {
            int t = idx % EQT, k = idx / EQT;
            uint64_t sub = iseq + (uint64_t)t + (uint64_t)EQT * B;
            g[idx] = inj_H(seed, sub, 2ull * k);
            g[h + idx] = inj_H(seed, sub, 2ull * k + 1);
        }
        for (int t = 0; t < MSB; ++t) active[B * MSB + t] = (B * MSB + t) < R;
    }
}

/* acceptance thresholds, PAisingMSC.cu:674-675 */
void or_msc_thresholds(double beta, uint32_t thr[2]) {
    thr[0] = (uint32_t)ceil(4294967296. * exp(-4 * beta));
    thr[1] = (uint32_t)ceil(4294967296. * exp(-8 * beta));
}

/* bitsliced count of anti-parallel neighbours, PAisingMSC.cu:207-218 */
static inline void adder(uint32_t I1, uint32_t I2, uint32_t I3, uint32_t I4, uint32_t* s0, uint32_t* s1,
                         uint32_t* s2) {
    uint32_t x12 = I1 ^ I2, x34 = I3 ^ I4, a12 = I1 & I2, a34 = I3 & I4;
    *s0 = x12 ^ x34;
    *s1 = (x12 & x34) ^ a12 ^ a34;
    *s2 = a12 & a34;
}

/* checkKerALL, PAisingMSC.cu:191-266 */
void or_msc_sweep(uint32_t* words, int L, int rg, int sweeps, const uint32_t thr[2], uint64_t seed,
                  uint64_t iseq) {
    int N = L * L, h = N / 2;
#pragma omp parallel for schedule(static)
    for (int B = 0; B < rg; ++B) {
        uint32_t* gA = words + (size_t)B * N;
        uint32_t* gB = gA + h;
        for (int sw = 0; sw < sweeps; ++sw)
            for (int half = 0; half < 2; ++half) {
                uint32_t* s = half ? gB : gA;
                const uint32_t* o = half ? gA : gB;
                for (int idx = 0; idx < h; ++idx) {
                    int t = idx % EQT, k = idx / EQT, K = kt_count(h, t);
                    int i1, i3, i4;
                    nbr(L, idx, half, &i1, &i3, &i4);
                    uint32_t ms = s[idx], s0, s1, s2;
                    adder(ms ^ o[i1], ms ^ o[idx], ms ^ o[i3], ms ^ o[i4], &s0, &s1, &s2);
                    uint64_t sub = iseq + (uint64_t)t + (uint64_t)EQT * B;
                    uint32_t ran = inj_H(seed, sub, (uint64_t)sw * 2 * K + (uint64_t)half * K + k);
                    uint32_t c4 = 0, c8 = 0, im = 1;
                    for (int i = 0; i < MSB; ++i) {
                        if (ran < thr[0]) c4 |= im;
                        if (ran < thr[1]) c8 |= im;
                        im <<= 1;
                        ran = LCG_A * ran + LCG_C;
                    }
                    uint32_t hi = s1 | s2;
                    uint32_t acc = hi | (~hi & ((s0 & c4) | (~s0 & c8)));
                    s[idx] = ms ^ acc;
                }
            }
    }
}

/* energyKer, PAisingMSC.cu:268-317 */
void or_msc_energy(const uint32_t* words, int L, int rg, int32_t* E, int32_t* M) {
    int N = L * L, h = N / 2, hw = L / 2;
#pragma omp parallel for schedule(static)
    for (int B = 0; B < rg; ++B) {
        const uint32_t* gA = words + (size_t)B * N;
        const uint32_t* gB = gA + h;
        int e[MSB], m[MSB];
        for (int i = 0; i < MSB; ++i) e[i] = m[i] = 0;
        for (int idx = 0; idx < h; ++idx) {
            uint32_t sA = gA[idx], sB = gB[idx];
            int ty = idx / hw, tx = idx - ty * hw;
            int iL = ty * hw + (tx + hw - 1) % hw, iU = ((ty + 1) % L) * hw + tx;
            uint32_t Ai2, Bi2;
            if (ty & 1) { Ai2 = sB; Bi2 = gA[iL]; }
            else { Ai2 = gB[iL]; Bi2 = sA; }
            uint32_t Ai4 = gB[iU], Bi4 = gA[iU], s0, s1, s2;
            adder(sA ^ Ai2, sA ^ Ai4, sB ^ Bi2, sB ^ Bi4, &s0, &s1, &s2);
            for (int i = 0; i < MSB; ++i) {
                e[i] += 2 * (int)(((s0 >> i) & 1) + 2 * ((s1 >> i) & 1) + 4 * ((s2 >> i) & 1)) - 4;
                m[i] += 2 * (int)(((sA >> i) & 1) + ((sB >> i) & 1)) - 2;
            }
        }
        for (int i = 0; i < MSB; ++i) { E[B * MSB + i] = e[i]; M[B * MSB + i] = m[i]; }
    }
}

/* QKer, PAisingMSC.cu:319-345: per-group warp tree, then 1024-blocks, then
 * the serial accumulation of block sums */
double or_msc_q(const int32_t* E, const uint8_t* active, int rg, double dB, double Emean) {
    double* g = (double*)malloc(sizeof(double) * rg);
    for (int b = 0; b < rg; ++b) {
        double f[32];
        for (int k = 0; k < MSB; ++k)
            f[k] = active[b * MSB + k] ? exp(-dB * (E[b * MSB + k] - Emean)) : 0.0;
        g[b] = warp_tree(f);
    }
    const int nb = rg > 0 ? (rg + NT - 1) / NT : 0;
    double* part = (double*)malloc(sizeof(double) * (size_t)(nb > 0 ? nb : 1));
    double buf[NT];
    for (int b = 0; b < nb; ++b) {
        for (int t = 0; t < NT; ++t) buf[t] = (t + NT * b < rg) ? g[t + NT * b] : 0.0;
        part[b] = block_tree_1024(buf);
    }
    double q = reduce_partials(part, nb);
    free(g);
    free(part);
    return q;
}

/* CalcTauKer, PAisingMSC.cu:347-360: subsequence iseq + br + 32*idx */
uint32_t or_msc_copy_numbers(const int32_t* E, const uint8_t* active, int rg, int Rinit, int R, double lnQ,
                             double dB, uint64_t seed, uint64_t iseq, uint32_t* roff) {
    uint64_t tot = 0;
#pragma omp parallel for reduction(+ : tot) schedule(static)
    for (int i = 0; i < rg * MSB; ++i) {
        roff[i] = active[i] ? copies(Rinit, R, E[i], lnQ, dB, inj_H(seed, iseq + (uint64_t)i, 0)) : 0;
        tot += roff[i];
    }
    return (uint32_t)tot;
}

/* resampleKer, PAisingMSC.cu:397-435: offspring s of replica (g, k) goes to
 * group s % rg_new, bit s / rg_new.  neu must be zeroed by the caller. */
void or_msc_resample(const uint32_t* old, const int32_t* E_old, int L, int rg_old, const uint32_t* roff,
                     const uint32_t* offs, int rg_new, uint32_t* neu, uint8_t* new_active, int32_t* E_new) {
    int N = L * L;
    for (int i = 0; i < rg_new * MSB; ++i) new_active[i] = 0;
    for (int g = 0; g < rg_old; ++g)
        for (int k = 0; k < MSB; ++k)
            for (uint32_t p = 0; p < roff[g * MSB + k]; ++p) {
                uint32_t s = offs[g * MSB + k] + p, nk = s / rg_new, nj = s % rg_new;
                new_active[nj * MSB + nk] = 1;
                if (E_new) E_new[nj * MSB + nk] = E_old[g * MSB + k];
                const uint32_t* src = old + (size_t)g * N;
                uint32_t* dst = neu + (size_t)nj * N;
                for (int i = 0; i < N; ++i) dst[i] |= ((src[i] >> k) & 1u) << nk;
            }
}

/* ============================================================ full anneal */

/* One full run of the reference's main loop (PAisingSSC.cu:481-692 /
 * PAisingMSC.cu:640-842) for `runs` independent runs.  rows receives, per
 * run, nB rows of the 10 output columns as written to PA_results_run_<r>.dat
 * (beta, E/N, C/N, M/N, M2/N^2, M4/N^4, BF/N, S/N, R, lnQ).  max_steps > 0
 * stops each run after that many temperatures (bounded CPU samples).
 * Returns the number of rows per run, or -1 on error.  *attempts receives
 * sweeps * N * sum_i R_i (the reference's spin-flip count, PAisingSSC.cu:632). */
/* Histogram overlap of inverse-temperature step dB for the current population
 * (CalcOverlap + HistogramOverlap, PAisingSSC.cu:308-334, PAisingMSC.cu:464-500):
 * lnQ from the Q sum around Emean, then the mean of min(1, Rinit/R exp(-dB E - lnQ)). */
static double overlap(int msc, const int32_t* E, const uint8_t* act, int rg, int R, int Rinit, double dB,
                      double Emean) {
    const double q = msc ? or_msc_q(E, act, rg, dB, Emean) : or_ssc_q(E, R, dB, Emean);
    const double lnQ = -dB * Emean + log(q) - log((double)R);
    const int n = msc ? rg * MSB : R;
    double s = 0.0;
    for (int i = 0; i < n; ++i)
        if (!msc || act[i]) s += fmin(1.0, ((double)Rinit) / R * exp(-dB * (double)E[i] - lnQ));
    return s / R;
}

/* Next inverse-temperature step of the AdaptiveStep build (PAisingSSC.cu:644-660):
 * grow the previous step by 1.1x while the overlap is >= MaxOverlap and beta
 * stays below Bfin; otherwise bisect in (0, step) until MinOverlap <= overlap
 * < MaxOverlap (at most 200 halvings; the reference does not bound them);
 * clamp the last step onto Bfin. */
static double next_step(int msc, const int32_t* E, const uint8_t* act, int rg, int R, int Rinit, double Emean,
                        double Bprev, double Bfin, double deltaBeta, double minov, double maxov) {
    double ov, dBmin = 0, dBmax = deltaBeta, dBmean;
    for (;;) {
        ov = overlap(msc, E, act, rg, R, Rinit, dBmax, Emean);
        if (ov >= maxov && Bprev + dBmax < Bfin) dBmax *= 1.1; else break;
    }
    if (ov >= minov) {
        dBmean = dBmax;
    } else {
        for (int it = 0;; ++it) {
            dBmean = 0.5 * (dBmin + dBmax);
            ov = overlap(msc, E, act, rg, R, Rinit, dBmean, Emean);
            if (it + 1 >= 200) break;
            if (ov < minov) dBmax = dBmean;
            else if (ov >= maxov) dBmin = dBmean;
            else break;
        }
    }
    return (Bprev < Bfin && Bprev + dBmean > Bfin) ? Bfin - Bprev : dBmean;
}

/* Family statistics of a population (not written by the reference; the
 * usual equilibration diagnostics of population annealing): with c_f the
 * replicas descended from initial replica f and R the population size,
 * out = {number of families with c_f > 0, rho_t = sum_f c_f^2 / R,
 *        S_f = -sum_f (c_f/R) ln(c_f/R) = ln R - (1/R) sum_f c_f ln c_f}.
 * anc[i] is the ancestor of replica slot i (MSC: linear 32*group + bit,
 * counted where active). */
static void family_stats(const int32_t* anc, const uint8_t* act, int n, int Rinit, int R, double out[3]) {
    uint32_t* cnt = (uint32_t*)calloc((size_t)Rinit, sizeof(uint32_t));
    for (int i = 0; i < n; ++i)
        if (!act || act[i]) cnt[anc[i]]++;
    long long nf = 0, c2 = 0;
    double clnc = 0.0;
    for (int f = 0; f < Rinit; ++f) {
        const long long c = cnt[f];
        if (!c) continue;
        nf++;
        c2 += c * c;
        clnc += (double)c * log((double)c);
    }
    out[0] = (double)nf;
    out[1] = (double)c2 / R;
    out[2] = log((double)R) - clnc / R;
    free(cnt);
}

int or_anneal2(int msc, int L, int Rinit, int sweeps, double dBinit, double Bfin, int runs, uint64_t seed,
               int max_steps, int adaptive, double minov, double maxov, double* rows, int max_rows,
               double* fam, double* attempts);

/* The engine's native-stream MSC gather (native_stream.c). */
void or_msc_resample_linear(const uint32_t* old, const int32_t* E_old, int L, int rg_old, const uint32_t* roff,
                            const uint32_t* offs, int rg_new, uint32_t* neu, uint8_t* new_active, int32_t* E_new);

/* The engine's native-stream MSC sweeps (native_stream.c). */
void or_msc_sweep_native2(uint32_t* words, int L, int rg, int sweeps, uint32_t T4, uint32_t T8, uint64_t key,
                          uint32_t step, uint32_t tag, int threads, int G, int cs);

int or_ssc_sweep_bits_native(int8_t* spins, int L, int R, int sweeps, uint32_t T4, uint32_t T8, uint64_t key,
                             uint32_t step, uint32_t tag, int G);
void or_ssc_sweep_native(int8_t* spins, int L, int R, int sweeps, uint32_t T4, uint32_t T8, uint64_t key,
                         uint32_t step, uint32_t tag);

/* Native-stream sweeps in place of checkKerALL's: key, tag, threads per CTA,
 * groups (MSC) or replicas (SSC bit planes; 0: the int8 SSC sweep) per work
 * unit and CTAs per group of or_msc_sweep_native2 / or_ssc_sweep_bits_native
 * / or_ssc_sweep_native; temperature i of run r is counter word i | r << 14. */
typedef struct {
    uint64_t key;
    uint32_t tag;
    int threads, G, cs;
} native_sweep_cfg;

static int anneal_impl(int msc, int L, int Rinit, int sweeps, double dBinit, double Bfin, int runs, uint64_t seed,
                       int max_steps, int adaptive, double minov, double maxov, double* rows, int max_rows,
                       double* fam, double* attempts, const native_sweep_cfg* nat, uint64_t iseq0);

int or_anneal(int msc, int L, int Rinit, int sweeps, double dBinit, double Bfin, int runs, uint64_t seed,
              int max_steps, double* rows, int max_rows, double* attempts) {
    return or_anneal2(msc, L, Rinit, sweeps, dBinit, Bfin, runs, seed, max_steps, 0, 0.0, 0.0, rows, max_rows,
                      NULL, attempts);
}

/* or_anneal with the adaptive temperature step (adaptive = 1): the first run
 * chooses its schedule, later runs replay it (PAisingSSC.cu:644,662).  fam
 * (optional) receives per run and temperature the family statistics above
 * (max_rows x 3 per run); the ancestors follow the replicas through every
 * resampling (SSC: new replica offs[j] + p copies old j; MSC: offspring s at
 * group s % rg_new, bit s / rg_new, PAisingMSC.cu:413-414). */
int or_anneal2(int msc, int L, int Rinit, int sweeps, double dBinit, double Bfin, int runs, uint64_t seed,
               int max_steps, int adaptive, double minov, double maxov, double* rows, int max_rows,
               double* fam, double* attempts) {
    return anneal_impl(msc, L, Rinit, sweeps, dBinit, Bfin, runs, seed, max_steps, adaptive, minov, maxov, rows,
                       max_rows, fam, attempts, NULL, 0);
}

/* or_anneal2 for MSC with the engine's native-stream sweeps (the
 * initialisation and the copy-number draws stay in reference coordinates,
 * as in the engine); runs are sequential and continue the subsequence
 * counter, which starts at iseq0 (population k of an engine batch with the
 * native stream starts at k << 40 and sweeps with tag | k). */
int or_anneal_msc_native(int L, int Rinit, int sweeps, double dBinit, double Bfin, int runs, uint64_t seed,
                         uint64_t key, uint32_t tag, uint64_t iseq0, int threads, int G, int cs, double* rows,
                         int max_rows, double* attempts) {
    const native_sweep_cfg nat = {key, tag, threads, G, cs};
    return anneal_impl(1, L, Rinit, sweeps, dBinit, Bfin, runs, seed, 0, 0, 0.0, 0.0, rows, max_rows, NULL,
                       attempts, &nat, iseq0);
}

/* The same for SSC with the bit-plane sweep (tile replicas per work unit),
 * or with the int8 sweep (tile = 0). */
int or_anneal_ssc_bits_native(int L, int Rinit, int sweeps, double dBinit, double Bfin, int runs, uint64_t seed,
                              uint64_t key, uint32_t tag, uint64_t iseq0, int tile, double* rows, int max_rows,
                              double* attempts) {
    const native_sweep_cfg nat = {key, tag, 256, tile, 1};
    return anneal_impl(0, L, Rinit, sweeps, dBinit, Bfin, runs, seed, 0, 0, 0.0, 0.0, rows, max_rows, NULL,
                       attempts, &nat, iseq0);
}

static int anneal_impl(int msc, int L, int Rinit, int sweeps, double dBinit, double Bfin, int runs, uint64_t seed,
                       int max_steps, int adaptive, double minov, double maxov, double* rows, int max_rows,
                       double* fam, double* attempts, const native_sweep_cfg* nat, uint64_t iseq0) {
    int N = L * L;
    const int nBmax = 10000;
    double* B = (double*)calloc(nBmax, sizeof(double));
    double* E = (double*)calloc(nBmax, sizeof(double));
    double* C = (double*)calloc(nBmax, sizeof(double));
    double* Mv = (double*)calloc(nBmax, sizeof(double));
    double* M2 = (double*)calloc(nBmax, sizeof(double));
    double* M4 = (double*)calloc(nBmax, sizeof(double));
    double* lnQ = (double*)calloc(nBmax, sizeof(double));
    double* BF = (double*)calloc(nBmax, sizeof(double));
    double* S = (double*)calloc(nBmax, sizeof(double));
    int* Rn = (int*)calloc(nBmax, sizeof(int));
    uint64_t iseq = iseq0;
    double tot_att = 0;
    int nB = 0, ret = 0;
    BF[0] = -N * log(2.0);
    Rn[0] = Rinit;
    for (int r = 0; r < runs && ret == 0; ++r) {
        double sumlnQ = 0.0, Emean = 0.0;
        int Rcap = 2 * Rinit + 1024, rg = (Rinit + MSB - 1) / MSB;
        int rgcap = (Rcap + MSB - 1) / MSB;
        int8_t *sp = NULL, *sp2 = NULL;
        uint32_t *wd = NULL, *wd2 = NULL;
        uint8_t *act = NULL, *act2 = NULL;
        int32_t* Ev = (int32_t*)malloc(sizeof(int32_t) * (size_t)rgcap * MSB);
        int32_t* Mm = (int32_t*)malloc(sizeof(int32_t) * (size_t)rgcap * MSB);
        uint32_t* roff = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)rgcap * MSB);
        uint32_t* offs = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)rgcap * MSB);
        int32_t* anc = (int32_t*)calloc((size_t)rgcap * MSB, sizeof(int32_t));
        int32_t* anc2 = (int32_t*)calloc((size_t)rgcap * MSB, sizeof(int32_t));
        double* fr = fam ? fam + (size_t)r * max_rows * 3 : NULL;
        for (int j = 0; j < Rinit; ++j) anc[j] = j;  /* MSC: linear 32*group + bit */
        if (fr) family_stats(anc, NULL, Rinit, Rinit, Rinit, fr);
        if (!msc) {
            sp = (int8_t*)malloc((size_t)Rcap * N);
            sp2 = (int8_t*)malloc((size_t)Rcap * N);
            or_ssc_init(sp, L, Rinit, seed, iseq);
            iseq += (uint64_t)Rinit * EQT;
            or_ssc_energy(sp, L, Rinit, Ev, Mm);
        } else {
            wd = (uint32_t*)calloc((size_t)rgcap * N, 4);
            wd2 = (uint32_t*)calloc((size_t)rgcap * N, 4);
            act = (uint8_t*)calloc((size_t)rgcap * MSB, 1);
            act2 = (uint8_t*)calloc((size_t)rgcap * MSB, 1);
            or_msc_init(wd, act, L, Rinit, rg, seed, iseq);
            iseq += (uint64_t)rg * EQT;
            or_msc_energy(wd, L, rg, Ev, Mm);
        }
        int i = 1;
        double deltaBeta = dBinit;
        B[1] = B[0] + dBinit;
        while (B[i] <= Bfin) {
            double dB = B[i] - B[i - 1];
            int Rp = Rn[i - 1];
            double q = msc ? or_msc_q(Ev, act, rg, dB, Emean) : or_ssc_q(Ev, Rp, dB, Emean);
            lnQ[i] = -(B[i] - B[i - 1]) * Emean + log(q) - log((double)Rp);
            uint32_t Rnew;
            if (!msc) {
                Rnew = or_ssc_copy_numbers(Ev, Rp, Rinit, lnQ[i], dB, seed, iseq, roff);
                iseq += (uint64_t)Rp;
                or_scan(roff, Rp, offs);
                if ((int)Rnew > Rcap) { ret = -1; break; }
                or_ssc_resample(sp, L, Rp, roff, offs, sp2);
                int8_t* t = sp; sp = sp2; sp2 = t;
                for (int j = 0; j < Rp; ++j)
                    for (uint32_t p = 0; p < roff[j]; ++p) anc2[offs[j] + p] = anc[j];
                int32_t* ta2 = anc; anc = anc2; anc2 = ta2;
                Rn[i] = (int)Rnew;
                if (fr) family_stats(anc, NULL, Rn[i], Rinit, Rn[i], fr + (size_t)i * 3);
                if (nat) {
                    uint32_t thr[2];
                    or_msc_thresholds(B[i], thr);
                    const uint32_t word = (uint32_t)i | ((uint32_t)r << 14);
                    if (nat->G == 0)
                        or_ssc_sweep_native(sp, L, Rn[i], sweeps, thr[0], thr[1], nat->key, word, nat->tag);
                    else if (!or_ssc_sweep_bits_native(sp, L, Rn[i], sweeps, thr[0], thr[1], nat->key, word,
                                                       nat->tag, nat->G)) {
                        ret = -1;
                        break;
                    }
                } else {
                    double tab[10];
                    or_ssc_boltz(B[i], tab);
                    or_ssc_sweep(sp, L, Rn[i], sweeps, tab, seed, iseq);
                }
                iseq += (uint64_t)Rn[i] * EQT;
                or_ssc_energy(sp, L, Rn[i], Ev, Mm);
                double avg[5];
                or_averages(Ev, Mm, NULL, Rn[i], avg);
                E[i] = Emean = avg[0] / Rn[i];
                C[i] = (avg[1] / Rn[i] - E[i] * E[i]) * B[i] * B[i];
                Mv[i] = avg[2] / Rn[i]; M2[i] = avg[3] / Rn[i]; M4[i] = avg[4] / Rn[i];
            } else {
                Rnew = or_msc_copy_numbers(Ev, act, rg, Rinit, Rp, lnQ[i], dB, seed, iseq, roff);
                iseq += (uint64_t)rg * MSB;
                or_scan(roff, rg * MSB, offs);
                if ((int)Rnew > Rcap) { ret = -1; break; }
                int rgn = (int)((Rnew + MSB - 1) / MSB);
                memset(wd2, 0, (size_t)rgn * N * 4);
                /* the engine's own stream places offspring s at slot s, the
                 * reference's at group s % rgn, bit s / rgn */
                if (nat)
                    or_msc_resample_linear(wd, Ev, L, rg, roff, offs, rgn, wd2, act2, NULL);
                else
                    or_msc_resample(wd, Ev, L, rg, roff, offs, rgn, wd2, act2, NULL);
                for (int lin = 0; lin < rg * MSB; ++lin)
                    for (uint32_t p = 0; p < roff[lin]; ++p) {
                        const uint32_t s = offs[lin] + p;
                        anc2[nat ? s : (s % rgn) * MSB + s / rgn] = anc[lin];
                    }
                int32_t* ta2 = anc; anc = anc2; anc2 = ta2;
                uint32_t* t = wd; wd = wd2; wd2 = t;
                uint8_t* ta = act; act = act2; act2 = ta;
                rg = rgn;
                Rn[i] = (int)Rnew;
                if (fr) family_stats(anc, act, rg * MSB, Rinit, Rn[i], fr + (size_t)i * 3);
                uint32_t thr[2];
                or_msc_thresholds(B[i], thr);
                if (nat)
                    or_msc_sweep_native2(wd, L, rg, sweeps, thr[0], thr[1], nat->key,
                                         (uint32_t)i | ((uint32_t)r << 14), nat->tag, nat->threads, nat->G, nat->cs);
                else
                    or_msc_sweep(wd, L, rg, sweeps, thr, seed, iseq);
                iseq += (uint64_t)rg * EQT;
                or_msc_energy(wd, L, rg, Ev, Mm);
                double avg[5];
                or_averages(Ev, Mm, act, rg * MSB, avg);
                E[i] = Emean = avg[0] / Rn[i];
                C[i] = (avg[1] / Rn[i] - E[i] * E[i]) * B[i] * B[i];
                Mv[i] = avg[2] / Rn[i]; M2[i] = avg[3] / Rn[i]; M4[i] = avg[4] / Rn[i];
            }
            sumlnQ -= lnQ[i];
            BF[i] = -N * log(2.0) + sumlnQ;
            S[i] = B[i] * E[i] - BF[i];
            tot_att += (double)sweeps * N * Rn[i];
            ++i;
            if (i >= nBmax || i > max_rows - 1) { ret = -1; break; }
            if (max_steps > 0 && i > max_steps) { B[i] = Bfin + 1.0; break; }
            if (!adaptive) {
                B[i] = B[i - 1] + dBinit;
            } else if (r == 0) {
                deltaBeta = next_step(msc, Ev, act, rg, Rn[i - 1], Rinit, Emean, B[i - 1], Bfin, deltaBeta, minov,
                                      maxov);
                B[i] = B[i - 1] + deltaBeta;
            }  /* later runs: B[i] as the first run left it */
        }
        nB = i;
        if (rows && ret == 0) {
            double* o = rows + (size_t)r * max_rows * 10;
            for (int k = 0; k < nB; ++k) {
                double* w = o + (size_t)k * 10;
                w[0] = B[k]; w[1] = E[k] / N; w[2] = C[k] / N; w[3] = Mv[k] / N;
                w[4] = M2[k] / N / N; w[5] = M4[k] / N / N / N / N; w[6] = BF[k] / N;
                w[7] = S[k] / N; w[8] = Rn[k]; w[9] = lnQ[k];
            }
        }
        free(sp); free(sp2); free(wd); free(wd2); free(act); free(act2);
        free(Ev); free(Mm); free(roff); free(offs); free(anc); free(anc2);
    }
    if (attempts) *attempts = tot_att;
    free(B); free(E); free(C); free(Mv); free(M2); free(M4); free(lnQ); free(BF); free(S); free(Rn);
    return ret == 0 ? nB : -1;
}
