/*
 * native_stream.c -- CPU restatement of the engine's NATIVE random stream and
 * of the multi-spin-coded sweep that consumes it.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links or calls
 * this file; it is built into oracle/_build/libpaoracle.so beside the
 * restatement of the reference (pa_oracle.c) and used by tests/ to check the
 * engine's production sweep bit for bit.
 *
 * The reference has no counterpart: its MSC sweep draws one cuRAND word per
 * word-site and expands it to 32 numbers with an LCG (PAisingMSC.cu:220-225).
 * The engine's native stream instead decides every replica's Metropolis test
 * U < T/2^32 (T = ceil(2^32 e^{-4 beta}) or ceil(2^32 e^{-8 beta}), the
 * reference's thresholds, PAisingMSC.cu:674-675) exactly, from fresh
 * Philox4x32-10 bits.  This file restates that specification independently of
 * the CUDA code (written from the description, in plain C):
 *
 *   key      = the stream seed (k0 = low word, k1 = high word)
 *   counter  = (c0, c1 | sub, step, tag)   c1 = (2 sweep + half) << 4
 *   head     : word-site k of a thread's batch of four: digits 0..3 of its 32
 *              comparisons from block (site_k, c1 | 0): word j = digit j
 *   merge    : the still-undecided bits of sites 1..3 are rotated left by the
 *              smallest r that keeps them clear of the bits already merged
 *              (site 0's at rotation 0); a site with no such r "overflows"
 *   tail     : the merged word takes digits 4..7 from block (chain, c1 | 1);
 *              an overflowing site from block (site_k, c1 | 8)
 *   finish   : a bit still undecided after digit 7 is decided at once by
 *              U mod 2^24 < T mod 2^24, U's remaining 24 digits being the top
 *              24 bits of one fresh word: lowest bit first, four bits per
 *              block (c0, c1 | (fsub + k), step, tag ^ 0x20000000), k = 0..7,
 *              fsub = 0 for the merged word and 8 for an overflowing site
 *
 * A digit-serial comparison: digit j of U is bit i of word j for replica bit
 * i; while the digits agree with T's the bit stays undecided; at the first
 * difference it is decided, "less" iff T's digit is 1.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "inj_stream.h"

#define FINISH_TAG_FLIP 0x20000000u

static inline uint32_t rotl32(uint32_t x, uint32_t r) { return r ? (x << r) | (x >> (32u - r)) : x; }
static inline uint32_t rotr32(uint32_t x, uint32_t r) { return r ? (x >> r) | (x << (32u - r)) : x; }

static inline void blk(uint64_t key, uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t o[4]) {
    const uint32_t k[2] = {(uint32_t)key, (uint32_t)(key >> 32)};
    const uint32_t c[4] = {c0, c1, c2, c3};
    inj_philox4x32_10(k, c, o);
}

/* one digit j (0 = most significant) for every bit in *und; bits of `a` use
 * T4's digit, the others T8's */
static inline void digit(uint32_t u, uint32_t a, uint32_t T4, uint32_t T8, int j, uint32_t* und, uint32_t* lt) {
    const uint32_t d4 = (T4 >> (31 - j)) & 1u ? 0xFFFFFFFFu : 0u;
    const uint32_t d8 = (T8 >> (31 - j)) & 1u ? 0xFFFFFFFFu : 0u;
    const uint32_t t = (a & d4) | (~a & d8);
    const uint32_t differ = *und & (t ^ u);
    *lt |= differ & t;
    *und &= ~differ;
}

/* digits 4.. of one word's undecided bits; returns the bits decided "less" */
static uint32_t finish_word(uint32_t und, uint32_t a, uint32_t c0, uint32_t c1, uint32_t sub, uint32_t fsub,
                            uint32_t step, uint32_t tag, uint64_t key, uint32_t T4, uint32_t T8) {
    uint32_t lt = 0, o[4];
    if (!und) return 0;
    blk(key, c0, c1 | sub, step, tag, o);
    for (int j = 0; j < 4; ++j) digit(o[j], a, T4, T8, 4 + j, &und, &lt);
    for (uint32_t k = 0; k < 8 && und; ++k) {
        blk(key, c0, c1 | (fsub + k), step, tag ^ FINISH_TAG_FLIP, o);
        for (int n = 0; n < 4 && und; ++n) {
            int i = 0;
            while (!((und >> i) & 1u)) ++i;
            const uint32_t t = ((a >> i) & 1u ? T4 : T8) & 0xFFFFFFu;
            if ((o[n] >> 8) < t) lt |= 1u << i;
            und &= ~(1u << i);
        }
    }
    return lt;
}

/* Acceptance of nvalid (<= 4) word-sites of one thread batch.
 *   a[k]   bits with one anti-parallel neighbour (threshold T4), else T8
 *   und[k] bits that need a random decision
 *   acc[k] in: bits accepted outright; out: all accepted bits */
void or_native_accept4(const uint32_t a[4], const uint32_t und_in[4], uint32_t acc[4], const uint32_t site[4],
                       int nvalid, uint32_t chain, uint32_t c1, uint32_t step, uint32_t tag, uint64_t key,
                       uint32_t T4, uint32_t T8) {
    uint32_t und[4], o[4];
    for (int k = 0; k < 4; ++k) {
        und[k] = k < nvalid ? und_in[k] : 0u;
        if (!und[k]) continue;
        blk(key, site[k], c1, step, tag, o);
        for (int j = 0; j < 4; ++j) digit(o[j], a[k], T4, T8, j, &und[k], &acc[k]);
    }
    uint32_t m = und[0], am = a[0] & und[0], rot[4] = {0, 0, 0, 0}, ovf[4] = {0, 0, 0, 0};
    for (int k = 1; k < 4; ++k) {
        uint32_t r = 0;
        while (r < 32u && (m & rotl32(und[k], r))) ++r;
        if (r == 32u) {
            ovf[k] = 1;
            continue;
        }
        rot[k] = r;
        m |= rotl32(und[k], r);
        am |= rotl32(a[k] & und[k], r);
    }
    const uint32_t lt = finish_word(m, am, chain, c1, 1u, 0u, step, tag, key, T4, T8);
    acc[0] |= lt & und[0];
    for (int k = 1; k < 4; ++k)
        acc[k] |= ovf[k] ? finish_word(und[k], a[k] & und[k], site[k], c1, 8u, 8u, step, tag, key, T4, T8)
                         : rotr32(lt, rot[k]) & und[k];
}

/* Bitsliced count of anti-parallel neighbours (PAisingMSC.cu:207-218). */
static inline void count4(uint32_t s, const uint32_t n[4], uint32_t* c0, uint32_t* c1, uint32_t* c2) {
    uint32_t b0 = 0, b1 = 0, b2 = 0;
    for (int k = 0; k < 4; ++k) {  /* ripple-add one input plane at a time */
        const uint32_t x = s ^ n[k];
        const uint32_t carry0 = b0 & x;
        b0 ^= x;
        const uint32_t carry1 = b1 & carry0;
        b1 ^= carry0;
        b2 |= carry1;
    }
    *c0 = b0;
    *c1 = b1;
    *c2 = b2;
}

/* One thread's batches of one half-sweep: word column tx of the rows
 * first_row + rsub + pass * rpp (interleaved) or first_row + rsub * npass +
 * pass (consecutive), pass < npass, row index below first_row + nrows, of a
 * stack of sublattice rows in which row v belongs to group group0 + v / L at
 * row v % L (a one-group unit: nrows = L; a stacked tile: nrows = groups * L;
 * a cluster stripe: the stripe's rows of one group).  Batch b of the thread
 * is Philox chain chain0 + b. */
static void thread_half(uint32_t* words, int L, int group0, int first_row, int nrows, int rsub, int tx, int rpp,
                        int npass, int consecutive, int hf, uint32_t c1, uint32_t chain0, uint64_t key, uint32_t step,
                        uint32_t tag, uint32_t T4, uint32_t T8) {
    const int N = L * L, h = N / 2, Wr = L / 2;
    for (int p0 = 0; p0 < npass; p0 += 4) {
        uint32_t a[4] = {0}, und[4] = {0}, acc[4] = {0}, site[4] = {0};
        uint32_t* word[4] = {NULL, NULL, NULL, NULL};
        for (int k = 0; k < 4; ++k) {
            const int pass = p0 + k, v = first_row + (consecutive ? rsub * npass + pass : rsub + pass * rpp);
            if (pass >= npass || v >= first_row + nrows) continue;
            const int g = group0 + v / L, y = v % L, i = y * Wr + tx;
            uint32_t* self = words + (size_t)g * N + (hf ? h : 0);
            const uint32_t* oth = words + (size_t)g * N + (hf ? 0 : h);
            /* horizontal neighbour: left for A in even rows and B in odd
             * rows, else right */
            const int left = (hf == 0) == ((y & 1) == 0);
            const int xs = left ? (tx + Wr - 1) % Wr : (tx + 1) % Wr;
            const uint32_t n[4] = {oth[y * Wr + xs], oth[i], oth[((y + L - 1) % L) * Wr + tx],
                                   oth[((y + 1) % L) * Wr + tx]};
            uint32_t c0, cc1, cc2;
            count4(self[i], n, &c0, &cc1, &cc2);
            a[k] = c0;
            acc[k] = cc1 | cc2;  /* two or more anti-parallel: dE <= 0 */
            und[k] = ~(cc1 | cc2);
            site[k] = (uint32_t)g * (uint32_t)h + (uint32_t)i;
            word[k] = self + i;
        }
        or_native_accept4(a, und, acc, site, npass - p0, chain0 + (uint32_t)(p0 / 4), c1, step, tag, key, T4, T8);
        for (int k = 0; k < 4; ++k)
            if (word[k]) *word[k] ^= acc[k];
    }
}

/* `sweeps` native checkerboard sweeps of rg groups of 32 replicas at
 * thresholds T4, T8, with the thread layouts of the engine's MSC sweeps:
 *   cs = 1: one CTA of `threads` threads per work unit of G groups (tile
 *           ti = groups G ti .. G ti + G - 1, the last one possibly short),
 *           whose sublattices form one stack of G L rows; thread
 *           (rsub, tx) = (tid / (L/2), tid % (L/2)) updates word column tx of
 *           stacked rows rsub + pass * rpp (G > 1) or of its own consecutive
 *           rows rsub * npass + pass (G = 1), rpp = min(threads / (L/2), G L),
 *           npass = ceil(G L / rpp); its batch of four passes p0 / 4 is chain
 *           (ti threads + tid) nbatch + p0 / 4;
 *   cs > 1: a cluster of cs CTAs per group; CTA `rank` updates rows
 *           [rank L/cs, (rank + 1) L/cs), thread (rsub, tx) the consecutive
 *           rows rank L/cs + rsub * npass + pass, with rpp the largest divisor
 *           of L/cs with (L/2) rpp <= threads and npass = L/cs / rpp; chain
 *           ((g cs + rank) threads + tid) nbatch + p0 / 4.
 * Within a half-sweep every update reads the other sublattice only, so the
 * order in which threads are visited does not matter.  Layout as the
 * reference's MSC Replica (PAisingMSC.cu:84-92): group g at words + g*N,
 * sublattice A then B, site (x, y) of a sublattice at y*L/2 + x/2; the
 * horizontal neighbour of an A site in an even row is on its left
 * (PAisingMSC.cu:203, 238). */
void or_msc_sweep_native2(uint32_t* words, int L, int rg, int sweeps, uint32_t T4, uint32_t T8, uint64_t key,
                          uint32_t step, uint32_t tag, int threads, int G, int cs) {
    const int Wr = L / 2;
    int rpp, npass, nunits;
    if (cs <= 1) {
        rpp = threads / Wr;
        if (rpp > G * L) rpp = G * L;
        npass = (G * L + rpp - 1) / rpp;
        nunits = (rg + G - 1) / G;
    } else {
        const int LR = L / cs;
        rpp = 1;
        for (int r = 1; r <= LR; ++r)
            if (LR % r == 0 && Wr * r <= threads) rpp = r;
        npass = LR / rpp;
        nunits = rg * cs;
    }
    const int nbatch = (npass + 3) / 4;
#pragma omp parallel for schedule(static)
    for (int u = 0; u < nunits; ++u) {
        /* units touch disjoint groups except the CTAs of one cluster, which
         * are visited together below */
        if (cs > 1 && u % cs) continue;
        const int g0 = cs > 1 ? u / cs : u * G, gc = cs > 1 ? 1 : (rg - g0 < G ? rg - g0 : G);
        for (int sw = 0; sw < sweeps; ++sw)
            for (int hf = 0; hf < 2; ++hf) {
                const uint32_t c1 = (uint32_t)(sw * 2 + hf) << 4;
                for (int rank = 0; rank < (cs > 1 ? cs : 1); ++rank)
                    for (int tid = 0; tid < Wr * rpp; ++tid) {
                        const uint32_t unit = cs > 1 ? (uint32_t)(g0 * cs + rank) : (uint32_t)u;
                        const uint32_t chain0 = (unit * (uint32_t)threads + (uint32_t)tid) * (uint32_t)nbatch;
                        const int first = cs > 1 ? rank * (L / cs) : 0, nrows = cs > 1 ? L / cs : gc * L;
                        thread_half(words, L, g0, first, nrows, tid / Wr, tid % Wr, rpp, npass, cs > 1 || G == 1,
                                    hf, c1, chain0, key, step, tag, T4, T8);
                    }
            }
    }
}

/* The one-CTA sweep over one group per work unit (cs = 1, G = 1). */
void or_msc_sweep_native(uint32_t* words, int L, int rg, int sweeps, uint32_t T4, uint32_t T8, uint64_t key,
                         uint32_t step, uint32_t tag, int threads) {
    or_msc_sweep_native2(words, L, rg, sweeps, T4, T8, key, step, tag, threads, 1, 1);
}

/* ---------------------------------------------------------------------------
 * SSC populations swept on bit planes (native stream; no counterpart in the
 * reference, whose SSC sweep draws one cuRAND double per site,
 * PAisingSSC.cu:159-193).
 *
 * Row layout: a sublattice row of S = L/2 sites is Wq words of seg sites,
 * the smallest Wq (at most 8) with seg = S/Wq a multiple of 4 and at most 32;
 * when Wq = 1, segs = floor(32/seg) replicas share a word, replica j of the
 * word in bits [j seg, (j + 1) seg); bit i of a segment is site x = c seg + i
 * of the row (c = word of the row).  A tile holds G replicas (G a multiple of
 * segs), i.e. G/segs word groups of wpp = L Wq words per sublattice; the last
 * tile of a population may be short: the word groups it touches are complete,
 * the missing replicas' segments start at bit 0 and are swept like the others
 * (their decisions take part in the acceptance's merging) but never stored.
 * Half-sweep: 256 threads; word it = tid + 256 q of the tile's plane goes to
 * thread tid, four words (q = q0..q0+3) per batch, batch chain
 * (tile 256 + tid) 8 + q0/4; word-site number (tile G/segs + word group) wpp
 * + word of the group.  L = 64 and 128 (rows of Wq = 1 or 2 full 32-site
 * words) instead: with GM = 1024 / (L Wq) and RL = 8 / Wq, thread
 * tid = 32 w + lane, lane = (gl RL + rl) Wq + c, takes word column c of rows
 * 4 (RL (w / (GM/4)) + rl) .. + 3 of word group 4 (w % (GM/4)) + gl as its
 * one batch, chain (tile 256 + tid) 8.
 * ------------------------------------------------------------------------- */
static int bits_layout_c(int L, int* Wq, int* seg, int* segs) {
    if (L < 8 || L % 8 != 0 || L > 256) return 0;
    const int S = L / 2;
    for (int w = (S + 31) / 32; w <= 8; ++w)
        if (S % w == 0 && (S / w) % 4 == 0) {
            *Wq = w;
            *seg = S / w;
            *segs = w == 1 ? 32 / *seg : 1;
            return 1;
        }
    return 0;
}

/* returns 0 where L has no bit-plane layout or G is not a multiple of segs */
int or_ssc_sweep_bits_native(int8_t* spins, int L, int R, int sweeps, uint32_t T4, uint32_t T8, uint64_t key,
                             uint32_t step, uint32_t tag, int G) {
    int Wq, seg, segs;
    if (!bits_layout_c(L, &Wq, &seg, &segs) || G < segs || G % segs) return 0;
    const int N = L * L, h = N / 2, S = L / 2, wpp = L * Wq, GW = G / segs, ntiles = (R + G - 1) / G;
#pragma omp parallel for schedule(static)
    for (int ti = 0; ti < ntiles; ++ti) {
        const int r0 = ti * G, gc = R - r0 < G ? R - r0 : G;
        const int ngroups = (gc + segs - 1) / segs, slots = ngroups * segs, items = ngroups * wpp;
        /* sp[slot][X][y][x] in {0, 1} (1 == +1); slots beyond gc start at 0 */
        uint8_t* sp = (uint8_t*)calloc((size_t)slots * N, 1);
        for (int r = 0; r < gc; ++r)
            for (int i = 0; i < N; ++i) sp[(size_t)r * N + i] = spins[(size_t)(r0 + r) * N + i] > 0;
        for (int sw = 0; sw < sweeps; ++sw)
            for (int hf = 0; hf < 2; ++hf) {
                const uint32_t c1 = (uint32_t)(sw * 2 + hf) << 4;
                const int full = seg == 32 && (Wq == 1 || Wq == 2);
                for (int tid = 0; tid < 256; ++tid)
                    for (int q0 = 0; q0 * 256 < (full ? 1 : items); q0 += 4) {
                        uint32_t a[4] = {0}, und[4] = {0}, acc[4] = {0}, site[4] = {0};
                        int item[4] = {-1, -1, -1, -1}, nvalid = 0;
                        for (int k = 0; k < 4; ++k) {
                            int it = tid + (q0 + k) * 256;
                            if (full) {
                                const int GM = 1024 / (L * Wq), RL = 8 / Wq, w = tid / 32, lane = tid % 32;
                                const int cc = lane % Wq, gl = lane / Wq / RL, rl = lane / Wq % RL;
                                const int gg = 4 * (w % (GM / 4)) + gl, y0 = 4 * (RL * (w / (GM / 4)) + rl);
                                it = gg < ngroups ? gg * wpp + (y0 + k) * Wq + cc : items;
                            }
                            if (it >= items) continue;
                            const int g = it / wpp, wr = it % wpp, y = wr / Wq, c = wr % Wq;
                            const int left = (hf == 0) == ((y & 1) == 0);
                            for (int j = 0; j < segs; ++j)
                                for (int i = 0; i < seg; ++i) {
                                    const uint8_t* me = sp + (size_t)(g * segs + j) * N + (hf ? h : 0);
                                    const uint8_t* ot = sp + (size_t)(g * segs + j) * N + (hf ? 0 : h);
                                    const int x = c * seg + i, xs = left ? (x + S - 1) % S : (x + 1) % S;
                                    const int s = me[y * S + x];
                                    const int n = (s != ot[y * S + x]) + (s != ot[y * S + xs]) +
                                                  (s != ot[((y + L - 1) % L) * S + x]) +
                                                  (s != ot[((y + 1) % L) * S + x]);
                                    const uint32_t bit = 1u << (j * seg + i);
                                    if (n >= 2) acc[k] |= bit;
                                    else und[k] |= bit;
                                    if (n == 1) a[k] |= bit;
                                }
                            site[k] = (uint32_t)(ti * GW + g) * (uint32_t)wpp + (uint32_t)wr;
                            item[k] = it;
                            ++nvalid;
                        }
                        or_native_accept4(a, und, acc, site, nvalid, ((uint32_t)ti * 256u + (uint32_t)tid) * 8u +
                                          (uint32_t)(q0 / 4), c1, step, tag, key, T4, T8);
                        for (int k = 0; k < 4; ++k) {
                            if (item[k] < 0) continue;
                            const int g = item[k] / wpp, wr = item[k] % wpp, y = wr / Wq, c = wr % Wq;
                            for (int j = 0; j < segs; ++j)
                                for (int i = 0; i < seg; ++i)
                                    if ((acc[k] >> (j * seg + i)) & 1u)
                                        sp[(size_t)(g * segs + j) * N + (hf ? h : 0) + y * S + c * seg + i] ^= 1;
                        }
                    }
            }
        for (int r = 0; r < gc; ++r)
            for (int i = 0; i < N; ++i) spins[(size_t)(r0 + r) * N + i] = sp[(size_t)r * N + i] ? 1 : -1;
        free(sp);
    }
    return 1;
}

/* ---------------------------------------------------------------------------
 * SSC populations swept one int8 spin per site (native stream; the sweep of
 * lattices without a dense bit-plane layout, or when asked for).
 *
 * A site with dE <= 0 flips; otherwise it flips iff U < T (T4 for one
 * anti-parallel neighbour, T8 for none), decided a byte at a time.  Words of
 * four sites (site x = 4 c + j of a sublattice row is byte j of word c) are
 * handled in pairs: thread (rsub, c) = (tid / (L/8), tid % (L/8)) of the
 * replica's unit, tid < (L/8) rpp (rpp the largest divisor of L with
 * (L/8) rpp <= 256), takes rows ty0 = rsub, rsub + 2 rpp, ... and with each
 * also row ty1 = ty0 + rpp if ty1 < L.  Block (r h/4 + w0, 2 (2 sweep + half),
 * step, tag), w0 = ty0 L/8 + c: word x gives U's top bytes for row ty0, word
 * y for row ty1; a site whose top byte equals T's is decided by U's low 24
 * bits, taken in order of (row ty0 sites, row ty1 sites) from words z, w,
 * then from blocks (r h/4 + w0, 2 (2 sweep + half) + 1, step, tag | k << 12),
 * k = 0, 1, four words each.
 * ------------------------------------------------------------------------- */
void or_ssc_sweep_native(int8_t* spins, int L, int R, int sweeps, uint32_t T4, uint32_t T8, uint64_t key,
                         uint32_t step, uint32_t tag) {
    const int N = L * L, h = N / 2, S = L / 2, Wr = L / 8, hw = h / 4;
    int rpp = 1;
    for (int q = 1; q <= L; ++q)
        if (L % q == 0 && Wr * q <= 256) rpp = q;
#pragma omp parallel for schedule(static)
    for (int r = 0; r < R; ++r) {
        int8_t* A = spins + (size_t)r * N;
        for (int sw = 0; sw < sweeps; ++sw)
            for (int hf = 0; hf < 2; ++hf) {
                int8_t* self = A + (hf ? h : 0);
                const int8_t* oth = A + (hf ? 0 : h);
                const uint32_t c1 = (uint32_t)(sw * 2 + hf) * 2u;
                for (int tid = 0; tid < Wr * rpp; ++tid) {
                    const int c = tid % Wr, rsub = tid / Wr;
                    for (int ty0 = rsub; ty0 < L; ty0 += 2 * rpp) {
                        const int rows[2] = {ty0, ty0 + rpp}, nrow = ty0 + rpp < L ? 2 : 1;
                        uint32_t o[4];
                        blk(key, (uint32_t)(r * hw + ty0 * Wr + c), c1, step, tag, o);
                        int flip[8] = {0}, pend[8], npend = 0, na_of[8];
                        for (int q = 0; q < nrow; ++q) {
                            const int y = rows[q], left = (hf == 0) == ((y & 1) == 0);
                            for (int j = 0; j < 4; ++j) {
                                const int x = 4 * c + j, xs = left ? (x + S - 1) % S : (x + 1) % S;
                                const int s = self[y * S + x];
                                const int na = (s != oth[y * S + x]) + (s != oth[y * S + xs]) +
                                               (s != oth[((y + L - 1) % L) * S + x]) +
                                               (s != oth[((y + 1) % L) * S + x]);
                                na_of[4 * q + j] = na;
                                if (na >= 2) {
                                    flip[4 * q + j] = 1;
                                    continue;
                                }
                                const uint32_t T = na == 1 ? T4 : T8;
                                const uint32_t ub = (o[q] >> (8 * j)) & 0xFFu, tb = T >> 24;
                                if (ub < tb) flip[4 * q + j] = 1;
                                else if (ub == tb) pend[npend++] = 4 * q + j;
                            }
                        }
                        uint32_t words[10] = {o[2], o[3]};
                        if (npend > 2) {
                            blk(key, (uint32_t)(r * hw + ty0 * Wr + c), c1 + 1u, step, tag, words + 2);
                            if (npend > 6) blk(key, (uint32_t)(r * hw + ty0 * Wr + c), c1 + 1u, step, tag | (1u << 12),
                                               words + 6);
                        }
                        for (int p = 0; p < npend; ++p) {
                            const int b = pend[p];
                            const uint32_t T = na_of[b] == 1 ? T4 : T8;
                            if ((words[p] & 0xFFFFFFu) < (T & 0xFFFFFFu)) flip[b] = 1;
                        }
                        for (int q = 0; q < nrow; ++q)
                            for (int j = 0; j < 4; ++j)
                                if (flip[4 * q + j]) self[rows[q] * S + 4 * c + j] = (int8_t)-self[rows[q] * S + 4 * c + j];
                    }
                }
            }
    }
}

/* The engine's MSC gather with its own stream (no counterpart in the
 * reference): offspring s -- in the scan order of old linear slots
 * 32 * group + bit -- goes to new slot s, i.e. group s / 32, bit s % 32
 * (the reference places it at group s % rg_new, bit s / rg_new,
 * PAisingMSC.cu:413-414, which only its own random stream needs).  Same
 * arguments as or_msc_resample; new_active[s] = s < R_new. */
void or_msc_resample_linear(const uint32_t* old, const int32_t* E_old, int L, int rg_old, const uint32_t* roff,
                            const uint32_t* offs, int rg_new, uint32_t* neu, uint8_t* new_active, int32_t* E_new) {
    const int N = L * L;
    for (int i = 0; i < rg_new * 32; ++i) new_active[i] = 0;
    for (int g = 0; g < rg_old; ++g)
        for (int k = 0; k < 32; ++k)
            for (uint32_t p = 0; p < roff[g * 32 + k]; ++p) {
                const uint32_t s = offs[g * 32 + k] + p, nj = s / 32, nk = s % 32;
                new_active[s] = 1;
                if (E_new) E_new[s] = E_old[g * 32 + k];
                const uint32_t* src = old + (size_t)g * N;
                uint32_t* dst = neu + (size_t)nj * N;
                for (int i = 0; i < N; ++i) dst[i] |= ((src[i] >> k) & 1u) << nk;
            }
}
