// pa_msc_cluster.cu -- multi-spin-coded sweep of one group by a thread-block
// cluster, for lattices whose two sublattices (4 N bytes per group) do not
// fit one CTA's shared memory (L = 256: 256 KB > 227 KB).
//
// CTA r of a cluster of CS holds rows [r L/CS, (r+1) L/CS) of both
// sublattices in its shared memory, each stripe framed by two halo rows.
// During a half-sweep only one sublattice changes, so after the cluster
// barrier that ends the previous half-sweep every CTA copies the rows of the
// other sublattice just above and below its stripe out of the neighbouring
// CTAs' shared memory (distributed shared memory) into its halo rows; the
// update itself then reads local shared memory only.  Random draws,
// decisions, energies and statistics are the ones of msc_sweep_kernel
// (pa_msc.cu): with the reference stream both give identical lattices
// (every draw is keyed by global site coordinates).
#include <cooperative_groups.h>

#include <climits>
#include <type_traits>

#include "pa_kernels.h"
#include "pa_msc_core.cuh"

namespace cg = cooperative_groups;

namespace pa {

using namespace msc;

// This CTA's stripe (rows row0 .. row0+LR-1) of both sublattices of group
// gi <-> shared memory, below a halo row of Wr words each (stripe X at
// lat + X*SH + Wr).  Out of line: keeps the sweep loop's registers free.
__device__ __noinline__ void cluster_move_stripe(const UnitParams& P, uint32_t* lat, int gi, int row0, int LR, int SH,
                                                 bool to_smem) {
  const int Wr = P.Wr, SW = LR * Wr;
  uint4* ga = (uint4*)(P.words + (size_t)gi * P.N + (size_t)row0 * Wr);
  uint4* gb = (uint4*)(P.words + (size_t)gi * P.N + P.h + (size_t)row0 * Wr);
  uint4* la = (uint4*)(lat + Wr);
  uint4* lb = (uint4*)(lat + SH + Wr);
  for (int v = threadIdx.x; v < (SW >> 2); v += blockDim.x) {
    if (to_smem) {
      la[v] = ga[v];
      lb[v] = gb[v];
    } else {
      ga[v] = la[v];
      gb[v] = lb[v];
    }
  }
}

// Energy and magnetisation counts of this stripe per replica bit: left and
// up bond of every A and B site (PAisingMSC.cu:272-294), the up neighbours
// of the last row taken from the lower halos; lane k of every warp adds bit
// k's counts to cntE / cntM.
__device__ __noinline__ void cluster_count(const UnitParams& P, const uint32_t* lat, int row0, int LR, int SH, int tx,
                                           int txl, int rsub, bool worker, int* cntE, int* cntM) {
  const int Wr = P.Wr, rpp = P.rpp, npass = P.npass, lane = threadIdx.x & 31;
  const uint32_t* A = lat + Wr;
  const uint32_t* Bs = lat + SH + Wr;
  BitCounters bc;  // npass <= 32 words per lane
  bc.reset();
  for (int pass = 0; pass < npass; ++pass) {
    const int lr = rsub + pass * rpp;
    const bool valid = worker && lr < LR;
    uint32_t s0 = 0, s1 = 0, s2 = 0, sA = 0, sB = 0;
    if (valid) {
      const int ty = row0 + lr, row = lr * Wr;
      sA = A[row + tx];
      sB = Bs[row + tx];
      uint32_t Ai2, Bi2;
      if (ty & 1) { Ai2 = sB; Bi2 = A[row + txl]; }
      else { Ai2 = Bs[row + txl]; Bi2 = sA; }
      const uint32_t Ai4 = Bs[row + Wr + tx], Bi4 = A[row + Wr + tx];
      adder4(sA ^ Ai2, sA ^ Ai4, sB ^ Bi2, sB ^ Bi4, s0, s1, s2);
    }
    bc.add(s0, s1, s2, sA, sB);
  }
  int cE, cM;  // lane k: bit k
  bc.totals(lane, cE, cM);
  atomicAdd(&cntE[lane], cE);
  atomicAdd(&cntM[lane], cM);
}

template <int MODE, int CS, int THREADS>
__global__ void __launch_bounds__(THREADS, 1024 / THREADS)
    msc_sweep_cluster_kernel(BatchDev* b, int energy_only, unsigned long long stream_seed) {
  const PhiloxKeys keys(stream_seed);
  extern __shared__ __align__(16) uint32_t lat[];  // stripe of A (LR*Wr words), then stripe of B
  __shared__ int s_unit, s_pop;
  __shared__ int s_cntE[kMsb], s_cntM[kMsb];
  __shared__ uint2 s_dig[kMsb];
  __shared__ UnitParams P;
  __shared__ BitStats stats;  // used by rank 0

  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int prev = (rank + CS - 1) % CS, next = (rank + 1) % CS;
  const int tid = threadIdx.x;
  const int total = b->unit_prefix[b->npop];
  int cur = -1;
  int tx = 0, rsub = 0, txl = 0, txr = 0;
  bool worker = false;
  if (tid < kMsb) stats.reset(tid);

  for (;;) {
    cluster.sync();  // the previous group is finished everywhere (including remote reads)
    if (rank == 0 && tid == 0) {
      const int u = (int)atomicAdd(&b->work_next, 1u);
      int loc = 0;
      const int p = u < total ? queue_pop(b, u, &loc) : -1;
      for (int r = 0; r < CS; ++r) {
        *cluster.map_shared_rank(&s_pop, r) = p;
        *cluster.map_shared_rank(&s_unit, r) = loc;
      }
    }
    cluster.sync();
    const int p = s_pop, gi = s_unit;
    if (p < 0) break;  // every CTA of the cluster leaves after the same barrier
    if (tid < kMsb) { s_cntE[tid] = 0; s_cntM[tid] = 0; }
    if (p != cur) {  // cluster-uniform
      if (rank == 0 && tid < kMsb && cur >= 0) stats.flush(b->pops + cur, tid);
      if (tid == 0) {
        const PopDev* st = b->pops + p;
        P.L = st->L; P.N = st->N; P.h = st->N >> 1; P.Wr = st->Wr; P.rpp = st->rpp; P.npass = st->npass;
        P.kconst = st->kconst;
        P.step = (int)native_step_word(st);
        P.sweeps = energy_only ? 0 : st->sweeps;
        P.nbatch = (st->npass + kKB - 1) / kKB;
        P.tag = kTagMscSweep | (uint32_t)st->pop_id;
        P.T4 = st->thr[(size_t)st->step * kThrPerStep + 10];
        P.T8 = st->thr[(size_t)st->step * kThrPerStep + 11];
        P.seed = st->seed;
        const int rg_prev = (st->R_prev + kMsb - 1) / kMsb;
        P.iseq = st->iseq + (st->step > 0 ? (unsigned long long)rg_prev * kMsb : 0ull);
        P.words = (uint32_t*)st->spins[st->parity];
        P.act = st->active[st->parity];
        P.E = st->E;
        P.M = st->M;
      }
      __syncthreads();
      cur = p;
      const int Wr = P.Wr;
      worker = tid < Wr * P.rpp;
      tx = worker ? tid % Wr : 0;
      rsub = worker ? tid / Wr : 0;
      txl = (tx == 0 ? Wr - 1 : tx - 1);
      txr = (tx + 1 == Wr ? 0 : tx + 1);
      if (tid < kMsb) {
        s_dig[tid] = digit_table(P.T4, P.T8, tid);
      }
    }
    // stripe of a sublattice in shared memory: halo row, LR rows, halo row
    const int h = P.h, Wr = P.Wr, L = P.L, LR = L / CS, SW = LR * Wr, SH = SW + 2 * Wr;
    const int row0 = rank * LR;
    cluster_move_stripe(P, lat, gi, row0, LR, SH, true);
    cluster.sync();
    // halo rows of sublattice X (0: A, 1: B): the last row of the previous
    // stripe and the first row of the next one
    auto fetch_halo = [&](int X) {
      uint32_t* own = lat + X * SH;
      const uint32_t* up = cluster.map_shared_rank(own, prev);
      const uint32_t* dn = cluster.map_shared_rank(own, next);
      for (int v = tid; v < 2 * Wr; v += blockDim.x)
        own[v < Wr ? v : SW + v] = v < Wr ? up[SW + v] : dn[v];
    };

    const int sweeps = P.sweeps;
    for (int sw = 0; sw < sweeps; ++sw) {
#pragma unroll 1
      for (int hf = 0; hf < 2; ++hf) {
        fetch_halo(hf ? 0 : 1);
        __syncthreads();
        uint32_t* self = lat + (hf ? SH : 0) + Wr;
        const uint32_t* oth = lat + (hf ? 0 : SH) + Wr;
        const int rpp = P.rpp, npass = P.npass;
        if (MODE == kRefCoords) {
#pragma unroll 1
          for (int pass = 0; pass < npass; ++pass) {
            const int lr = rsub + pass * rpp;
            const bool valid = worker && lr < LR;
            const int lrc = valid ? lr : 0, ty = row0 + lrc;
            const int row = lrc * Wr, idx = ty * Wr + tx;
            const bool left = (hf == 0) == ((ty & 1) == 0);
            const uint32_t s = self[row + tx];
            const uint32_t n1 = oth[row + (left ? txl : txr)], n2 = oth[row + tx];
            const uint32_t n3 = oth[row - Wr + tx], n4 = oth[row + Wr + tx];
            uint32_t s0, s1, s2;
            adder4(s ^ n1, s ^ n2, s ^ n3, s ^ n4, s0, s1, s2);
            const int t = idx & (kRefThreads - 1), k = idx >> 7;
            const int K = P.kconst ? P.kconst : (t < h ? (h - t + kRefThreads - 1) / kRefThreads : 0);
            const unsigned long long sub = P.iseq + (unsigned long long)t + (unsigned long long)kRefThreads * gi;
            uint32_t ran = ref_word(P.seed, sub, (unsigned long long)sw * 2 * K + (unsigned long long)hf * K + k);
            const uint32_t T4 = P.T4, T8 = P.T8;
            uint32_t c4 = 0, c8 = 0;
#pragma unroll 8
            for (int i = 0; i < kMsb; ++i) {
              c4 |= (ran < T4 ? 1u : 0u) << i;
              c8 |= (ran < T8 ? 1u : 0u) << i;
              ran = kLcgA * ran + kLcgC;
            }
            const uint32_t hi = s1 | s2;
            const uint32_t acc = hi | (~hi & ((s0 & c4) | (~s0 & c8)));
            if (valid) self[row + tx] = s ^ acc;
          }
        } else if (THREADS > 256 && P.L == 256) {
          // L = 256 with every size fixed at compile time: rows of 128 words,
          // THREADS/128 thread rows of kRows consecutive stripe rows each,
          // every offset an immediate (same batches as the general form below);
          // the 256-thread clusters serve L <= 128 only
          constexpr int kW = 128, kLR = 256 / CS, kRpp = THREADS / kW, kRows = kLR / kRpp;
          static_assert(kLR % kRpp == 0 && kRows % kKB == 0, "whole batches");
          const uint32_t c1 = (uint32_t)((sw * 2 + hf) << 4);
          const int vb0 = rsub * kRows;
          // stripes and batches start on even rows: the side neighbour of
          // even rows is x-1 for A, x+1 for B (PAisingMSC.cu:203, 238)
          const uint32_t* txs = oth + (hf == 0 ? txl : txr);
          const uint32_t* txo = oth + (hf == 0 ? txr : txl);
#pragma unroll 1
          for (int p0 = 0; p0 < kRows; p0 += kKB) {
            const int vb = vb0 + p0;
            const uint32_t* po = oth + (vb - 1) * kW + tx;  // stripe rows vb-1 .. vb+4 (halos included)
            uint32_t* ps = self + vb * kW + tx;
            uint32_t av[kKB], un[kKB], ac[kKB], site[kKB];
#pragma unroll
            for (int k = 0; k < kKB; ++k) {
              const uint32_t s = ps[k * kW];
              const uint32_t side = ((k & 1) ? txo : txs)[(vb + k) * kW];
              count_masks(s, side, po[(k + 1) * kW], po[k * kW], po[(k + 2) * kW], av[k], ac[k]);
              un[k] = 0xFFFFFFFFu - ac[k];  // = ~ac, on the FMA pipe
              site[k] = (uint32_t)gi * (uint32_t)h + (uint32_t)((row0 + vb + k) * kW + tx);
            }
            const uint32_t chain = (((uint32_t)gi * CS + (uint32_t)rank) * blockDim.x + (uint32_t)tid) *
                                       (uint32_t)(kRows / kKB) + (uint32_t)(p0 / kKB);
            accept_native(av, un, ac, site, chain, c1, (uint32_t)P.step, P.tag, keys, s_dig, kKB, P.T4, P.T8);
#pragma unroll
            for (int k = 0; k < kKB; ++k) ps[k * kW] ^= ac[k];
          }
        } else if (THREADS == 256 && ((CS == 2 && P.L == 64) || P.L == 128)) {
          // L = 64 (clusters of 2) and 128 on 256-thread CTAs with every size
          // fixed at compile time: rows of kW = L/2 words, THREADS/kW thread
          // rows of kRows consecutive stripe rows (whole batches), rows -1 and
          // LR are the halo rows; same batches, numbering and draws as the
          // general form below, so the same results
          auto fixed = [&](auto l_c) {
            constexpr int kL = decltype(l_c)::value, kW = kL / 2, kLR = kL / CS, kR = THREADS / kW;
            constexpr int kRows = kLR / kR;
            if constexpr (kRows % kKB == 0 && kR * kW == THREADS && kLR % kR == 0) {
              const uint32_t c1 = (uint32_t)((sw * 2 + hf) << 4);
              const int vb0 = rsub * kRows;
              // stripes and batches start on even rows: the side neighbour of
              // even rows is x-1 for A, x+1 for B (PAisingMSC.cu:203, 238)
              const uint32_t* txs = oth + (hf == 0 ? txl : txr);
              const uint32_t* txo = oth + (hf == 0 ? txr : txl);
#pragma unroll 1
              for (int p0 = 0; p0 < kRows; p0 += kKB) {
                const int vb = vb0 + p0;
                const uint32_t* po = oth + (vb - 1) * kW + tx;  // stripe rows vb-1 .. vb+4 (halos included)
                uint32_t* ps = self + vb * kW + tx;
                uint32_t av[kKB], un[kKB], ac[kKB], site[kKB];
#pragma unroll
                for (int k = 0; k < kKB; ++k) {
                  const uint32_t s = ps[k * kW];
                  const uint32_t side = ((k & 1) ? txo : txs)[(vb + k) * kW];
                  count_masks(s, side, po[(k + 1) * kW], po[k * kW], po[(k + 2) * kW], av[k], ac[k]);
                  un[k] = 0xFFFFFFFFu - ac[k];  // = ~ac, on the FMA pipe
                  site[k] = (uint32_t)gi * (uint32_t)h + (uint32_t)((row0 + vb + k) * kW + tx);
                }
                const uint32_t chain = (((uint32_t)gi * CS + (uint32_t)rank) * blockDim.x + (uint32_t)tid) *
                                           (uint32_t)(kRows / kKB) + (uint32_t)(p0 / kKB);
                accept_native(av, un, ac, site, chain, c1, (uint32_t)P.step, P.tag, keys, s_dig, kKB, P.T4, P.T8);
#pragma unroll
                for (int k = 0; k < kKB; ++k) ps[k * kW] ^= ac[k];
              }
            }
          };
          if (P.L == 64) fixed(std::integral_constant<int, 64>());
          else fixed(std::integral_constant<int, 128>());
        } else {
          // thread rsub owns the consecutive stripe rows rsub*npass ..
          // rsub*npass + npass - 1 of column tx: a batch of kKB rows shares
          // the other sublattice's rows around them (halo rows included)
          const uint32_t c1 = (uint32_t)((sw * 2 + hf) << 4);
#pragma unroll 1
          for (int p0 = 0; p0 < npass; p0 += kKB) {
            const int vb = rsub * npass + p0;  // first stripe row of the batch
            uint32_t o[kKB + 2];  // other sublattice, stripe rows vb-1 .. vb+kKB (clamped to the lower halo)
#pragma unroll
            for (int j = 0; j < kKB + 2; ++j) o[j] = oth[min(vb - 1 + j, LR) * Wr + tx];
            const bool left0 = (hf == 0) == (((row0 + vb) & 1) == 0);  // alternates by row
            uint32_t av[kKB], un[kKB], ac[kKB], site[kKB];
            uint32_t vm = 0;  // slots holding a site
#pragma unroll
            for (int k = 0; k < kKB; ++k) {
              const int lr = vb + k;
              const bool valid = worker && p0 + k < npass && lr < LR;
              const int row = min(lr, LR) * Wr;
              const uint32_t s = self[row + tx];
              const uint32_t side = oth[row + ((left0 != ((k & 1) != 0)) ? txl : txr)];
              count_masks(s, side, o[k + 1], o[k], o[k + 2], av[k], ac[k]);
              un[k] = valid ? 0xFFFFFFFFu - ac[k] : 0u;  // = ~ac, on the FMA pipe
              vm |= valid ? 1u << k : 0u;
              site[k] = (uint32_t)gi * (uint32_t)h + (uint32_t)((row0 + lr) * Wr + tx);
            }
            const uint32_t chain =
                (((uint32_t)gi * CS + (uint32_t)rank) * blockDim.x + (uint32_t)tid) * (uint32_t)P.nbatch + (uint32_t)(p0 / kKB);
            accept_native(av, un, ac, site, chain, c1, (uint32_t)P.step, P.tag, keys, s_dig, npass - p0, P.T4, P.T8);
#pragma unroll
            for (int k = 0; k < kKB; ++k)
              if (vm >> k & 1u) self[(vb + k) * Wr + tx] ^= ac[k];
          }
        }
        cluster.sync();
      }
    }

    // energy and magnetisation of this stripe: left and up bond of every A
    // and B site (PAisingMSC.cu:272-294); the up neighbours of the last row
    // are the first row of the next stripe, fetched into the lower halos.
    fetch_halo(0);
    fetch_halo(1);
    __syncthreads();
    cluster_count(P, lat, row0, LR, SH, tx, txl, rsub, worker, s_cntE, s_cntM);
    cluster_move_stripe(P, lat, gi, row0, LR, SH, false);
    cluster.sync();  // all stripes' counts are complete
    if (rank == 0 && tid < kMsb) {
      int ce = 0, cm = 0;
      for (int r = 0; r < CS; ++r) {
        ce += *cluster.map_shared_rank(&s_cntE[tid], r);
        cm += *cluster.map_shared_rank(&s_cntM[tid], r);
      }
      const int N = P.N;
      const int E = 2 * ce - 2 * N, Mg = 2 * cm - N;
      P.E[gi * kMsb + tid] = E;
      P.M[gi * kMsb + tid] = Mg;
      if (P.act[gi * kMsb + tid]) stats.add(tid, E, Mg);
    }
  }
  if (rank == 0 && tid < kMsb && cur >= 0) stats.flush(b->pops + cur, tid);
}

// -------------------------------------------------------------- geometry
bool msc_cluster_geom(int L, int cs, int threads, SweepGeom* g) {
  if (L < 8 || L % 2 != 0 || L > 256 || (cs != 2 && cs != 4) || L % cs != 0) return false;
  const int LR = L / cs;
  if (LR < 2) return false;
  g->L = L;
  g->N = L * L;
  g->half = g->N / 2;
  g->Wr = L / 2;
  if (g->Wr > threads) return false;
  int best = 1;
  for (int r = 1; r <= LR; ++r)
    if (LR % r == 0 && g->Wr * r <= threads) best = r;
  g->rpp = best;
  g->T = g->Wr * g->rpp;
  g->npass = LR / g->rpp;
  g->kconst = (g->half % kRefThreads == 0) ? g->half / kRefThreads : 0;
  g->smem = 2 * (LR + 2) * g->Wr * 4;  // both sublattice stripes with their halo rows
  // stripes are moved with 16-byte vectors: rows start on a 4-word boundary
  return g->Wr % 4 == 0;
}

// -------------------------------------------------------------- launchers
template <int MODE, int CS, int THREADS>
static cudaError_t cluster_launch(BatchDev* b, int energy_only, unsigned long long seed, const SweepLaunch* sl,
                                  SweepLaunch* setup, cudaStream_t s) {
  auto fn = msc_sweep_cluster_kernel<MODE, CS, THREADS>;
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CS;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cfg.blockDim = dim3(THREADS);
  cfg.stream = s;
  if (setup) {  // persistent grid: as many clusters as can be resident
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, setup->smem);
    if (e != cudaSuccess) return e;
    cfg.gridDim = dim3(CS);
    cfg.dynamicSmemBytes = setup->smem;
    int nclusters = 0;
    e = cudaOccupancyMaxActiveClusters(&nclusters, fn, &cfg);
    if (e != cudaSuccess) return e;
    if (nclusters < 1) return cudaErrorInvalidConfiguration;
    setup->grid = nclusters * CS;
    setup->block = THREADS;
    return cudaSuccess;
  }
  cfg.gridDim = dim3(sl->grid);
  cfg.dynamicSmemBytes = sl->smem;
  return cudaLaunchKernelEx(&cfg, fn, b, energy_only, seed);
}

template <int CS, int THREADS>
static cudaError_t cluster_dispatch(int rng_mode, BatchDev* b, int energy_only, unsigned long long seed,
                                    const SweepLaunch* sl, SweepLaunch* setup, cudaStream_t s) {
  return rng_mode == kRefCoords ? cluster_launch<kRefCoords, CS, THREADS>(b, energy_only, seed, sl, setup, s)
                                : cluster_launch<kNative, CS, THREADS>(b, energy_only, seed, sl, setup, s);
}

// Threads per CTA of a cluster: lattices up to L = 128 take 256 (a stripe of
// L/cs rows of L/2 words then gives every thread whole batches of kKB rows,
// as the one-CTA sweep does), larger ones 1024 (clusters of 2) or 512 (4).
int msc_cluster_threads(int cs, int maxL) { return maxL <= 128 ? 256 : cs == 2 ? 1024 : 512; }

cudaError_t msc_cluster_setup(int cs, int threads, int rng_mode, int smem, SweepLaunch* out) {
  out->smem = smem;
  if (cs == 2 && threads == 256) return cluster_dispatch<2, 256>(rng_mode, nullptr, 0, 0, nullptr, out, nullptr);
  if (cs == 4 && threads == 256) return cluster_dispatch<4, 256>(rng_mode, nullptr, 0, 0, nullptr, out, nullptr);
  if (cs == 2 && threads == 1024) return cluster_dispatch<2, 1024>(rng_mode, nullptr, 0, 0, nullptr, out, nullptr);
  if (cs == 4 && threads == 512) return cluster_dispatch<4, 512>(rng_mode, nullptr, 0, 0, nullptr, out, nullptr);
  return cudaErrorInvalidValue;
}

cudaError_t launch_msc_cluster_sweep(int cs, int threads, BatchDev* b, int rng_mode, int energy_only,
                                     unsigned long long seed, const SweepLaunch& sl, cudaStream_t s) {
  if (cs == 2 && threads == 256) return cluster_dispatch<2, 256>(rng_mode, b, energy_only, seed, &sl, nullptr, s);
  if (cs == 4 && threads == 256) return cluster_dispatch<4, 256>(rng_mode, b, energy_only, seed, &sl, nullptr, s);
  if (cs == 2 && threads == 1024) return cluster_dispatch<2, 1024>(rng_mode, b, energy_only, seed, &sl, nullptr, s);
  if (cs == 4 && threads == 512) return cluster_dispatch<4, 512>(rng_mode, b, energy_only, seed, &sl, nullptr, s);
  return cudaErrorInvalidValue;
}

}  // namespace pa
