// Transport engine: kernels, resident device state and the omc_engine_*
// C ABI (include/omc_gpu.h).
//
// One run = nbatch launches of the persistent transport kernel, each
// transporting nperbatch histories, each followed by the batch
// accumulation (accumEndep, omc_dosxyz.c:696-717).  A lane (CUDA thread)
// owns one RANMAR stream, seeded like the reference's OpenMP threads, and
// one particle stack; lanes take histories from a global counter, the GPU
// form of "#pragma omp parallel for schedule(dynamic)"
// (omc_dosxyz.c:1252).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../host/common.h"
#include "physics.cuh"

using namespace omcgpu;
using omc::fail;

namespace {

constexpr int kBlock = 128;  // lanes per block
// Shared memory of a block: the RANMAR states of its lanes, 3 bytes a word.
constexpr size_t kRngSmem = static_cast<size_t>(RNG_WORDS) * kBlock * 3;
// Blocks per SM the register budget is sized for, measured on the 6 MV
// slab.  Wavefront kernel, with electrons near a boundary in their own
// queue (before the photon flight cap): FP32 5 blocks (96 registers)
// 8.39e7 hist/s, against 8.23e7 with
// 4; FP64 2 blocks (248 registers) 7.04e6 at 96 particles per thread in
// flight, against 6.88e6 with 3 blocks (168 registers) and 6.90e6 with 4
// (128 registers, 368 bytes of spills) at the same number in flight.
// Per-lane kernel: 5 and 3.
#ifndef OMC_MIN_BLOCKS_FP32
#define OMC_MIN_BLOCKS_FP32 5
#endif
#ifndef OMC_MIN_BLOCKS_FP64
#define OMC_MIN_BLOCKS_FP64 3
#endif
#ifndef OMC_WF_MIN_BLOCKS_FP64
#define OMC_WF_MIN_BLOCKS_FP64 2
#endif
template <typename R>
struct Occupancy {
  static constexpr int kMinBlocks = sizeof(R) == 4 ? OMC_MIN_BLOCKS_FP32 : OMC_MIN_BLOCKS_FP64;
  static constexpr int kWavefrontMinBlocks = sizeof(R) == 4 ? OMC_MIN_BLOCKS_FP32 : OMC_WF_MIN_BLOCKS_FP64;
};
constexpr int kDefaultDepth = 48;
// History-by-history block pool: blocks per particle in flight, times 2.
#ifndef OMC_HBH_POOL_X2
#define OMC_HBH_POOL_X2 6
#endif

#define CUDA_TRY(expr)                                                                           \
  do {                                                                                           \
    cudaError_t e_ = (expr);                                                                     \
    if (e_ != cudaSuccess) return fail(OMC_ERR_CUDA, "%s: %s", #expr, cudaGetErrorString(e_)); \
  } while (0)

// ---------------------------------------------------------------------------
// Kernels.
// ---------------------------------------------------------------------------
__global__ void seed_kernel(int ixx, int jxx, int nlanes, int *rng_u, int *rng_ijc) {
  int lane = blockIdx.x * blockDim.x + threadIdx.x;
  if (lane >= nlanes) return;
  int ik, jk;
  stream_seeds(ixx, jxx, lane, &ik, &jk);
  ranmar_seed(ik, jk, rng_u + lane, nlanes);
  rng_ijc[lane] = 97;
  rng_ijc[nlanes + lane] = 33;
  rng_ijc[2 * nlanes + lane] = 362436;
}

__global__ void ranmar_draw_kernel(int nlanes, long long n, int *rng_u, int *rng_ijc, int *out) {
  int lane = blockIdx.x * blockDim.x + threadIdx.x;
  if (lane >= nlanes) return;
  RanmarGlobal r;
  r.u = rng_u + lane;
  r.stride = nlanes;
  r.i = rng_ijc[lane];
  r.j = rng_ijc[nlanes + lane];
  r.c = rng_ijc[2 * nlanes + lane];
  for (long long k = 0; k < n; k++) out[static_cast<size_t>(lane) * n + k] = r.next_int();
  rng_ijc[lane] = r.i;
  rng_ijc[nlanes + lane] = r.j;
  rng_ijc[2 * nlanes + lane] = r.c;
}

// Shared-memory RANMAR planes of a block: [97][kBlock] low halves, then
// [97][kBlock] high bytes.
struct RngPlanes {
  unsigned short *lo;
  unsigned char *hi;
};
__device__ __forceinline__ RngPlanes rng_planes(unsigned char *smem) {
  return RngPlanes{reinterpret_cast<unsigned short *>(smem), smem + static_cast<size_t>(RNG_WORDS) * kBlock * 2};
}
__device__ __forceinline__ void rng_to_smem(const int *g, int nlanes, int gl, RngPlanes s, int t) {
  for (int k = 0; k < RNG_WORDS; k++) {
    int v = g[static_cast<size_t>(k) * nlanes + gl];
    s.lo[k * kBlock + t] = static_cast<unsigned short>(v & 0xffff);
    s.hi[k * kBlock + t] = static_cast<unsigned char>(v >> 16);
  }
}
__device__ __forceinline__ void rng_from_smem(int *g, int nlanes, int gl, RngPlanes s, int t) {
  for (int k = 0; k < RNG_WORDS; k++)
    g[static_cast<size_t>(k) * nlanes + gl] =
        static_cast<int>(s.lo[k * kBlock + t]) | (static_cast<int>(s.hi[k * kBlock + t]) << 16);
}

template <typename R>
__global__ void __launch_bounds__(kBlock, Occupancy<R>::kMinBlocks) transport_kernel(Params<R> P) {
  extern __shared__ unsigned char s_raw[];
  const int t = threadIdx.x;
  const int lane = blockIdx.x * kBlock + t;
  if (lane >= P.nlanes) return;
  RngPlanes sp = rng_planes(s_raw);
  rng_to_smem(P.rng_u, P.nlanes, lane, sp, t);
  Lane<R, false> L(P, lane, sp.lo + t, sp.hi + t, kBlock);
  L.rng.i = P.rng_ijc[lane];
  L.rng.j = P.rng_ijc[P.nlanes + lane];
  L.rng.c = P.rng_ijc[2 * P.nlanes + lane];
  unsigned long long events = 0;
  long long hist_events = 0;
  for (;;) {
    if (L.np < 0) {
      unsigned long long h = atomicAdd(P.next, 1ull);
      if (h >= static_cast<unsigned long long>(P.nhist)) break;
      L.init_history(static_cast<long long>(h));
      hist_events = 0;
    }
    if (L.p.iq == 0) L.photon_event();
    else L.electron_event();
    events++;
    if (++hist_events > kEventCap) {
      L.err |= ERR_EVENTS;
      L.np = -1;
    }
  }
  rng_from_smem(P.rng_u, P.nlanes, lane, sp, t);
  P.rng_ijc[lane] = L.rng.i;
  P.rng_ijc[P.nlanes + lane] = L.rng.j;
  P.rng_ijc[2 * P.nlanes + lane] = L.rng.c;
  atomicAdd(P.ensrc, L.ensrc);
  atomicAdd(P.events, events);
  atomicAdd(P.n_geom, L.n_geom);
  atomicAdd(P.n_dep, L.n_dep);
  atomicMax(P.max_np, L.max_np);
  if (L.err) atomicOr(P.err, L.err);
}

// ---------------------------------------------------------------------------
// Wavefront schedule.  One cooperative, persistent launch per batch; every
// thread keeps its RANMAR stream in shared memory for the whole batch.
// Iteration: read the queue counters (identical in every thread), then one
// phase in which warps claim 32-wide chunks of [new histories | photons |
// electrons] until none is left, then one grid barrier.  Queue buffers
// alternate between iterations; counters rotate over three slots so a slot
// is zeroed only when no phase reads or appends it.
// ---------------------------------------------------------------------------
template <typename R>
struct Wavefront {
  R *ph_f[2];
  int *ph_k[2];
  R *el_f[2];
  int *el_k[2];
  int *ph_s[2], *el_s[2]; // tally slot per queued particle (beamlet jobs), else null
  R *ei_f[2];             // electrons waiting for a discrete interaction
  int *ei_k[2];
  int *ei_s[2];
  R *pi_f[2];             // photons waiting for their interaction
  int *pi_k[2];
  int *pi_s[2];
  R *ph_t[2];             // photon flights: mean free paths left (-1: a new flight)
  unsigned cap;           // slots per queue
  unsigned *ctr;          // [0..2] photon, [3..5] electron, [6..8] electron-interaction,
                          // [9..11] photon-interaction, [12..14] boundary-electron counters
                          // (boundary electrons fill the electron queue from the top)
  unsigned long long *work;      // [3] chunk counters of the phase
  unsigned long long *injected;  // [2] histories injected before the iteration
  unsigned *bar_arrive;
  unsigned *bar_gen;
  unsigned target;        // particles kept in flight
  int max_iters;
  int *iters;             // iterations used (output)
  unsigned *hwm;          // queue high-water mark (output)
  unsigned long long *trace;  // per iteration {ns, photons, electrons, injected}, or null
  int trace_cap;              // iterations the trace holds
  int chunk_events;           // electron steps per take before re-queueing
  unsigned long long drain_below;  // drain mode below this many particles in flight
  // history-by-history scoring: pool counters {pushed, popped} as an
  // iteration ended ([2][2] by iteration parity, written in the barrier)
  // and the blocks an iteration keeps back for continuation blocks
  unsigned long long *hbh_free;
  unsigned long long hbh_reserve;
  int flight_cap;          // voxel crossings of a photon flight per event (nsplit = 1)
};

constexpr int kDefaultChunkEvents = 1;

// End-of-run drain: once every history is injected and fewer than
// kDrainPerWarp particles per 32 threads are in flight, the GPU is short
// of work and each particle's remaining events would take one iteration
// each.  Electron interactions then run inline and an electron take runs up
// to kDrainSteps condensed-history steps, so a track ends in one iteration.
// Above that the one-step takes keep warps full, which is worth more.
// Measured on the 6 MV slab, 10 batches in one launch, job time against no
// drain mode: 32 per warp FP32 3.4% and FP64 8.7% shorter; 8 per warp FP32
// 2.0% shorter; 128 per warp FP32 0.7% shorter but FP64 12% longer.
constexpr int kDrainPerWarp = 32;
constexpr int kDrainSteps = 4096;

template <typename R>
constexpr unsigned long long kInflightPerThread = sizeof(R) == 4 ? 128 : 96;

// Voxel crossings of a photon flight per event (nsplit = 1), measured on the
// 6 MV slab (hist/s): FP32 9.52e7 / 9.72e7 / 9.63e7 / 9.20e7 at 8 / 16 / 32
// / 64, against 8.40e7 with flights run to their end; FP64 7.25e6 / 7.41e6
// / 7.48e6 / 7.36e6, against 7.03e6.
template <typename R>
constexpr int kFlightCap = sizeof(R) == 4 ? 16 : 32;

constexpr long long kBarrierSpinCap = 1ll << 28;  // x ~64 ns: well past any phase

// Grid-wide barrier for a cooperative launch (all blocks co-resident).  The
// wait is bounded: on timeout the error flag is set and the block goes on,
// so the kernel always ends.
// snap_src/snap_dst (optional): the last block to arrive -- when every
// other block has finished the iteration -- copies two counters to
// snap_dst before it releases the others, so the next iteration reads
// values that no thread changes any more.
__device__ bool grid_barrier(unsigned *arrive, unsigned *gen, unsigned nblocks,
                             const unsigned long long *snap_src = nullptr, unsigned long long *snap_dst = nullptr) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    s_ok = 1;
    volatile unsigned *vgen = gen;
    unsigned g = *vgen;
    __threadfence();
    if (atomicAdd(arrive, 1u) == nblocks - 1) {
      if (snap_src) {
        __threadfence();
        snap_dst[0] = *static_cast<const volatile unsigned long long *>(snap_src);
        snap_dst[1] = *static_cast<const volatile unsigned long long *>(snap_src + 1);
      }
      atomicExch(arrive, 0u);
      __threadfence();
      atomicAdd(gen, 1u);
    } else {
      long long spins = 0;
      while (*vgen == g) {
        __nanosleep(64);
        if (++spins > kBarrierSpinCap) {
          s_ok = 0;
          break;
        }
      }
    }
    __threadfence();
  }
  __syncthreads();
  return s_ok != 0;
}

__device__ __forceinline__ unsigned vload(const unsigned *p) { return *static_cast<const volatile unsigned *>(p); }

template <typename R, bool MULTI, bool HBH = false>
__global__ void __launch_bounds__(kBlock, Occupancy<R>::kWavefrontMinBlocks) wavefront_kernel(Params<R> P, Wavefront<R> W) {
  extern __shared__ unsigned char s_raw[];
  const int t = threadIdx.x;
  const int gtid = blockIdx.x * kBlock + t;
  const int lane_id = t & 31;
  RngPlanes sp = rng_planes(s_raw);
  rng_to_smem(P.rng_u, P.nlanes, gtid, sp, t);
  Lane<R, true, MULTI, HBH> L(P, gtid, sp.lo + t, sp.hi + t, kBlock);
  if constexpr (HBH) {
    // Each warp's table for merging a completed history's deposits.
    __shared__ int s_hir[kBlock / 32][kHbhRegions];
    __shared__ double s_hx[kBlock / 32][kHbhRegions];
    L.hbh_tir = s_hir[t >> 5];
    L.hbh_tx = s_hx[t >> 5];
  }
  L.rng.i = P.rng_ijc[gtid];
  L.rng.j = P.rng_ijc[P.nlanes + gtid];
  L.rng.c = P.rng_ijc[2 * P.nlanes + gtid];
  L.queue_cap = W.cap;
  // Photon and discrete electron interactions run in their own chunks
  // (measured on the 6 MV slab: electrons FP32 2.85e7 -> 3.10e7 and FP64
  // 2.02e6 -> 2.22e6 hist/s; photons then 3.96e7 -> 4.29e7).
  L.defer_interactions = true;
  unsigned long long events = 0;
  int it = 0;
  for (; it < W.max_iters; it++) {
    const int bin = it & 1, bout = bin ^ 1;
    const int cin = it % 3, cout = (it + 1) % 3, cfree = (it + 2) % 3;
    // Everything below is read after the last barrier, so every thread
    // sees the same values and takes the same branches.
    // A counter counts the appends that did not fit too (they set
    // ERR_QUEUE): the reads below stay inside the queues.  The two ends of
    // the electron queue must not have met, else records were overwritten.
    const unsigned n_ph = min(vload(W.ctr + cin), W.cap);
    const unsigned n_el = min(vload(W.ctr + 3 + cin), W.cap);
    const unsigned n_ei = min(vload(W.ctr + 6 + cin), W.cap);
    const unsigned n_pi = min(vload(W.ctr + 9 + cin), W.cap);
    const unsigned n_eb = min(vload(W.ctr + 12 + cin), W.cap - n_el);
    if (gtid == 0 && static_cast<unsigned long long>(vload(W.ctr + 3 + cin)) + vload(W.ctr + 12 + cin) > W.cap)
      L.err |= ERR_QUEUE;
    const unsigned long long injected = *static_cast<volatile unsigned long long *>(W.injected + bin);
    const long long remaining = P.nhist - static_cast<long long>(injected);
    const unsigned long long inflight = static_cast<unsigned long long>(n_ph) + n_el + n_ei + n_pi + n_eb;
    if (W.trace && gtid == 0 && it < W.trace_cap) {
      unsigned long long ns;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(ns));
      unsigned long long *r = W.trace + 4 * static_cast<size_t>(it);
      r[0] = ns;
      r[1] = n_ph;
      r[2] = n_el + n_eb;
      r[3] = injected;
    }
    if (remaining <= 0 && inflight == 0) break;
    const bool drain = remaining <= 0 && inflight < W.drain_below;
    long long m = static_cast<long long>(W.target) - static_cast<long long>(inflight);
    if (m < 0) m = 0;
    if (m > remaining) m = remaining;
    if constexpr (HBH) {
      // Pool counters as the last iteration ended (snapshot taken in the
      // barrier): ring entries below the push count are written, and the
      // free blocks are exact.  A new history needs a head block; some
      // blocks are kept for continuations.
      const unsigned long long *snap = W.hbh_free + 2 * bin;
      const unsigned long long pushed = *static_cast<const volatile unsigned long long *>(snap);
      const unsigned long long popped = *static_cast<const volatile unsigned long long *>(snap + 1);
      L.hbh_pop_limit = pushed;
      const long long nfree = static_cast<long long>(pushed - popped) - static_cast<long long>(W.hbh_reserve);
      if (m > nfree) m = nfree > 0 ? nfree : 0;
    }
    if (gtid == 0) {
      W.ctr[cfree] = 0;
      W.ctr[3 + cfree] = 0;
      W.ctr[6 + cfree] = 0;
      W.ctr[9 + cfree] = 0;
      W.ctr[12 + cfree] = 0;
      W.work[cfree] = 0;
      W.injected[bout] = injected + static_cast<unsigned long long>(m);
    }
    // One phase: new histories, then photons, then electrons, each range
    // padded to a multiple of 32 so that a warp's chunk is one code path.
    // Everything produced goes to the next iteration's queues.
    L.out = EmitTargets<R>{W.ph_f[bout], W.ph_k[bout], W.ctr + cout,     W.el_f[bout], W.el_k[bout],
                           W.ctr + 3 + cout, W.ph_s[bout], W.el_s[bout],     W.ei_f[bout], W.ei_k[bout],
                           W.ctr + 6 + cout, W.ei_s[bout], W.pi_f[bout],     W.pi_k[bout], W.ctr + 9 + cout,
                           W.pi_s[bout], W.ctr + 12 + cout, W.ph_t[bout]};
    // In the drain a flight runs to its end: the GPU is short of work and
    // every re-queued photon would cost an iteration.
    L.flight_cap = drain ? kNoFlightCap : W.flight_cap;
    // Chunk ranges of the phase in claim order [new histories | photon
    // flights | photon interactions | electron steps | electron steps near
    // a boundary | electron interactions], each padded to a multiple of 32
    // so that a warp's chunk is one code path.  (Claiming the electron
    // steps first, largest work first, measured 3% slower.)
    const unsigned long long el_pad = (static_cast<unsigned long long>(n_el) + 31) & ~31ull;
    const unsigned long long ph_pad = (static_cast<unsigned long long>(n_ph) + 31) & ~31ull;
    const unsigned long long pi_pad = (static_cast<unsigned long long>(n_pi) + 31) & ~31ull;
    const unsigned long long ei_pad = (static_cast<unsigned long long>(n_ei) + 31) & ~31ull;
    const unsigned long long eb_pad = (static_cast<unsigned long long>(n_eb) + 31) & ~31ull;
    const unsigned long long r_in = 0, r_ph = r_in + ((static_cast<unsigned long long>(m) + 31) & ~31ull),
                             r_pi = r_ph + ph_pad, r_el = r_pi + pi_pad, r_eb = r_el + el_pad, r_ei = r_eb + eb_pad,
                             total = r_ei + ei_pad;
    for (;;) {
      unsigned long long base = 0;
      if (lane_id == 0) base = atomicAdd(W.work + cin, 32ull);
      base = __shfl_sync(0xffffffffu, base, 0);
      if (base >= total) break;
      const unsigned long long i = base + lane_id;
      if (base >= r_in && base < r_in + ((static_cast<unsigned long long>(m) + 31) & ~31ull)) {
        const unsigned long long k = i - r_in;
        if (k < static_cast<unsigned long long>(m)) {
          L.init_history(static_cast<long long>(injected + k));
          if constexpr (HBH) L.hbh_start();
          L.emit(L.p);
          if constexpr (HBH) L.hbh_finish(0);
        }
      } else if (base >= r_ph && base < r_ph + ph_pad) {
        const unsigned long long k = i - r_ph;
        if (k < n_ph) {
          L.take(W.ph_f[bin], W.ph_k[bin], static_cast<unsigned>(k), W.ph_s[bin]);
          L.taken_mfp = __ldcg(W.ph_t[bin] + k);
          L.wf_photon_event();
          events++;
          if constexpr (HBH) L.hbh_finish(1);
        }
      } else if (base >= r_pi && base < r_pi + pi_pad) {
        const unsigned long long k = i - r_pi;
        if (k < n_pi) {
          L.take(W.pi_f[bin], W.pi_k[bin], static_cast<unsigned>(k), W.pi_s[bin]);
          const bool survivor = L.p.iq == 2;
          L.p.iq = 0;
          L.deferred_photon_interaction(survivor);
          if constexpr (HBH) L.hbh_finish(1);
        }
      } else if (base >= r_el && base < r_eb + eb_pad) {
        // A chunk lies in one of the two electron ranges.
        const bool nb = base >= r_eb;
        const unsigned long long k = i - (nb ? r_eb : r_el);
        if (k < (nb ? n_eb : n_el)) {
          // Up to chunk_events iterations of electron()'s tstep loop on
          // this electron; it goes back to a queue if it is still alive
          // (or if an interaction left a photon on top), to the
          // interaction queue if its step ended at a deferred interaction.
          // In the drain the interaction runs at once and the take goes on
          // with whatever electron is left on top.
          L.take(W.el_f[bin], W.el_k[bin], nb ? W.cap - 1 - static_cast<unsigned>(k) : static_cast<unsigned>(k),
                 W.el_s[bin]);
          L.pending_interaction = false;
          int n = 0;
          do {
            L.electron_event();
            events++;
            if (drain && L.pending_interaction) {
              L.pending_interaction = false;
              L.deferred_interaction();
            }
          } while (L.alive && !L.pending_interaction && L.p.iq != 0 && ++n < (drain ? kDrainSteps : W.chunk_events));
          if (L.alive) {
            if (L.pending_interaction) L.emit_pending();
            else L.emit_step(L.p);
          }
          if constexpr (HBH) L.hbh_finish(1);
        }
      } else {
        const unsigned long long k = i - r_ei;
        if (k < n_ei) {
          L.take(W.ei_f[bin], W.ei_k[bin], static_cast<unsigned>(k), W.ei_s[bin]);
          L.deferred_interaction();
          if (L.alive) L.emit(L.p);
          if constexpr (HBH) L.hbh_finish(1);
        }
      }
      // Every lane of the warp is here (a chunk is one code path): the warp
      // merges the histories its lanes just completed.
      if constexpr (HBH) L.hbh_warp_merge();
    }
    bool bar_ok;
    if constexpr (HBH) bar_ok = grid_barrier(W.bar_arrive, W.bar_gen, gridDim.x, P.hbh.ctr, W.hbh_free + 2 * bout);
    else bar_ok = grid_barrier(W.bar_arrive, W.bar_gen, gridDim.x);
    if (!bar_ok) L.err |= ERR_BARRIER;
  }
  if (it >= W.max_iters) L.err |= ERR_LOOP;
  rng_from_smem(P.rng_u, P.nlanes, gtid, sp, t);
  P.rng_ijc[gtid] = L.rng.i;
  P.rng_ijc[P.nlanes + gtid] = L.rng.j;
  P.rng_ijc[2 * P.nlanes + gtid] = L.rng.c;
  atomicAdd(P.ensrc, L.ensrc);
  atomicAdd(P.events, events);
  atomicAdd(P.n_geom, L.n_geom);
  atomicAdd(P.n_dep, L.n_dep);
  atomicMax(W.hwm, L.queue_hwm);
  if constexpr (HBH) {
    if (L.hbh_merged) atomicAdd(P.hbh.histories, L.hbh_merged);
    if (L.hbh_split) atomicAdd(P.hbh.split, L.hbh_split);
  }
  if (gtid == 0) *W.iters = it;
  if (L.err) atomicOr(P.err, L.err);
}

// Batch statistics: accum += e, accum2 += e^2, e = 0.
__global__ void accumulate_kernel(double *endep, double *acc, double *acc2, long long n) {
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    double e = endep[i];
    acc[i] += e;
    acc2[i] += e * e;
    endep[i] = 0.0;
  }
}

// ---------------------------------------------------------------------------
// Dose-influence matrix (omc_matrad.c:839-919 and :1426-1482), one tally
// slot per beamlet: dose in place, slot maximum, then threshold and an
// order-preserving compaction into CSC columns.  Tiles of kDijTile voxels
// are counted, the counts scanned, and each tile written in 16 coalesced
// rounds of 256 voxels.
// ---------------------------------------------------------------------------
constexpr int kDijThreads = 256;
constexpr int kDijRounds = 16;
constexpr int kDijTile = kDijThreads * kDijRounds;

// Per-voxel dose factor, once per tally group, in the reference's
// operation order (omc_matrad.c:868-882): mass = dx*dy*dz*rho, factor =
// 1.602e-10 / (mass * nhist) when every beamlet of the group has nhist
// histories, else 1.602e-10 / mass (the beamlet's 1/nhist is applied per
// element); zero below 0.044 g/cm^3, where the reference zeroes the dose.
__global__ void dij_factor_kernel(long long nvox, int nx, int ny, const double *xb, const double *yb, const double *zb,
                                  const double *density, double nhist, double *factor) {
  for (long long v = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; v < nvox;
       v += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int ix = static_cast<int>(v % nx);
    const long long r = v / nx;
    const int iy = static_cast<int>(r % ny);
    const int iz = static_cast<int>(r / ny);
    double mass = __dmul_rn(__dmul_rn(__dsub_rn(xb[ix + 1], xb[ix]), __dsub_rn(yb[iy + 1], yb[iy])),
                            __dsub_rn(zb[iz + 1], zb[iz]));
    const double rho = density[v];
    mass = __dmul_rn(mass, rho);
    double f = nhist > 0.0 ? __ddiv_rn(1.602E-10, __dmul_rn(mass, nhist)) : __ddiv_rn(1.602E-10, mass);
    if (rho < 0.044) f = 0.0;
    factor[v] = f;
  }
}

// Energy to dose in place, (sum / nbatch) * factor, and each slot's
// maximum.  Grid: x over voxels, y over slots.  When the beamlets of the
// group have different history counts, the factor leaves out 1/nhist: it
// is a positive constant of the slot, so the maximum and the threshold
// test are taken on the unscaled values and only the kept entries are
// scaled (dij_fill_kernel), one FP64 multiply per entry instead of one per
// voxel.
__global__ void dij_dose_kernel(double *__restrict__ tally, long long nreg, const double *__restrict__ factor,
                                int nbatch, unsigned long long *__restrict__ slot_max) {
  const int s = blockIdx.y;
  double *__restrict__ t = tally + static_cast<size_t>(s) * nreg + 1;
  const long long nvox = nreg - 1;
  const double nb = static_cast<double>(nbatch);
  // The maximum is taken on the bit patterns as signed 64-bit integers
  // (non-negative doubles order like their bits; -0.0 and negative values
  // fall below every non-negative one): the FP64 pipe of this GPU is narrow
  // and the conversion itself has to use it.  Four independent elements
  // per thread and round keep several loads in flight.
  long long m = 0;
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  for (long long v0 = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; v0 < nvox; v0 += 4 * stride) {
    double e[4], f[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const long long v = v0 + k * stride;
      e[k] = v < nvox ? t[v] : 0.0;
      f[k] = v < nvox ? __ldg(factor + v) : 0.0;
    }
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const long long v = v0 + k * stride;
      if (v >= nvox) break;
      double endep = e[k];
      if (nbatch != 1) endep = __ddiv_rn(endep, nb);
      endep = __dmul_rn(endep, f[k]);
      t[v] = endep;
      m = max(m, __double_as_longlong(endep));
    }
  }
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0 && m > 0) atomicMax(slot_max + s, static_cast<unsigned long long>(m));
}

// The threshold of slot s as the bit pattern of a non-negative double:
// t > threshold compares as signed 64-bit integers (see dij_dose_kernel).
__device__ __forceinline__ long long slot_threshold(const unsigned long long *slot_max, int s, double rel) {
  return __double_as_longlong(__dmul_rn(__longlong_as_double(static_cast<long long>(slot_max[s])), rel));
}

// Entries above the threshold per tile.  Grid: x over tiles, y over slots.
__global__ void dij_count_kernel(const double *tally, long long nreg, int ntiles, const unsigned long long *slot_max,
                                 double rel, long long *tile_count) {
  __shared__ int red[kDijThreads / 32];
  const int s = blockIdx.y;
  const long long thresh = slot_threshold(slot_max, s, rel);
  const long long *t = reinterpret_cast<const long long *>(tally + static_cast<size_t>(s) * nreg + 1);
  const long long nvox = nreg - 1;
  const long long v0 = static_cast<long long>(blockIdx.x) * kDijTile;
  int c = 0;
  for (int r = 0; r < kDijRounds; r++) {
    long long v = v0 + r * kDijThreads + threadIdx.x;
    if (v < nvox && t[v] > thresh) c++;
  }
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    long long sum = 0;
    for (int w = 0; w < kDijThreads / 32; w++) sum += red[w];
    tile_count[static_cast<size_t>(s) * ntiles + blockIdx.x] = sum;
  }
}

// Exclusive scan of n counts by one block of 1024 threads; off[n] = total.
__global__ void dij_scan_kernel(const long long *cnt, long long n, long long *off) {
  __shared__ long long part[1024];
  const int t = threadIdx.x;
  const long long per = (n + 1023) / 1024;
  const long long lo = t * per, hi = lo + per < n ? lo + per : n;
  long long sum = 0;
  for (long long i = lo; i < hi; i++) sum += cnt[i];
  part[t] = sum;
  __syncthreads();
  for (int d = 1; d < 1024; d <<= 1) {
    long long v = t >= d ? part[t - d] : 0;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  long long run = part[t] - sum;
  for (long long i = lo; i < hi; i++) {
    off[i] = run;
    run += cnt[i];
  }
  if (t == 1023) off[n] = part[1023];
}

// Rows (voxel index = region - 1) and values of the kept entries, in voxel
// order within each slot.
__global__ void dij_fill_kernel(const double *tally, long long nreg, int ntiles, const unsigned long long *slot_max,
                                double rel, const long long *off, const double *slot_inv_nhist, int *rows,
                                double *vals, float *vals32) {
  __shared__ int wtot[kDijThreads / 32];
  const int s = blockIdx.y;
  const double inv_nh = slot_inv_nhist ? slot_inv_nhist[s] : 1.0;
  const long long thresh = slot_threshold(slot_max, s, rel);
  const double *t = tally + static_cast<size_t>(s) * nreg + 1;
  const long long nvox = nreg - 1;
  const long long v0 = static_cast<long long>(blockIdx.x) * kDijTile;
  long long base = off[static_cast<size_t>(s) * ntiles + blockIdx.x];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int r = 0; r < kDijRounds; r++) {
    const long long v = v0 + r * kDijThreads + threadIdx.x;
    double d = 0.0;
    bool keep = false;
    if (v < nvox) {
      d = t[v];
      keep = __double_as_longlong(d) > thresh;
    }
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    if (lane == 0) wtot[warp] = __popc(m);
    __syncthreads();
    int wbase = 0, tot = 0;
    for (int w = 0; w < kDijThreads / 32; w++) {
      const int c = wtot[w];
      if (w < warp) wbase += c;
      tot += c;
    }
    if (keep) {
      const long long o = base + wbase + __popc(m & lanemask_lt());
      if (slot_inv_nhist) d = __dmul_rn(d, inv_nh);
      rows[o] = static_cast<int>(v);
      if (vals) vals[o] = d;
      else vals32[o] = static_cast<float>(d);
    }
    base += tot;
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Device memory helpers.
// ---------------------------------------------------------------------------
struct DevBuf {
  void *p = nullptr;
  size_t n = 0;
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  omc_status ensure(size_t bytes) {
    if (n >= bytes && p) return OMC_OK;
    release();
    if (cudaMalloc(&p, bytes) != cudaSuccess) {
      p = nullptr;
      return fail(OMC_ERR_NOMEM, "cudaMalloc of %zu bytes failed", bytes);
    }
    n = bytes;
    return OMC_OK;
  }
};

// A set of device arrays converted from host doubles to R.
template <typename R>
struct DevArrays {
  std::vector<DevBuf> bufs;
  void clear() {
    for (auto &b : bufs) b.release();
    bufs.clear();
  }
  const R *put(const double *src, size_t n) {
    std::vector<R> h(n ? n : 1);
    for (size_t i = 0; i < n; i++) h[i] = static_cast<R>(src[i]);
    DevBuf b;
    if (b.ensure(h.size() * sizeof(R)) != OMC_OK) return nullptr;
    cudaMemcpy(b.p, h.data(), n * sizeof(R), cudaMemcpyHostToDevice);
    bufs.push_back(b);
    return static_cast<const R *>(b.p);
  }
  const V4<R> *put4(const std::vector<V4<R>> &h) {
    DevBuf b;
    if (b.ensure((h.size() ? h.size() : 1) * sizeof(V4<R>)) != OMC_OK) return nullptr;
    cudaMemcpy(b.p, h.data(), h.size() * sizeof(V4<R>), cudaMemcpyHostToDevice);
    bufs.push_back(b);
    return static_cast<const V4<R> *>(b.p);
  }
  const int *put_int(const int *src, size_t n) {
    DevBuf b;
    if (b.ensure((n ? n : 1) * sizeof(int)) != OMC_OK) return nullptr;
    cudaMemcpy(b.p, src, n * sizeof(int), cudaMemcpyHostToDevice);
    bufs.push_back(b);
    return static_cast<const int *>(b.p);
  }
};

template <typename R>
struct PrecisionState {
  DevArrays<R> tables, geom, source;
  Tables<R> T{};
  Geometry<R> G{};
  Source<R> S{};
  DevBuf stk, key;
  DevBuf queue;  // wavefront: 4 queues of 8 planes + keys (+ slot tags)
  bool tables_ok = false, geom_ok = false, source_ok = false;
  // beamlet source (omc_engine_set_beamlets)
  DevArrays<R> beamlets;
  const R *bixel = nullptr, *beam_src = nullptr;
  const int *ibeam = nullptr;
};

// Histories of one launch spread over tally slots (beamlet jobs).
struct SlotJob {
  int nslots;
  const long long *first;  // device [nslots+1]
  const int *beamlet;      // device [nslots] (beamlet jobs), else null
  double *tally;           // device [nslots][nreg] (beamlet and batch jobs), else null
  long long nhist;         // histories of the launch
  const void *jobs;        // device JobSlot<R>[nslots] (multi-job launches), else null
  bool beamlets = true;    // slots are beamlets (false: batches of one job)
};

}  // namespace

struct omc_engine {
  int device = 0;
  int nsm = 0;
  cudaStream_t stream = nullptr;
  PrecisionState<double> f64;
  PrecisionState<float> f32;
  // geometry scalars
  int nreg = 0;
  // per-lane RNG state
  DevBuf rng_u, rng_ijc;
  int seeded_lanes = 0;  // lane count the current streams were seeded for
  // tallies and counters
  DevBuf endep, acc, acc2, counters, wf_counters;
  // voxel densities (FP64) for the dose conversion of beamlet jobs
  DevBuf density;
  int nbeamlets = 0, nbeams = 0;
  // beamlet-job buffers
  DevBuf dij_tally, dij_first, dij_beamlet, dij_nhist, dij_max, dij_cnt, dij_off, dij_rows, dij_vals, dij_factor;
  // multi-job rounds
  DevBuf multi_slots, multi_first;
  // batch tallies when all batches of a run share one launch
  DevBuf batch_tally, batch_first;
  int batch_tallies = 0;  // batches whose tallies the last run left in batch_tally (0: none)
  DevBuf weights, batch_dot;
  // history-by-history scoring: block pool, rings, counters, sums
  DevBuf hbh_blocks, hbh_ring, hbh_ctr, hbh_sum, hbh_sum2;
  bool hbh_valid = false;  // the last run tracked histories
  long long hbh_histories = 0, hbh_split = 0;
  // per-iteration trace of the last wavefront launch (diagnostics)
  DevBuf trace;
  int trace_cap = 0;
  int trace_iters = 0;
  // host copies needed across uploads
  omc_tables host_tables_dims{};
};

namespace {

struct Counters {
  unsigned long long next;
  unsigned long long events;
  unsigned long long n_geom;
  unsigned long long n_dep;
  double ensrc;
  int max_np;
  unsigned err;
};

template <typename R>
omc_status upload_tables(PrecisionState<R> &S, const omc_tables *t) {
  S.tables.clear();
  int nmed = t->nmed;
  size_t ng = static_cast<size_t>(nmed) * MXGE, ne = static_cast<size_t>(nmed) * MXEKE;
  size_t nms = static_cast<size_t>(MXL_MS + 1) * (MXQ_MS + 1) * (MXU_MS + 1);
  size_t nspin = static_cast<size_t>(nmed) * 2 * (MXE_SPIN1 + 1) * (MXQ_SPIN + 1) * (MXU_SPIN + 1);
  DevArrays<R> &A = S.tables;
  Tables<R> &T = S.T;
  T.nmed = nmed;
  T.ge0 = A.put(t->ge0, nmed);
  T.ge1 = A.put(t->ge1, nmed);
  T.eke0 = A.put(t->eke0, nmed);
  T.eke1 = A.put(t->eke1, nmed);
  T.xcc = A.put(t->xcc, nmed);
  T.blcc = A.put(t->blcc, nmed);
  T.te = A.put(t->te, nmed);
  T.thmoll = A.put(t->thmoll, nmed);
  T.ap = A.put(t->ap, nmed);
  T.esig_e = A.put(t->esig_e, nmed);
  T.psig_e = A.put(t->psig_e, nmed);
  T.delcm = A.put(t->delcm, nmed);
  T.zbrang = A.put(t->zbrang, nmed);
  T.bpar0 = A.put(t->bpar0, nmed);
  T.bpar1 = A.put(t->bpar1, nmed);
  T.monotone = A.put_int(t->sig_ismonotone, 2 * nmed);
  T.meke = A.put_int(t->meke, nmed);
  T.gmfp0 = A.put(t->gmfp0, ng);
  T.gmfp1 = A.put(t->gmfp1, ng);
  T.gbr10 = A.put(t->gbr10, ng);
  T.gbr11 = A.put(t->gbr11, ng);
  T.gbr20 = A.put(t->gbr20, ng);
  T.gbr21 = A.put(t->gbr21, ng);
  T.cohe0 = A.put(t->cohe0, ng);
  T.cohe1 = A.put(t->cohe1, ng);
  T.pmax0 = A.put(t->pmax0, ng);
  T.pmax1 = A.put(t->pmax1, ng);
  // Rayleigh sampling reads medium 0's form-factor tables (see rayleigh()).
  T.xgrid = A.put(t->xgrid, MXRAYFF);
  T.fcum = A.put(t->fcum, MXRAYFF);
  T.b_array = A.put(t->b_array, MXRAYFF);
  T.c_array = A.put(t->c_array, MXRAYFF);
  T.i_array = A.put_int(t->i_array, MXRAYFF);
  T.dl1 = A.put(t->dl1, 8 * nmed);
  T.dl2 = A.put(t->dl2, 8 * nmed);
  T.dl3 = A.put(t->dl3, 8 * nmed);
  T.dl4 = A.put(t->dl4, 8 * nmed);
  T.dl5 = A.put(t->dl5, 8 * nmed);
  T.dl6 = A.put(t->dl6, 8 * nmed);
  T.esig0 = A.put(t->esig0, ne);
  T.esig1 = A.put(t->esig1, ne);
  T.psig0 = A.put(t->psig0, ne);
  T.psig1 = A.put(t->psig1, ne);
  T.ededx0 = A.put(t->ededx0, ne);
  T.ededx1 = A.put(t->ededx1, ne);
  T.pdedx0 = A.put(t->pdedx0, ne);
  T.pdedx1 = A.put(t->pdedx1, ne);
  T.ebr10 = A.put(t->ebr10, ne);
  T.ebr11 = A.put(t->ebr11, ne);
  T.pbr10 = A.put(t->pbr10, ne);
  T.pbr11 = A.put(t->pbr11, ne);
  T.pbr20 = A.put(t->pbr20, ne);
  T.pbr21 = A.put(t->pbr21, ne);
  T.tmxs0 = A.put(t->tmxs0, ne);
  T.tmxs1 = A.put(t->tmxs1, ne);
  T.blcce0 = A.put(t->blcce0, ne);
  T.blcce1 = A.put(t->blcce1, ne);
  T.etae0 = A.put(t->etae_ms0, ne);
  T.etae1 = A.put(t->etae_ms1, ne);
  T.etap0 = A.put(t->etap_ms0, ne);
  T.etap1 = A.put(t->etap_ms1, ne);
  T.q1ce0 = A.put(t->q1ce_ms0, ne);
  T.q1ce1 = A.put(t->q1ce_ms1, ne);
  T.q1cp0 = A.put(t->q1cp_ms0, ne);
  T.q1cp1 = A.put(t->q1cp_ms1, ne);
  T.q2ce0 = A.put(t->q2ce_ms0, ne);
  T.q2ce1 = A.put(t->q2ce_ms1, ne);
  T.q2cp0 = A.put(t->q2cp_ms0, ne);
  T.q2cp1 = A.put(t->q2cp_ms1, ne);
  T.e_array = A.put(t->e_array, ne);
  T.range_ep = A.put(t->range_ep, 2 * ne);
  T.b2spin_min = static_cast<R>(t->b2spin_min);
  T.dbeta2i = static_cast<R>(t->dbeta2i);
  T.espml = static_cast<R>(t->espml);
  T.dleneri = static_cast<R>(t->dleneri);
  T.dqq1i = static_cast<R>(t->dqq1i);
  T.spin_rej = A.put(t->spin_rej, nspin);
  T.ums = A.put(t->ums, nms);
  T.fms = A.put(t->fms, nms);
  T.wms = A.put(t->wms, nms);
  T.ims = A.put_int(t->ims, nms);
  T.dllambi = static_cast<R>(t->dllambi);
  T.dqmsi = static_cast<R>(t->dqmsi);
  // Packed interpolation records (layout in device.cuh).
  auto v4 = [](double a, double b, double c, double d) {
    return V4<R>{static_cast<R>(a), static_cast<R>(b), static_cast<R>(c), static_cast<R>(d)};
  };
  std::vector<V4<R>> pm(ng), pb(ng);
  for (size_t i = 0; i < ng; i++) {
    pm[i] = v4(t->gmfp1[i], t->gmfp0[i], t->cohe1[i], t->cohe0[i]);
    pb[i] = v4(t->gbr11[i], t->gbr10[i], t->gbr21[i], t->gbr20[i]);
  }
  T.ph_mfp = A.put4(pm);
  T.ph_br = A.put4(pb);
  std::vector<V4<R>> sd(2 * ne), te(2 * ne), rg(2 * ne), qv(2 * ne), ib(ne), ib2(ne);
  for (int q = 0; q < 2; q++)
    for (size_t i = 0; i < ne; i++) {
      size_t o = q * ne + i;
      if (q == 0) {
        sd[o] = v4(t->esig1[i], t->esig0[i], t->ededx1[i], t->ededx0[i]);
        te[o] = v4(t->tmxs1[i], t->tmxs0[i], t->etae_ms1[i], t->etae_ms0[i]);
        qv[o] = v4(t->q1ce_ms1[i], t->q1ce_ms0[i], t->q2ce_ms1[i], t->q2ce_ms0[i]);
      } else {
        sd[o] = v4(t->psig1[i], t->psig0[i], t->pdedx1[i], t->pdedx0[i]);
        te[o] = v4(t->tmxs1[i], t->tmxs0[i], t->etap_ms1[i], t->etap_ms0[i]);
        qv[o] = v4(t->q1cp_ms1[i], t->q1cp_ms0[i], t->q2cp_ms1[i], t->q2cp_ms0[i]);
      }
      rg[o] = v4(t->blcce1[i], t->blcce0[i], t->range_ep[o], t->e_array[i]);
    }
  for (size_t i = 0; i < ne; i++) {
    ib[i] = v4(t->ebr11[i], t->ebr10[i], t->pbr11[i], t->pbr10[i]);
    ib2[i] = v4(t->pbr21[i], t->pbr20[i], 0.0, 0.0);
  }
  T.el_sd = A.put4(sd);
  T.el_te = A.put4(te);
  T.el_rg = A.put4(rg);
  T.el_q = A.put4(qv);
  T.el_ib = A.put4(ib);
  T.el_ib2 = A.put4(ib2);
  for (auto &b : A.bufs)
    if (!b.p) return fail(OMC_ERR_NOMEM, "table upload failed");
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(OMC_ERR_CUDA, "table upload: %s", cudaGetErrorString(e));
  S.tables_ok = true;
  return OMC_OK;
}

template <typename R>
omc_status upload_geometry(PrecisionState<R> &S, const omc_phantom *ph, const std::vector<int8_t> &med,
                           const std::vector<double> &rhof, const double *ecut_m, const double *pcut_m, int nmed) {
  S.geom.clear();
  DevArrays<R> &A = S.geom;
  Geometry<R> &G = S.G;
  G.nx = ph->nx;
  G.ny = ph->ny;
  G.nz = ph->nz;
  G.nxy = ph->nx * ph->ny;
  G.div_nx = make_divisor(static_cast<unsigned>(ph->nx));
  G.div_nxy = make_divisor(static_cast<unsigned>(G.nxy));
  G.xb = A.put(ph->xbounds, ph->nx + 1);
  G.yb = A.put(ph->ybounds, ph->ny + 1);
  G.zb = A.put(ph->zbounds, ph->nz + 1);
  G.ecut_m = A.put(ecut_m, nmed + 1);
  G.pcut_m = A.put(pcut_m, nmed + 1);
  std::vector<VoxelRec<R>> vox(med.size());
  for (size_t i = 0; i < med.size(); i++) {
    vox[i].rhof = static_cast<R>(rhof[i]);
    vox[i].med = med[i];
  }
  DevBuf vb;
  if (vb.ensure(vox.size() * sizeof(VoxelRec<R>)) != OMC_OK) return OMC_ERR_NOMEM;
  cudaMemcpy(vb.p, vox.data(), vox.size() * sizeof(VoxelRec<R>), cudaMemcpyHostToDevice);
  A.bufs.push_back(vb);
  G.vox = static_cast<const VoxelRec<R> *>(vb.p);
  for (auto &b : A.bufs)
    if (!b.p) return fail(OMC_ERR_NOMEM, "geometry upload failed");
  S.geom_ok = true;
  return OMC_OK;
}

template <typename R>
omc_status upload_source(PrecisionState<R> &S, const omc_source *s) {
  S.source.clear();
  Source<R> &D = S.S;
  D.spectrum = s->spectrum;
  D.charge = s->charge;
  D.energy = static_cast<R>(s->energy);
  D.deltak = static_cast<R>(s->deltak);
  D.cdfinv1 = S.source.put(s->cdfinv1, OMC_INVDIM);
  D.cdfinv2 = S.source.put(s->cdfinv2, OMC_INVDIM);
  D.ssd = static_cast<R>(s->ssd);
  D.xinl = static_cast<R>(s->xinl);
  D.yinl = static_cast<R>(s->yinl);
  D.xsize = static_cast<R>(s->xsize);
  D.ysize = static_cast<R>(s->ysize);
  D.ixinl = s->ixinl;
  D.iyinl = s->iyinl;
  if (!D.cdfinv1 || !D.cdfinv2) return fail(OMC_ERR_NOMEM, "source upload failed");
  S.source_ok = true;
  return OMC_OK;
}

// Beamlet jobs: the launch's slot map, tally and source.
template <typename R>
void apply_job(Params<R> &P, const PrecisionState<R> &S, const SlotJob *job, long long nreg) {
  P.tally_stride = nreg;
  if (!job) return;
  P.nslots = job->nslots;
  P.slot_first = job->first;
  P.nhist = job->nhist;
  if (job->jobs) {
    P.jobs = static_cast<const JobSlot<R> *>(job->jobs);
    P.endep = nullptr;
    return;
  }
  P.slot_beamlet = job->beamlet;
  P.endep = job->tally;
  if (!job->beamlets) return;
  P.S.beamlets = 1;
  P.S.bixel = S.bixel;
  P.S.beam_src = S.beam_src;
  P.S.ibeam = S.ibeam;
}

template <typename R>
omc_status upload_beamlets(PrecisionState<R> &S, const omc_beamlets *b) {
  S.beamlets.clear();
  std::vector<double> bix(static_cast<size_t>(b->nbeamlets) * 9), src(static_cast<size_t>(b->nbeams) * 3);
  for (int i = 0; i < b->nbeamlets; i++) {
    double *o = bix.data() + static_cast<size_t>(i) * 9;
    o[0] = b->xcorner[i];
    o[1] = b->ycorner[i];
    o[2] = b->zcorner[i];
    o[3] = b->xside1[i];
    o[4] = b->yside1[i];
    o[5] = b->zside1[i];
    o[6] = b->xside2[i];
    o[7] = b->yside2[i];
    o[8] = b->zside2[i];
  }
  for (int i = 0; i < b->nbeams; i++) {
    src[3 * i] = b->xsource[i];
    src[3 * i + 1] = b->ysource[i];
    src[3 * i + 2] = b->zsource[i];
  }
  S.bixel = S.beamlets.put(bix.data(), bix.size());
  S.beam_src = S.beamlets.put(src.data(), src.size());
  S.ibeam = S.beamlets.put_int(b->ibeam, b->nbeamlets);
  if (!S.bixel || !S.beam_src || !S.ibeam) return fail(OMC_ERR_NOMEM, "beamlet upload failed");
  return OMC_OK;
}

template <typename R>
omc_status run_batches(omc_engine *e, PrecisionState<R> &S, const omc_run_config *cfg, int nlanes, int depth,
                       omc_run_stats *stats, const SlotJob *job = nullptr) {
  size_t plane = static_cast<size_t>(depth) * nlanes;
  if (S.stk.ensure(plane * 8 * sizeof(R)) != OMC_OK) return OMC_ERR_NOMEM;
  if (S.key.ensure(plane * sizeof(int)) != OMC_OK) return OMC_ERR_NOMEM;
  Counters *dc = static_cast<Counters *>(e->counters.p);
  Params<R> P{};
  P.T = S.T;
  P.G = S.G;
  P.S = S.S;
  P.nsplit = cfg->nsplit < 1 ? 1 : cfg->nsplit;
  P.nlanes = nlanes;
  P.depth = depth;
  P.nhist = cfg->nperbatch;
  P.next = &dc->next;
  P.rng_u = static_cast<int *>(e->rng_u.p);
  P.rng_ijc = static_cast<int *>(e->rng_ijc.p);
  P.stk = static_cast<R *>(S.stk.p);
  P.stk_key = static_cast<int *>(S.key.p);
  P.endep = static_cast<double *>(e->endep.p);
  P.ensrc = &dc->ensrc;
  P.events = &dc->events;
  P.n_geom = &dc->n_geom;
  P.n_dep = &dc->n_dep;
  P.max_np = &dc->max_np;
  P.err = &dc->err;
  apply_job(P, S, job, e->nreg);
  const int nlaunch = job ? 1 : cfg->nbatch;
  size_t smem = kRngSmem;
  cudaFuncSetAttribute(transport_kernel<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  int blocks = (nlanes + kBlock - 1) / kBlock;
  cudaEvent_t t0, t1;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  cudaEventRecord(t0, e->stream);
  for (int b = 0; b < nlaunch; b++) {
    cudaMemsetAsync(&dc->next, 0, sizeof(unsigned long long), e->stream);
    transport_kernel<R><<<blocks, kBlock, smem, e->stream>>>(P);
    if (job) continue;
    accumulate_kernel<<<std::max(1, std::min(4 * e->nsm, (e->nreg + 255) / 256)), 256, 0, e->stream>>>(
        static_cast<double *>(e->endep.p), static_cast<double *>(e->acc.p), static_cast<double *>(e->acc2.p),
        e->nreg);
  }
  cudaEventRecord(t1, e->stream);
  cudaError_t err = cudaStreamSynchronize(e->stream);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, t0, t1);
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  if (err != cudaSuccess) return fail(OMC_ERR_CUDA, "transport: %s", cudaGetErrorString(err));
  err = cudaGetLastError();
  if (err != cudaSuccess) return fail(OMC_ERR_CUDA, "transport launch: %s", cudaGetErrorString(err));
  Counters hc{};
  cudaMemcpy(&hc, dc, sizeof hc, cudaMemcpyDeviceToHost);
  if (stats) {
    stats->ensrc = hc.ensrc;
    stats->transport_ms = ms;
    stats->histories = job ? job->nhist : cfg->nperbatch * cfg->nbatch;
    stats->steps = static_cast<long long>(hc.events);
    stats->voxel_steps = static_cast<long long>(hc.n_geom);
    stats->deposits = static_cast<long long>(hc.n_dep);
    stats->kernel_ms = ms;
    stats->max_stack = hc.max_np + 1;
    stats->error_flags = static_cast<int>(hc.err & ~ERR_TABLE);
    stats->warnings = static_cast<int>(hc.err & ERR_TABLE);
  }
  if (hc.err & ERR_STACK) return fail(OMC_ERR_STACK, "particle stack overflow (depth %d); histories were dropped", depth);
  if (hc.err & (ERR_LOOP | ERR_EVENTS)) return fail(OMC_ERR_LIMIT, "a device loop hit its iteration limit");
  return OMC_OK;
}

struct WfCounters {
  unsigned ctr[15];
  unsigned long long work[3];
  unsigned long long injected[2];
  unsigned bar_arrive, bar_gen;
  int iters;
  unsigned hwm;
};

template <typename R, bool MULTI = false, bool HBH = false>
int wavefront_blocks(omc_engine *e) {
  size_t smem = kRngSmem;
  cudaFuncSetAttribute(wavefront_kernel<R, MULTI, HBH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       static_cast<int>(smem));
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, wavefront_kernel<R, MULTI, HBH>, kBlock, smem);
  return (per_sm < 1 ? 1 : per_sm) * e->nsm;
}

// Counters of the history-by-history pool (one device buffer).
struct HbhCounters {
  unsigned long long ctr[2];   // {pushed, popped}: HbhPool::ctr
  unsigned long long snap[4];  // Wavefront::hbh_free
  unsigned long long histories, split;
};

// A full pool: every block id in the ring.
__global__ void hbh_init_kernel(int *ring, int nblocks, HbhCounters *c) {
  // ring positions are taken modulo a power of two >= nblocks; the first
  // nblocks hold every block id
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < nblocks;
       i += static_cast<long long>(gridDim.x) * blockDim.x)
    ring[i] = static_cast<int>(i);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    c->ctr[0] = static_cast<unsigned long long>(nblocks);
    c->ctr[1] = 0;
    c->snap[0] = static_cast<unsigned long long>(nblocks);  // iteration 0 reads slot 0
    c->snap[1] = 0;
  }
}

template <typename R>
omc_status run_wavefront(omc_engine *e, PrecisionState<R> &S, const omc_run_config *cfg, int nlanes,
                         omc_run_stats *stats, const SlotJob *job = nullptr) {
  const int nsplit = cfg->nsplit < 1 ? 1 : cfg->nsplit;
  const int blocks = nlanes / kBlock;
  // Particles in flight: more keeps every iteration full and amortises its
  // grid barrier (measured on the 6 MV slab: FP32 7.75e7 / 7.90e7 / 7.97e7
  // histories/s at 32 / 64 / 128 per thread; FP64 with 2 blocks per SM
  // 6.96e6 / 7.04e6 / 7.01e6 at 64 / 96 / 128).
  unsigned long long target = cfg->inflight > 0 ? static_cast<unsigned long long>(cfg->inflight)
                                                 : static_cast<unsigned long long>(nlanes) * kInflightPerThread<R>;
  // Worst case growth in one iteration: every photon of a cycle leaves up
  // to two particles per split, every electron step up to two.
  unsigned long long cap = target * (4ull + 2ull * nsplit) + 4ull * nlanes;
  if (cap > 0x7fffffffull) cap = 0x7fffffffull;
  const bool hbh = cfg->history_stats != 0 && !(job && job->jobs);
  const size_t tag_bytes = (job || hbh) ? static_cast<size_t>(cap) * sizeof(int) : 0;
  size_t per_queue = static_cast<size_t>(cap) * (8 * sizeof(R) + sizeof(int)) + tag_bytes;
  // photons, electrons (those near a boundary from the top), electron and
  // photon interactions; two generations each
  const int nqueues = 8;
  // and the photon flights' mean free paths left, two generations
  const size_t mfp_bytes = (static_cast<size_t>(cap) * sizeof(R) + 255) & ~static_cast<size_t>(255);
  if (S.queue.ensure(nqueues * per_queue + 2 * mfp_bytes) != OMC_OK) return OMC_ERR_NOMEM;
  if (e->wf_counters.ensure(sizeof(WfCounters)) != OMC_OK) return OMC_ERR_NOMEM;
  char *qb = static_cast<char *>(S.queue.p);
  Wavefront<R> W{};
  for (int q = 0; q < nqueues; q++) {
    R *f = reinterpret_cast<R *>(qb + q * per_queue);
    int *k = reinterpret_cast<int *>(qb + q * per_queue + static_cast<size_t>(cap) * 8 * sizeof(R));
    int *tag = (job || hbh) ? k + cap : nullptr;
    if (q < 2) {
      W.ph_f[q] = f;
      W.ph_k[q] = k;
      W.ph_s[q] = tag;
    } else if (q < 4) {
      W.el_f[q - 2] = f;
      W.el_k[q - 2] = k;
      W.el_s[q - 2] = tag;
    } else if (q < 6) {
      W.ei_f[q - 4] = f;
      W.ei_k[q - 4] = k;
      W.ei_s[q - 4] = tag;
    } else {
      W.pi_f[q - 6] = f;
      W.pi_k[q - 6] = k;
      W.pi_s[q - 6] = tag;
    }
  }
  W.ph_t[0] = reinterpret_cast<R *>(qb + nqueues * per_queue);
  W.ph_t[1] = reinterpret_cast<R *>(qb + nqueues * per_queue + mfp_bytes);
  W.flight_cap = kFlightCap<R>;
  WfCounters *wc = static_cast<WfCounters *>(e->wf_counters.p);
  W.cap = static_cast<unsigned>(cap);
  W.ctr = wc->ctr;
  W.work = wc->work;
  W.injected = wc->injected;
  W.bar_arrive = &wc->bar_arrive;
  W.bar_gen = &wc->bar_gen;
  W.target = static_cast<unsigned>(target > 0xffffffffull ? 0xffffffffull : target);
  W.max_iters = 1 << 21;
  W.iters = &wc->iters;
  W.hwm = &wc->hwm;
  W.trace = static_cast<unsigned long long *>(e->trace.p);
  W.trace_cap = e->trace_cap;
  W.chunk_events = cfg->chunk_events > 0 ? cfg->chunk_events : kDefaultChunkEvents;
  W.drain_below = cfg->drain_per_warp < 0
                      ? 0ull
                      : static_cast<unsigned long long>(cfg->drain_per_warp > 0 ? cfg->drain_per_warp
                                                                                 : kDrainPerWarp) *
                            static_cast<unsigned long long>(nlanes / 32);
  Counters *dc = static_cast<Counters *>(e->counters.p);
  Params<R> P{};
  P.T = S.T;
  P.G = S.G;
  P.S = S.S;
  P.nsplit = nsplit;
  P.nlanes = nlanes;
  P.nhist = cfg->nperbatch;
  P.next = &dc->next;
  P.rng_u = static_cast<int *>(e->rng_u.p);
  P.rng_ijc = static_cast<int *>(e->rng_ijc.p);
  P.endep = static_cast<double *>(e->endep.p);
  P.ensrc = &dc->ensrc;
  P.events = &dc->events;
  P.n_geom = &dc->n_geom;
  P.n_dep = &dc->n_dep;
  P.max_np = &dc->max_np;
  P.err = &dc->err;
  apply_job(P, S, job, e->nreg);
  // History-by-history pool: a head block per history in flight plus
  // continuation blocks; an iteration keeps 4 blocks per thread back for
  // continuations.
  HbhCounters *hc_dev = nullptr;
  int hbh_nblocks = 0;
  if (hbh) {
    const unsigned long long nb = target * OMC_HBH_POOL_X2 / 2 + 8ull * nlanes;
    if (nb > 0x7fffffffull) return fail(OMC_ERR_ARG, "history tracking: %llu blocks exceed the pool index", nb);
    hbh_nblocks = static_cast<int>(nb);
    if (e->hbh_blocks.ensure(nb * sizeof(HbhBlock<R>)) != OMC_OK) return OMC_ERR_NOMEM;
    unsigned long long ring = 1;
    while (ring < nb) ring <<= 1;
    if (e->hbh_ring.ensure(ring * sizeof(int)) != OMC_OK) return OMC_ERR_NOMEM;
    if (e->hbh_ctr.ensure(sizeof(HbhCounters)) != OMC_OK) return OMC_ERR_NOMEM;
    hc_dev = static_cast<HbhCounters *>(e->hbh_ctr.p);
    CUDA_TRY(cudaMemsetAsync(hc_dev, 0, sizeof(HbhCounters), e->stream));
    P.hbh.blocks = static_cast<HbhBlock<R> *>(e->hbh_blocks.p);
    P.hbh.nblocks = hbh_nblocks;
    P.hbh.ring_mask = static_cast<unsigned>(ring - 1);
    P.hbh.ring = static_cast<int *>(e->hbh_ring.p);
    P.hbh.ctr = hc_dev->ctr;
    P.hbh.sum = static_cast<double *>(e->hbh_sum.p);
    P.hbh.sum2 = static_cast<double *>(e->hbh_sum2.p);
    P.hbh.histories = &hc_dev->histories;
    P.hbh.split = &hc_dev->split;
    W.hbh_free = hc_dev->snap;
    W.hbh_reserve = 4ull * nlanes;
  }
  const int nlaunch = job ? 1 : cfg->nbatch;
  size_t smem = kRngSmem;
  cudaEvent_t t0, t1;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  cudaEventRecord(t0, e->stream);
  int iters_total = 0;
  cudaError_t err = cudaSuccess;
  for (int b = 0; b < nlaunch && err == cudaSuccess; b++) {
    cudaMemsetAsync(wc, 0, sizeof(WfCounters), e->stream);
    if (hbh) {
      hbh_init_kernel<<<std::max(1, std::min(4 * e->nsm, (hbh_nblocks + 255) / 256)), 256, 0, e->stream>>>(
          P.hbh.ring, hbh_nblocks, hc_dev);
    }
    void *args[] = {&P, &W};
    void *fn = (job && job->jobs) ? reinterpret_cast<void *>(wavefront_kernel<R, true>)
               : hbh              ? reinterpret_cast<void *>(wavefront_kernel<R, false, true>)
                                  : reinterpret_cast<void *>(wavefront_kernel<R, false>);
    err = cudaLaunchCooperativeKernel(fn, dim3(blocks), dim3(kBlock), args, smem, e->stream);
    if (job) continue;
    accumulate_kernel<<<std::max(1, std::min(4 * e->nsm, (e->nreg + 255) / 256)), 256, 0, e->stream>>>(
        static_cast<double *>(e->endep.p), static_cast<double *>(e->acc.p), static_cast<double *>(e->acc2.p),
        e->nreg);
  }
  cudaEventRecord(t1, e->stream);
  cudaError_t serr = cudaStreamSynchronize(e->stream);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, t0, t1);
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  if (err != cudaSuccess) return fail(OMC_ERR_CUDA, "wavefront launch: %s", cudaGetErrorString(err));
  if (serr != cudaSuccess) return fail(OMC_ERR_CUDA, "wavefront transport: %s", cudaGetErrorString(serr));
  Counters hc{};
  WfCounters hw{};
  cudaMemcpy(&hc, dc, sizeof hc, cudaMemcpyDeviceToHost);
  cudaMemcpy(&hw, wc, sizeof hw, cudaMemcpyDeviceToHost);
  if (hbh) {
    HbhCounters hh{};
    cudaMemcpy(&hh, hc_dev, sizeof hh, cudaMemcpyDeviceToHost);
    e->hbh_histories += static_cast<long long>(hh.histories);
    e->hbh_split += static_cast<long long>(hh.split);
  }
  iters_total = hw.iters;
  e->trace_iters = hw.iters;
  if (stats) {
    stats->ensrc = hc.ensrc;
    stats->transport_ms = ms;
    stats->kernel_ms = ms;
    stats->histories = job ? job->nhist : cfg->nperbatch * cfg->nbatch;
    stats->steps = static_cast<long long>(hc.events);
    stats->voxel_steps = static_cast<long long>(hc.n_geom);
    stats->deposits = static_cast<long long>(hc.n_dep);
    stats->max_stack = static_cast<int>(hw.hwm + 1);
    stats->error_flags = static_cast<int>(hc.err & ~ERR_TABLE);
    stats->warnings = static_cast<int>(hc.err & ERR_TABLE);
  }
  (void)iters_total;
  if (hc.err & ERR_QUEUE) return fail(OMC_ERR_STACK, "wavefront queue overflow (capacity %llu); particles were dropped", cap);
  if (hc.err & (ERR_LOOP | ERR_EVENTS | ERR_BARRIER)) return fail(OMC_ERR_LIMIT, "a device loop hit its iteration limit");
  return OMC_OK;
}

omc_status ensure_device(omc_engine *e) {
  CUDA_TRY(cudaSetDevice(e->device));
  return OMC_OK;
}

template <typename R>
int default_lanes(omc_engine *e) {
  int per_sm = 0;
  size_t smem = kRngSmem;
  cudaFuncSetAttribute(transport_kernel<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, transport_kernel<R>, kBlock, smem);
  if (per_sm < 1) per_sm = 1;
  return e->nsm * per_sm * kBlock;
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" omc_status omc_engine_create(int device, omc_engine **out) {
  if (!out) return fail(OMC_ERR_ARG, "null argument");
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return fail(OMC_ERR_CUDA, "no CUDA device available");
  if (device < 0 || device >= n) return fail(OMC_ERR_ARG, "device %d outside 0..%d", device, n - 1);
  auto *e = new omc_engine();
  e->device = device;
  if (cudaSetDevice(device) != cudaSuccess) {
    delete e;
    return fail(OMC_ERR_CUDA, "cudaSetDevice(%d) failed", device);
  }
  cudaDeviceGetAttribute(&e->nsm, cudaDevAttrMultiProcessorCount, device);
  cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking);
  if (e->counters.ensure(sizeof(Counters)) != OMC_OK) {
    delete e;
    return OMC_ERR_NOMEM;
  }
  *out = e;
  return OMC_OK;
}

extern "C" void omc_engine_destroy(omc_engine *e) {
  if (!e) return;
  cudaSetDevice(e->device);
  cudaStreamSynchronize(e->stream);
  e->f64.tables.clear();
  e->f64.geom.clear();
  e->f64.source.clear();
  e->f64.stk.release();
  e->f64.key.release();
  e->f64.queue.release();
  e->f32.queue.release();
  e->wf_counters.release();
  e->f32.tables.clear();
  e->f32.geom.clear();
  e->f32.source.clear();
  e->f32.stk.release();
  e->f32.key.release();
  e->rng_u.release();
  e->rng_ijc.release();
  e->endep.release();
  e->acc.release();
  e->acc2.release();
  e->counters.release();
  e->density.release();
  e->f64.beamlets.clear();
  e->f32.beamlets.clear();
  for (DevBuf *b : {&e->dij_tally, &e->dij_first, &e->dij_beamlet, &e->dij_nhist, &e->dij_max, &e->dij_cnt,
                    &e->dij_off, &e->dij_rows, &e->dij_vals, &e->multi_slots, &e->multi_first, &e->trace,
                    &e->batch_tally, &e->batch_first, &e->dij_factor, &e->weights, &e->batch_dot,
                    &e->hbh_blocks, &e->hbh_ring, &e->hbh_ctr, &e->hbh_sum, &e->hbh_sum2})
    b->release();
  cudaStreamDestroy(e->stream);
  delete e;
}

extern "C" omc_status omc_engine_set_tables(omc_engine *e, const omc_tables *t) {
  if (!e || !t) return fail(OMC_ERR_ARG, "null argument");
  omc_status s;
  if ((s = ensure_device(e)) != OMC_OK) return s;
  if ((s = upload_tables(e->f64, t)) != OMC_OK) return s;
  if ((s = upload_tables(e->f32, t)) != OMC_OK) return s;
  e->host_tables_dims.nmed = t->nmed;
  return OMC_OK;
}

namespace {

// Per-region medium, density ratio and per-medium cuts in the device
// layout.  ecut/pcut are per region in the reference; initRegions makes
// them a function of the medium, which is what the device stores.
struct RegionData {
  std::vector<int8_t> med;
  std::vector<double> rhof, ecut_m, pcut_m;
};

omc_status region_data(int nmed, const omc_phantom *ph, const omc_regions *r, RegionData &d) {
  int nreg = ph->nx * ph->ny * ph->nz + 1;
  if (r->nreg != nreg) return fail(OMC_ERR_ARG, "regions (%d) do not match the phantom (%d)", r->nreg, nreg);
  d.med.assign(nreg, 0);
  d.rhof.assign(r->rhof, r->rhof + nreg);
  d.ecut_m.assign(nmed + 1, 0.0);
  d.pcut_m.assign(nmed + 1, 0.0);
  std::vector<int> seen(nmed + 1, 0);
  for (int i = 0; i < nreg; i++) {
    int m = r->med[i];
    if (m < -1 || m >= nmed) return fail(OMC_ERR_ARG, "region %d: medium %d outside -1..%d", i, m, nmed - 1);
    d.med[i] = static_cast<int8_t>(m);
    if (i == 0) continue;
    if (!seen[m + 1]) {
      d.ecut_m[m + 1] = r->ecut[i];
      d.pcut_m[m + 1] = r->pcut[i];
      seen[m + 1] = 1;
    } else if (d.ecut_m[m + 1] != r->ecut[i] || d.pcut_m[m + 1] != r->pcut[i]) {
      return fail(OMC_ERR_ARG, "region %d: ecut/pcut differ within medium %d", i, m);
    }
  }
  d.ecut_m[0] = 0.0;
  d.pcut_m[0] = 0.0;
  return OMC_OK;
}

}  // namespace

extern "C" omc_status omc_engine_set_geometry(omc_engine *e, const omc_phantom *ph, const omc_regions *r) {
  if (!e || !ph || !r) return fail(OMC_ERR_ARG, "null argument");
  if (!e->f64.tables_ok) return fail(OMC_ERR_STATE, "omc_engine_set_tables must come first");
  int nmed = e->host_tables_dims.nmed;
  int nreg = ph->nx * ph->ny * ph->nz + 1;
  RegionData rd;
  omc_status s;
  if ((s = region_data(nmed, ph, r, rd)) != OMC_OK) return s;
  const std::vector<int8_t> &med = rd.med;
  const std::vector<double> &rhof = rd.rhof, &ecut_m = rd.ecut_m, &pcut_m = rd.pcut_m;
  if ((s = ensure_device(e)) != OMC_OK) return s;
  if ((s = upload_geometry(e->f64, ph, med, rhof, ecut_m.data(), pcut_m.data(), nmed)) != OMC_OK) return s;
  if ((s = upload_geometry(e->f32, ph, med, rhof, ecut_m.data(), pcut_m.data(), nmed)) != OMC_OK) return s;
  e->nreg = nreg;
  if ((s = e->density.ensure(static_cast<size_t>(nreg - 1) * sizeof(double))) != OMC_OK) return s;
  CUDA_TRY(cudaMemcpy(e->density.p, ph->density, static_cast<size_t>(nreg - 1) * sizeof(double),
                      cudaMemcpyHostToDevice));
  if ((s = e->endep.ensure(nreg * sizeof(double))) != OMC_OK) return s;
  if ((s = e->acc.ensure(nreg * sizeof(double))) != OMC_OK) return s;
  if ((s = e->acc2.ensure(nreg * sizeof(double))) != OMC_OK) return s;
  return OMC_OK;
}

extern "C" omc_status omc_engine_set_source(omc_engine *e, const omc_source *s) {
  if (!e || !s) return fail(OMC_ERR_ARG, "null argument");
  omc_status st;
  if ((st = ensure_device(e)) != OMC_OK) return st;
  if ((st = upload_source(e->f64, s)) != OMC_OK) return st;
  if ((st = upload_source(e->f32, s)) != OMC_OK) return st;
  return OMC_OK;
}

// accum = sum over batches, accum2 = sum of squares (accumEndep over
// batch tallies kept side by side: one launch's batches, or a job's).
__global__ void batch_accumulate_kernel(const double *tally, int nbatch, long long nreg, double *acc, double *acc2) {
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < nreg;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    double a = 0.0, a2 = 0.0;
    for (int b = 0; b < nbatch; b++) {
      double v = tally[static_cast<size_t>(b) * nreg + i];
      a += v;
      a2 += v * v;
    }
    acc[i] = a;
    acc2[i] = a2;
  }
}

static omc_status run_batches_one_launch(omc_engine *e, const omc_run_config *cfg, int nlanes, bool fp64,
                                         omc_run_stats *stats) {
  const int nb = cfg->nbatch;
  omc_status s;
  if ((s = e->batch_tally.ensure(static_cast<size_t>(nb) * e->nreg * sizeof(double))) != OMC_OK) return s;
  if ((s = e->batch_first.ensure((nb + 1) * sizeof(long long))) != OMC_OK) return s;
  std::vector<long long> first(nb + 1);
  for (int b = 0; b <= nb; b++) first[b] = static_cast<long long>(b) * cfg->nperbatch;
  CUDA_TRY(cudaMemcpyAsync(e->batch_first.p, first.data(), (nb + 1) * sizeof(long long), cudaMemcpyHostToDevice,
                           e->stream));
  CUDA_TRY(cudaMemsetAsync(e->batch_tally.p, 0, static_cast<size_t>(nb) * e->nreg * sizeof(double), e->stream));
  SlotJob job{nb, static_cast<const long long *>(e->batch_first.p), nullptr, static_cast<double *>(e->batch_tally.p),
              first[nb], nullptr, false};
  omc_run_stats gs{};
  s = fp64 ? run_wavefront(e, e->f64, cfg, nlanes, &gs, &job) : run_wavefront(e, e->f32, cfg, nlanes, &gs, &job);
  if (s != OMC_OK && s != OMC_ERR_STACK && s != OMC_ERR_LIMIT) return s;
  cudaEvent_t t0, t1;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  cudaEventRecord(t0, e->stream);
  batch_accumulate_kernel<<<std::max(1, static_cast<int>(std::min<long long>(4 * e->nsm, (e->nreg + 255) / 256))), 256,
                            0, e->stream>>>(static_cast<const double *>(e->batch_tally.p), nb, e->nreg,
                                            static_cast<double *>(e->acc.p), static_cast<double *>(e->acc2.p));
  cudaEventRecord(t1, e->stream);
  CUDA_TRY(cudaStreamSynchronize(e->stream));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, t0, t1);
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  gs.kernel_ms += ms;
  gs.transport_ms += ms;
  if (stats) *stats = gs;
  e->batch_tallies = nb;
  return s;
}

// Shared start of every run: validation, schedule and lane count, RANMAR
// streams (seeded unless continued).
struct RunPlan {
  bool fp64, wavefront;
  int nlanes, depth;
};

static omc_status prepare_run(omc_engine *e, const omc_run_config *cfg, RunPlan &rp) {
  if (!e || !cfg) return fail(OMC_ERR_ARG, "null argument");
  if (!e->f64.tables_ok || !e->f64.geom_ok || !e->f64.source_ok)
    return fail(OMC_ERR_STATE, "tables, geometry and source must be set before a run");
  if (cfg->nbatch < 1 || cfg->nperbatch < 0) return fail(OMC_ERR_ARG, "nbatch must be >= 1 and nperbatch >= 0");
  if (cfg->precision != OMC_FP64 && cfg->precision != OMC_FP32) return fail(OMC_ERR_ARG, "unknown precision");
  if (cfg->schedule < 0 || cfg->schedule > OMC_SCHEDULE_WAVEFRONT) return fail(OMC_ERR_ARG, "unknown schedule");
  omc_status s;
  if ((s = ensure_device(e)) != OMC_OK) return s;
  rp.fp64 = cfg->precision == OMC_FP64;
  rp.wavefront = !cfg->serial && cfg->schedule != OMC_SCHEDULE_LANES;
  if (cfg->history_stats && !rp.wavefront)
    return fail(OMC_ERR_ARG, "history-by-history scoring needs the wavefront schedule");
  if (rp.wavefront && cfg->history_stats)
    rp.nlanes = (rp.fp64 ? wavefront_blocks<double, false, true>(e) : wavefront_blocks<float, false, true>(e)) * kBlock;
  else if (rp.wavefront)
    rp.nlanes = (rp.fp64 ? wavefront_blocks<double>(e) : wavefront_blocks<float>(e)) * kBlock;
  else if (cfg->serial) rp.nlanes = 1;
  else rp.nlanes = cfg->nlanes > 0 ? cfg->nlanes : (rp.fp64 ? default_lanes<double>(e) : default_lanes<float>(e));
  rp.depth = cfg->stack_depth > 0 ? cfg->stack_depth : kDefaultDepth + 4 * std::max(1, cfg->nsplit);
  const int nlanes = rp.nlanes;
  // RANMAR streams, one per lane, seeded for this run.
  size_t rng_bytes = static_cast<size_t>(RNG_WORDS) * nlanes * sizeof(int);
  if (e->rng_u.n < rng_bytes) e->seeded_lanes = 0;  // reallocated: streams must be seeded
  if ((s = e->rng_u.ensure(rng_bytes)) != OMC_OK) return s;
  if ((s = e->rng_ijc.ensure(static_cast<size_t>(3) * nlanes * sizeof(int))) != OMC_OK) return s;
  if (!(cfg->continue_streams && e->seeded_lanes == nlanes)) {
    seed_kernel<<<(nlanes + 255) / 256, 256, 0, e->stream>>>(cfg->ixx, cfg->jxx, nlanes,
                                                            static_cast<int *>(e->rng_u.p),
                                                            static_cast<int *>(e->rng_ijc.p));
    e->seeded_lanes = nlanes;
  }
  return OMC_OK;
}

static omc_status engine_run(omc_engine *e, const omc_run_config *cfg, omc_run_stats *stats) {
  RunPlan rp;
  omc_status s = prepare_run(e, cfg, rp);
  if (s != OMC_OK) return s;
  const bool fp64 = rp.fp64, wavefront = rp.wavefront;
  const int nlanes = rp.nlanes, depth = rp.depth;
  e->batch_tallies = 0;
  e->hbh_valid = false;
  e->hbh_histories = e->hbh_split = 0;
  if (cfg->history_stats) {
    if ((s = e->hbh_sum.ensure(e->nreg * sizeof(double))) != OMC_OK) return s;
    if ((s = e->hbh_sum2.ensure(e->nreg * sizeof(double))) != OMC_OK) return s;
    CUDA_TRY(cudaMemsetAsync(e->hbh_sum.p, 0, e->nreg * sizeof(double), e->stream));
    CUDA_TRY(cudaMemsetAsync(e->hbh_sum2.p, 0, e->nreg * sizeof(double), e->stream));
  }
  cudaMemsetAsync(e->endep.p, 0, e->nreg * sizeof(double), e->stream);
  cudaMemsetAsync(e->acc.p, 0, e->nreg * sizeof(double), e->stream);
  cudaMemsetAsync(e->acc2.p, 0, e->nreg * sizeof(double), e->stream);
  cudaMemsetAsync(e->counters.p, 0, sizeof(Counters), e->stream);
  if (wavefront && cfg->nbatch > 1 && cfg->nbatch <= 65535) {
    // All batches in one launch: batch b is tally slot b, histories are
    // injected without a pause between batches, and the particles of one
    // batch drain while the next batch is already in flight.
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    const size_t tally_bytes = static_cast<size_t>(cfg->nbatch) * e->nreg * sizeof(double);
    if (tally_bytes <= fr * 3 / 10) return run_batches_one_launch(e, cfg, nlanes, fp64, stats);
  }
  if (wavefront) return fp64 ? run_wavefront(e, e->f64, cfg, nlanes, stats) : run_wavefront(e, e->f32, cfg, nlanes, stats);
  return fp64 ? run_batches(e, e->f64, cfg, nlanes, depth, stats) : run_batches(e, e->f32, cfg, nlanes, depth, stats);
}

extern "C" omc_status omc_engine_history_sums(omc_engine *e, double *sum, double *sum2, long long *histories,
                                              long long *split) {
  if (!e) return fail(OMC_ERR_ARG, "null argument");
  if (!e->hbh_valid) return fail(OMC_ERR_STATE, "the last run did not score history by history (history_stats)");
  omc_status s;
  if ((s = ensure_device(e)) != OMC_OK) return s;
  if (sum) CUDA_TRY(cudaMemcpy(sum, e->hbh_sum.p, e->nreg * sizeof(double), cudaMemcpyDeviceToHost));
  if (sum2) CUDA_TRY(cudaMemcpy(sum2, e->hbh_sum2.p, e->nreg * sizeof(double), cudaMemcpyDeviceToHost));
  if (histories) *histories = e->hbh_histories;
  if (split) *split = e->hbh_split;
  return OMC_OK;
}

extern "C" omc_status omc_engine_run(omc_engine *e, const omc_run_config *cfg, double *accum_endep,
                                     double *accum_endep2, omc_run_stats *stats) {
  omc_status s = engine_run(e, cfg, stats);
  if (cfg && cfg->history_stats && (s == OMC_OK || s == OMC_ERR_STACK || s == OMC_ERR_LIMIT)) e->hbh_valid = true;
  if (s != OMC_OK && s != OMC_ERR_STACK && s != OMC_ERR_LIMIT) return s;
  if (accum_endep) cudaMemcpy(accum_endep, e->acc.p, e->nreg * sizeof(double), cudaMemcpyDeviceToHost);
  if (accum_endep2) cudaMemcpy(accum_endep2, e->acc2.p, e->nreg * sizeof(double), cudaMemcpyDeviceToHost);
  return s;
}

extern "C" omc_status omc_engine_tune(omc_engine *e, const omc_run_config *cfg, long long sample_histories,
                                      omc_run_config *best, double *rates) {
  if (!e || !cfg || !best) return fail(OMC_ERR_ARG, "null argument");
  if (sample_histories < 2) return fail(OMC_ERR_ARG, "sample_histories must be >= 2");
  RunPlan rp;
  omc_run_config probe = *cfg;
  probe.schedule = OMC_SCHEDULE_WAVEFRONT;
  probe.serial = 0;
  probe.nbatch = 2;
  probe.nperbatch = sample_histories / 2;
  omc_status s = prepare_run(e, &probe, rp);  // seeds the streams once
  if (s != OMC_OK) return s;
  probe.continue_streams = 1;
  static const int per_thread[4] = {32, 64, 128, 192};
  double best_rate = -1.0;
  *best = *cfg;
  for (int k = 0; k < 8; k++) {
    probe.inflight = static_cast<long long>(rp.nlanes) * per_thread[k / 2];
    probe.chunk_events = 1 + k % 2;
    omc_run_stats st{};
    s = engine_run(e, &probe, &st);
    if (s != OMC_OK) return s;
    double rate = st.kernel_ms > 0 ? static_cast<double>(probe.nperbatch * probe.nbatch) / (st.kernel_ms * 1e-3) : 0;
    if (rates) rates[k] = rate;
    if (rate > best_rate) {
      best_rate = rate;
      best->inflight = probe.inflight;
      best->chunk_events = probe.chunk_events;
      best->schedule = OMC_SCHEDULE_WAVEFRONT;
    }
  }
  return OMC_OK;
}

extern "C" omc_status omc_engine_run_resident(omc_engine *e, const omc_run_config *cfg, const double **d_acc,
                                              const double **d_acc2, omc_run_stats *stats) {
  omc_status s = engine_run(e, cfg, stats);
  if (cfg && cfg->history_stats && (s == OMC_OK || s == OMC_ERR_STACK || s == OMC_ERR_LIMIT)) e->hbh_valid = true;
  if (d_acc) *d_acc = static_cast<const double *>(e->acc.p);
  if (d_acc2) *d_acc2 = static_cast<const double *>(e->acc2.p);
  return s;
}

// out[b] += sum over regions r of w[r] * tally[b][r].  Grid: x over regions,
// y over batches.
__global__ void batch_dot_kernel(const double *__restrict__ tally, long long nreg, const double *__restrict__ w,
                                 double *out) {
  __shared__ double part[256 / 32];
  const double *t = tally + static_cast<size_t>(blockIdx.y) * nreg;
  double acc = 0.0;
  for (long long r = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; r < nreg;
       r += static_cast<long long>(gridDim.x) * blockDim.x)
    acc += w[r] * t[r];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double sum = 0.0;
    for (int k = 0; k < static_cast<int>(blockDim.x) / 32; k++) sum += part[k];
    atomicAdd(out + blockIdx.y, sum);
  }
}

extern "C" omc_status omc_engine_batch_sums(omc_engine *e, const double *weights, double *out, int *nbatch) {
  if (!e || !weights || !out) return fail(OMC_ERR_ARG, "null argument");
  const int nb = e->batch_tallies;
  if (nb < 1) return fail(OMC_ERR_STATE, "the last run kept no batch tallies (a multi-batch wavefront run does)");
  omc_status s;
  if ((s = ensure_device(e)) != OMC_OK) return s;
  if ((s = e->weights.ensure(static_cast<size_t>(e->nreg) * sizeof(double))) != OMC_OK) return s;
  if ((s = e->batch_dot.ensure(static_cast<size_t>(nb) * sizeof(double))) != OMC_OK) return s;
  CUDA_TRY(cudaMemcpyAsync(e->weights.p, weights, static_cast<size_t>(e->nreg) * sizeof(double),
                           cudaMemcpyHostToDevice, e->stream));
  CUDA_TRY(cudaMemsetAsync(e->batch_dot.p, 0, static_cast<size_t>(nb) * sizeof(double), e->stream));
  const int bx = static_cast<int>(std::min<long long>((e->nreg + 255) / 256, std::max(1, 4 * e->nsm / nb + 1)));
  batch_dot_kernel<<<dim3(bx, nb), 256, 0, e->stream>>>(static_cast<const double *>(e->batch_tally.p), e->nreg,
                                                        static_cast<const double *>(e->weights.p),
                                                        static_cast<double *>(e->batch_dot.p));
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpyAsync(out, e->batch_dot.p, static_cast<size_t>(nb) * sizeof(double), cudaMemcpyDeviceToHost,
                           e->stream));
  CUDA_TRY(cudaStreamSynchronize(e->stream));
  if (nbatch) *nbatch = nb;
  return OMC_OK;
}

// ---------------------------------------------------------------------------
// Dose-influence matrix: beamlets in groups of resident tally slots.
// ---------------------------------------------------------------------------
extern "C" omc_status omc_engine_set_beamlets(omc_engine *e, const omc_beamlets *b) {
  if (!e || !b) return fail(OMC_ERR_ARG, "null argument");
  if (!e->f64.geom_ok) return fail(OMC_ERR_STATE, "omc_engine_set_geometry must come first");
  if (b->nbeamlets < 1 || b->nbeams < 1) return fail(OMC_ERR_ARG, "need at least one beamlet and one beam");
  if (!b->ibeam || !b->xsource || !b->ysource || !b->zsource || !b->xcorner || !b->ycorner || !b->zcorner ||
      !b->xside1 || !b->yside1 || !b->zside1 || !b->xside2 || !b->yside2 || !b->zside2)
    return fail(OMC_ERR_ARG, "null beamlet array");
  for (int i = 0; i < b->nbeamlets; i++)
    if (b->ibeam[i] < 0 || b->ibeam[i] >= b->nbeams)
      return fail(OMC_ERR_ARG, "beamlet %d: beam %d outside 0..%d", i, b->ibeam[i], b->nbeams - 1);
  omc_status s;
  if ((s = ensure_device(e)) != OMC_OK) return s;
  if ((s = upload_beamlets(e->f64, b)) != OMC_OK) return s;
  if ((s = upload_beamlets(e->f32, b)) != OMC_OK) return s;
  e->nbeamlets = b->nbeamlets;
  e->nbeams = b->nbeams;
  return OMC_OK;
}

extern "C" void omc_dij_free(omc_dij *d) {
  if (!d) return;
  std::free(d->col_ptr);
  std::free(d->row_idx);
  std::free(d->values);
  std::free(d->values_f32);
  std::free(d);
}

namespace {

void add_stats(omc_run_stats &acc, const omc_run_stats &g) {
  acc.ensrc += g.ensrc;
  acc.transport_ms += g.transport_ms;
  acc.kernel_ms += g.kernel_ms;
  acc.histories += g.histories;
  acc.steps += g.steps;
  acc.voxel_steps += g.voxel_steps;
  acc.deposits += g.deposits;
  acc.max_stack = std::max(acc.max_stack, g.max_stack);
  acc.error_flags |= g.error_flags;
  acc.warnings |= g.warnings;
}

// Dose, threshold and CSC columns of ng beamlet tallies [ng][nreg] (the
// beamlet's energy summed over its nbatch batches): dose in place in the
// reference's operation order (omc_matrad.c:839-919), entries above
// rel * the beamlet's maximum, appended to out as columns g0..g0+ng-1 (the
// host arrays grow; host_cap is their capacity).  nh: histories of each of
// the ng beamlets.
omc_status dij_group_to_csc(omc_engine *e, double *tally, int ng, long long nreg, int nx, int ny, const double *xb,
                            const double *yb, const double *zb, const double *density, const long long *nh,
                            int nbatch, double rel, bool f32v, omc_dij *out, int g0, long long &host_cap) {
  omc_status s;
  const long long nvox = nreg - 1;
  const int ntiles = static_cast<int>((nvox + kDijTile - 1) / kDijTile);
  const size_t vsize = f32v ? sizeof(float) : sizeof(double);
  if ((s = e->dij_nhist.ensure(ng * sizeof(double))) != OMC_OK) return s;
  if ((s = e->dij_max.ensure(ng * sizeof(unsigned long long))) != OMC_OK) return s;
  if ((s = e->dij_cnt.ensure(static_cast<size_t>(ng) * ntiles * sizeof(long long))) != OMC_OK) return s;
  if ((s = e->dij_off.ensure((static_cast<size_t>(ng) * ntiles + 1) * sizeof(long long))) != OMC_OK) return s;
  if ((s = e->dij_factor.ensure(static_cast<size_t>(nvox) * sizeof(double))) != OMC_OK) return s;
  std::vector<double> nhd(ng);
  std::vector<long long> tile0(ng);
  for (int i = 0; i < ng; i++) nhd[i] = 1.0 / static_cast<double>(nh[i]);  // per-slot 1/nhist (uneven counts)
  CUDA_TRY(cudaMemcpyAsync(e->dij_nhist.p, nhd.data(), ng * sizeof(double), cudaMemcpyHostToDevice, e->stream));
  CUDA_TRY(cudaMemsetAsync(e->dij_max.p, 0, ng * sizeof(unsigned long long), e->stream));
  auto *smax = static_cast<unsigned long long *>(e->dij_max.p);
  auto *cnt = static_cast<long long *>(e->dij_cnt.p);
  auto *off = static_cast<long long *>(e->dij_off.p);
  // Per-voxel factor; the group's history count goes into it when every
  // beamlet of the group has the same count (the reference's case, bit
  // for bit), else each slot applies its own 1/nhist.
  bool uniform = true;
  for (int i = 1; i < ng; i++) uniform = uniform && nh[i] == nh[0];
  double *factor = static_cast<double *>(e->dij_factor.p);
  dij_factor_kernel<<<static_cast<int>(std::min<long long>((nvox + 255) / 256, 16 * e->nsm)), 256, 0, e->stream>>>(
      nvox, nx, ny, xb, yb, zb, density, uniform ? static_cast<double>(nh[0]) : 0.0, factor);
  const int bx = static_cast<int>(std::min<long long>((nvox + 255) / 256, std::max(4, 64 * e->nsm / ng + 1)));
  dij_dose_kernel<<<dim3(bx, ng), 256, 0, e->stream>>>(tally, nreg, factor, nbatch, smax);
  dij_count_kernel<<<dim3(ntiles, ng), kDijThreads, 0, e->stream>>>(tally, nreg, ntiles, smax, rel, cnt);
  const long long ncnt = static_cast<long long>(ng) * ntiles;
  dij_scan_kernel<<<1, 1024, 0, e->stream>>>(cnt, ncnt, off);
  long long gnnz = 0;
  CUDA_TRY(cudaMemcpyAsync(&gnnz, off + ncnt, sizeof gnnz, cudaMemcpyDeviceToHost, e->stream));
  CUDA_TRY(cudaStreamSynchronize(e->stream));
  if ((s = e->dij_rows.ensure((gnnz ? gnnz : 1) * sizeof(int))) != OMC_OK) return s;
  if ((s = e->dij_vals.ensure((gnnz ? gnnz : 1) * vsize)) != OMC_OK) return s;
  dij_fill_kernel<<<dim3(ntiles, ng), kDijThreads, 0, e->stream>>>(
      tally, nreg, ntiles, smax, rel, off, uniform ? nullptr : static_cast<const double *>(e->dij_nhist.p),
      static_cast<int *>(e->dij_rows.p), f32v ? nullptr : static_cast<double *>(e->dij_vals.p),
      f32v ? static_cast<float *>(e->dij_vals.p) : nullptr);
  // Column starts: the offset of each slot's first tile.
  CUDA_TRY(cudaMemcpy2DAsync(tile0.data(), sizeof(long long), off, static_cast<size_t>(ntiles) * sizeof(long long),
                             sizeof(long long), ng, cudaMemcpyDeviceToHost, e->stream));
  if (out->nnz + gnnz > host_cap) {
    long long cap = std::max(out->nnz + gnnz, 2 * host_cap);
    int *r = static_cast<int *>(std::realloc(out->row_idx, (cap ? cap : 1) * sizeof(int)));
    if (r) out->row_idx = r;
    void *v = std::realloc(f32v ? static_cast<void *>(out->values_f32) : static_cast<void *>(out->values),
                           (cap ? cap : 1) * vsize);
    if (v) {
      if (f32v) out->values_f32 = static_cast<float *>(v);
      else out->values = static_cast<double *>(v);
    }
    if (!r || !v) return fail(OMC_ERR_NOMEM, "host allocation of %lld dij entries failed", cap);
    host_cap = cap;
  }
  if (gnnz > 0) {
    CUDA_TRY(cudaMemcpyAsync(out->row_idx + out->nnz, e->dij_rows.p, gnnz * sizeof(int), cudaMemcpyDeviceToHost,
                             e->stream));
    void *vdst = f32v ? static_cast<void *>(out->values_f32 + out->nnz) : static_cast<void *>(out->values + out->nnz);
    CUDA_TRY(cudaMemcpyAsync(vdst, e->dij_vals.p, gnnz * vsize, cudaMemcpyDeviceToHost, e->stream));
  }
  CUDA_TRY(cudaStreamSynchronize(e->stream));
  CUDA_TRY(cudaGetLastError());
  for (int i = 0; i < ng; i++) out->col_ptr[g0 + i] = out->nnz + tile0[i];
  out->nnz += gnnz;
  out->col_ptr[g0 + ng] = out->nnz;
  return OMC_OK;
}

omc_status run_dij(omc_engine *e, const omc_run_config *cfg, const omc_dij_config *dc, omc_dij *out,
                   omc_run_stats *stats) {
  if (cfg->history_stats) return fail(OMC_ERR_ARG, "history-by-history scoring is for dose runs, not dij runs");
  RunPlan rp;
  omc_status s = prepare_run(e, cfg, rp);
  if (s != OMC_OK) return s;
  const int nb = e->nbeamlets;
  const long long nreg = e->nreg, nvox = nreg - 1;
  std::vector<long long> nh(nb);
  for (int b = 0; b < nb; b++) {
    nh[b] = dc->nhist ? dc->nhist[b] : cfg->nperbatch * cfg->nbatch;
    if (nh[b] < 1) return fail(OMC_ERR_ARG, "beamlet %d: history count %lld must be >= 1", b, nh[b]);
  }
  // Slots per group: the tally budget (default: 40% of free device memory,
  // less the particle queues), at most 65535 (grid y) and nb.
  long long budget = dc->tally_bytes;
  if (budget <= 0) {
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    budget = static_cast<long long>(0.4 * static_cast<double>(fr));
  }
  long long slot_bytes = nreg * static_cast<long long>(sizeof(double));
  long long G = budget / slot_bytes;
  if (G < 1) G = 1;
  if (G > nb) G = nb;
  if (G > 65535) G = 65535;
  if ((s = e->dij_tally.ensure(static_cast<size_t>(G) * slot_bytes)) != OMC_OK) return s;
  if ((s = e->dij_first.ensure((G + 1) * sizeof(long long))) != OMC_OK) return s;
  if ((s = e->dij_beamlet.ensure(G * sizeof(int))) != OMC_OK) return s;

  out->nrows = static_cast<int>(nvox);
  out->ncols = nb;
  out->nnz = 0;
  out->col_ptr = static_cast<long long *>(std::calloc(static_cast<size_t>(nb) + 1, sizeof(long long)));
  if (!out->col_ptr) return fail(OMC_ERR_NOMEM, "host allocation failed");
  const bool f32v = dc->fp32_values != 0;
  long long host_cap = 0;
  omc_run_stats total{};
  omc_status worst = OMC_OK;
  const double *xb = static_cast<const double *>(e->f64.G.xb), *yb = e->f64.G.yb, *zb = e->f64.G.zb;
  std::vector<long long> first(G + 1);
  std::vector<int> bl(G);
  for (int g0 = 0; g0 < nb; g0 += static_cast<int>(G)) {
    const int ng = static_cast<int>(std::min<long long>(G, nb - g0));
    first[0] = 0;
    for (int i = 0; i < ng; i++) {
      first[i + 1] = first[i] + nh[g0 + i];
      bl[i] = g0 + i;
    }
    CUDA_TRY(cudaMemcpyAsync(e->dij_first.p, first.data(), (ng + 1) * sizeof(long long), cudaMemcpyHostToDevice,
                             e->stream));
    CUDA_TRY(cudaMemcpyAsync(e->dij_beamlet.p, bl.data(), ng * sizeof(int), cudaMemcpyHostToDevice, e->stream));
    CUDA_TRY(cudaMemsetAsync(e->dij_tally.p, 0, static_cast<size_t>(ng) * slot_bytes, e->stream));
    CUDA_TRY(cudaMemsetAsync(e->counters.p, 0, sizeof(Counters), e->stream));
    SlotJob job{ng, static_cast<const long long *>(e->dij_first.p), static_cast<const int *>(e->dij_beamlet.p),
                static_cast<double *>(e->dij_tally.p), first[ng], nullptr};
    omc_run_stats gs{};
    if (rp.wavefront) s = rp.fp64 ? run_wavefront(e, e->f64, cfg, rp.nlanes, &gs, &job)
                                  : run_wavefront(e, e->f32, cfg, rp.nlanes, &gs, &job);
    else s = rp.fp64 ? run_batches(e, e->f64, cfg, rp.nlanes, rp.depth, &gs, &job)
                     : run_batches(e, e->f32, cfg, rp.nlanes, rp.depth, &gs, &job);
    add_stats(total, gs);
    if (s != OMC_OK && s != OMC_ERR_STACK && s != OMC_ERR_LIMIT) return s;
    if (s != OMC_OK) worst = s;
    if ((s = dij_group_to_csc(e, static_cast<double *>(e->dij_tally.p), ng, nreg, e->f64.G.nx, e->f64.G.ny, xb, yb,
                              zb, static_cast<const double *>(e->density.p), nh.data() + g0, cfg->nbatch,
                              dc->rel_threshold, f32v, out, g0, host_cap)) != OMC_OK)
      return s;
  }
  if (stats) *stats = total;
  if (worst == OMC_ERR_STACK) return fail(OMC_ERR_STACK, "particle stack or queue overflow; histories were dropped");
  if (worst == OMC_ERR_LIMIT) return fail(OMC_ERR_LIMIT, "a device loop hit its iteration limit");
  return OMC_OK;
}

}  // namespace

extern "C" omc_status omc_engine_run_dij(omc_engine *e, const omc_run_config *cfg, const omc_dij_config *dcfg,
                                         omc_dij **out, omc_run_stats *stats) {
  if (!e || !cfg || !dcfg || !out) return fail(OMC_ERR_ARG, "null argument");
  *out = nullptr;
  if (e->nbeamlets < 1) return fail(OMC_ERR_STATE, "omc_engine_set_beamlets must come first");
  if (!(dcfg->rel_threshold >= 0.0)) return fail(OMC_ERR_ARG, "relative dose threshold must be >= 0");
  auto *d = static_cast<omc_dij *>(std::calloc(1, sizeof(omc_dij)));
  if (!d) return fail(OMC_ERR_NOMEM, "host allocation failed");
  omc_status s = run_dij(e, cfg, dcfg, d, stats);
  if (s != OMC_OK && s != OMC_ERR_STACK && s != OMC_ERR_LIMIT) {
    omc_dij_free(d);
    return s;
  }
  *out = d;
  return s;
}

// ---------------------------------------------------------------------------
// Resident dose jobs sharing the engine's tables; several jobs advance in
// one multi-job wavefront launch (a round).
// ---------------------------------------------------------------------------
struct omc_job {
  int precision;
  long long nperbatch = 0, nhist = 0, done = 0;
  int nbatch = 0;
  long long nreg = 0;
  PrecisionState<float> s32;   // geometry + source (+ beamlets) when precision is FP32
  PrecisionState<double> s64;  // ... FP64
  DevBuf tally;                // [nbatch][nreg], beamlet jobs [nbl][nreg]
  DevBuf ensrc;                // [1]
  DevBuf result;               // [2][nreg] batch sum and sum of squares (field jobs)
  // beamlet (dij) jobs
  int nbl = 0;
  int nx = 0, ny = 0;
  std::vector<long long> nh;   // histories of each beamlet
  DevBuf bl_first;             // [nbl + 1]
  DevBuf density, bounds;      // FP64 densities [nvox] and x/y/z bounds, for the dose conversion
};

namespace {

const PrecisionState<float> &job_state(const omc_job *j, float) { return j->s32; }
const PrecisionState<double> &job_state(const omc_job *j, double) { return j->s64; }

template <typename R>
JobSlot<R> job_slot(const PrecisionState<R> &S, omc_job *j) {
  JobSlot<R> js{};
  js.G = S.G;
  js.S = S.S;
  js.tally = static_cast<double *>(j->tally.p);
  js.ensrc = static_cast<double *>(j->ensrc.p);
  js.nreg = j->nreg;
  js.h0 = j->done;
  js.nperbatch = j->nperbatch;
  js.nbl = j->nbl;
  js.bl_first = static_cast<const long long *>(j->bl_first.p);
  if (j->nbl > 0) {
    js.S.beamlets = 1;
    js.S.bixel = S.bixel;
    js.S.beam_src = S.beam_src;
    js.S.ibeam = S.ibeam;
  }
  return js;
}

template <typename R>
omc_status job_round(omc_engine *e, PrecisionState<R> &S, omc_job *const *jobs, const long long *quota, int n,
                     const omc_run_config *cfg, omc_run_stats *stats) {
  const int nlanes = wavefront_blocks<R, true>(e) * kBlock;
  omc_status s;
  size_t rng_bytes = static_cast<size_t>(RNG_WORDS) * nlanes * sizeof(int);
  if (e->rng_u.n < rng_bytes) e->seeded_lanes = 0;
  if ((s = e->rng_u.ensure(rng_bytes)) != OMC_OK) return s;
  if ((s = e->rng_ijc.ensure(static_cast<size_t>(3) * nlanes * sizeof(int))) != OMC_OK) return s;
  if (!(cfg->continue_streams && e->seeded_lanes == nlanes)) {
    seed_kernel<<<(nlanes + 255) / 256, 256, 0, e->stream>>>(cfg->ixx, cfg->jxx, nlanes,
                                                            static_cast<int *>(e->rng_u.p),
                                                            static_cast<int *>(e->rng_ijc.p));
    e->seeded_lanes = nlanes;
  }
  std::vector<JobSlot<R>> slots(n);
  std::vector<long long> first(n + 1, 0);
  for (int i = 0; i < n; i++) {
    slots[i] = job_slot(job_state(jobs[i], R()), jobs[i]);
    first[i + 1] = first[i] + quota[i];
  }
  if ((s = e->multi_slots.ensure(n * sizeof(JobSlot<R>))) != OMC_OK) return s;
  if ((s = e->multi_first.ensure((n + 1) * sizeof(long long))) != OMC_OK) return s;
  CUDA_TRY(cudaMemcpyAsync(e->multi_slots.p, slots.data(), n * sizeof(JobSlot<R>), cudaMemcpyHostToDevice,
                           e->stream));
  CUDA_TRY(cudaMemcpyAsync(e->multi_first.p, first.data(), (n + 1) * sizeof(long long), cudaMemcpyHostToDevice,
                           e->stream));
  CUDA_TRY(cudaMemsetAsync(e->counters.p, 0, sizeof(Counters), e->stream));
  SlotJob job{n, static_cast<const long long *>(e->multi_first.p), nullptr, nullptr, first[n], e->multi_slots.p};
  s = run_wavefront(e, S, cfg, nlanes, stats, &job);
  if (s == OMC_OK || s == OMC_ERR_STACK || s == OMC_ERR_LIMIT)
    for (int i = 0; i < n; i++) jobs[i]->done += quota[i];
  return s;
}

}  // namespace

extern "C" size_t omc_job_device_bytes(const omc_phantom *ph, int nbatch, int precision) {
  if (!ph) return 0;
  size_t nreg = static_cast<size_t>(ph->nx) * ph->ny * ph->nz + 1;
  size_t rsize = precision == OMC_FP32 ? 4 : 8;
  return nreg * (1 + rsize) + nreg * 8 * (static_cast<size_t>(nbatch > 0 ? nbatch : 1) + 2) +
         (static_cast<size_t>(ph->nx + ph->ny + ph->nz + 3) + 2 * OMC_INVDIM) * rsize + 4096;
}

extern "C" omc_status omc_engine_job_add(omc_engine *e, const omc_phantom *ph, const omc_regions *r,
                                         const omc_source *src, long long nperbatch, int nbatch, int precision,
                                         omc_job **out) {
  if (!e || !ph || !r || !src || !out) return fail(OMC_ERR_ARG, "null argument");
  *out = nullptr;
  if (!e->f64.tables_ok) return fail(OMC_ERR_STATE, "omc_engine_set_tables must come first");
  if (nbatch < 1 || nbatch > kBatchTag || nperbatch < 1)
    return fail(OMC_ERR_ARG, "need 1 <= nbatch <= %d and nperbatch >= 1", kBatchTag);
  if (precision != OMC_FP32 && precision != OMC_FP64) return fail(OMC_ERR_ARG, "unknown precision");
  int nmed = e->host_tables_dims.nmed;
  RegionData rd;
  omc_status s;
  if ((s = region_data(nmed, ph, r, rd)) != OMC_OK) return s;
  if ((s = ensure_device(e)) != OMC_OK) return s;
  std::unique_ptr<omc_job> j(new omc_job());
  j->precision = precision;
  j->nperbatch = nperbatch;
  j->nbatch = nbatch;
  j->nhist = nperbatch * nbatch;
  j->nreg = r->nreg;
  if (precision == OMC_FP32) {
    if ((s = upload_geometry(j->s32, ph, rd.med, rd.rhof, rd.ecut_m.data(), rd.pcut_m.data(), nmed)) != OMC_OK)
      return s;
    if ((s = upload_source(j->s32, src)) != OMC_OK) return s;
  } else {
    if ((s = upload_geometry(j->s64, ph, rd.med, rd.rhof, rd.ecut_m.data(), rd.pcut_m.data(), nmed)) != OMC_OK)
      return s;
    if ((s = upload_source(j->s64, src)) != OMC_OK) return s;
  }
  if ((s = j->tally.ensure(static_cast<size_t>(nbatch) * j->nreg * sizeof(double))) != OMC_OK) return s;
  if ((s = j->ensrc.ensure(sizeof(double))) != OMC_OK) return s;
  if ((s = j->result.ensure(2 * static_cast<size_t>(j->nreg) * sizeof(double))) != OMC_OK) return s;
  CUDA_TRY(cudaMemset(j->tally.p, 0, static_cast<size_t>(nbatch) * j->nreg * sizeof(double)));
  CUDA_TRY(cudaMemset(j->ensrc.p, 0, sizeof(double)));
  *out = j.release();
  return OMC_OK;
}

extern "C" size_t omc_job_dij_device_bytes(const omc_phantom *ph, int nbeamlets, int precision) {
  if (!ph) return 0;
  size_t nreg = static_cast<size_t>(ph->nx) * ph->ny * ph->nz + 1;
  size_t rsize = precision == OMC_FP32 ? 4 : 8;
  return nreg * (1 + rsize) + nreg * 8 * (static_cast<size_t>(nbeamlets > 0 ? nbeamlets : 1) + 1) +
         (static_cast<size_t>(ph->nx + ph->ny + ph->nz + 3) + 2 * OMC_INVDIM) * (rsize + 8) +
         static_cast<size_t>(nbeamlets > 0 ? nbeamlets : 1) * (9 * rsize + 12) + 4096;
}

extern "C" omc_status omc_engine_job_add_dij(omc_engine *e, const omc_phantom *ph, const omc_regions *r,
                                             const omc_source *src, const omc_beamlets *bl, const long long *nhist,
                                             long long nperbatch, int nbatch, int precision, omc_job **out) {
  if (!e || !ph || !r || !src || !bl || !out) return fail(OMC_ERR_ARG, "null argument");
  *out = nullptr;
  if (!e->f64.tables_ok) return fail(OMC_ERR_STATE, "omc_engine_set_tables must come first");
  if (bl->nbeamlets < 1 || bl->nbeamlets > kBatchTag || bl->nbeams < 1)
    return fail(OMC_ERR_ARG, "need 1 to %d beamlets and at least one beam", kBatchTag);
  if (nbatch < 1) return fail(OMC_ERR_ARG, "need nbatch >= 1");
  if (precision != OMC_FP32 && precision != OMC_FP64) return fail(OMC_ERR_ARG, "unknown precision");
  for (int i = 0; i < bl->nbeamlets; i++) {
    if (bl->ibeam[i] < 0 || bl->ibeam[i] >= bl->nbeams) return fail(OMC_ERR_ARG, "beamlet %d: bad beam", i);
    const long long h = nhist ? nhist[i] : nperbatch * nbatch;
    if (h < 1) return fail(OMC_ERR_ARG, "beamlet %d: history count %lld must be >= 1", i, h);
  }
  int nmed = e->host_tables_dims.nmed;
  RegionData rd;
  omc_status s;
  if ((s = region_data(nmed, ph, r, rd)) != OMC_OK) return s;
  if ((s = ensure_device(e)) != OMC_OK) return s;
  std::unique_ptr<omc_job> j(new omc_job());
  j->precision = precision;
  j->nbatch = nbatch;
  j->nbl = bl->nbeamlets;
  j->nreg = r->nreg;
  j->nx = ph->nx;
  j->ny = ph->ny;
  j->nh.resize(j->nbl);
  std::vector<long long> first(j->nbl + 1, 0);
  for (int i = 0; i < j->nbl; i++) {
    j->nh[i] = nhist ? nhist[i] : nperbatch * nbatch;
    first[i + 1] = first[i] + j->nh[i];
  }
  j->nhist = first[j->nbl];
  j->nperbatch = j->nhist;  // one "batch" range: the beamlet decides the tally
  if (precision == OMC_FP32) {
    if ((s = upload_geometry(j->s32, ph, rd.med, rd.rhof, rd.ecut_m.data(), rd.pcut_m.data(), nmed)) != OMC_OK)
      return s;
    if ((s = upload_source(j->s32, src)) != OMC_OK) return s;
    if ((s = upload_beamlets(j->s32, bl)) != OMC_OK) return s;
  } else {
    if ((s = upload_geometry(j->s64, ph, rd.med, rd.rhof, rd.ecut_m.data(), rd.pcut_m.data(), nmed)) != OMC_OK)
      return s;
    if ((s = upload_source(j->s64, src)) != OMC_OK) return s;
    if ((s = upload_beamlets(j->s64, bl)) != OMC_OK) return s;
  }
  const size_t nvox = static_cast<size_t>(j->nreg - 1);
  const size_t nb = static_cast<size_t>(ph->nx + 1) + (ph->ny + 1) + (ph->nz + 1);
  if ((s = j->tally.ensure(static_cast<size_t>(j->nbl) * j->nreg * sizeof(double))) != OMC_OK) return s;
  if ((s = j->ensrc.ensure(sizeof(double))) != OMC_OK) return s;
  if ((s = j->bl_first.ensure(first.size() * sizeof(long long))) != OMC_OK) return s;
  if ((s = j->density.ensure(nvox * sizeof(double))) != OMC_OK) return s;
  if ((s = j->bounds.ensure(nb * sizeof(double))) != OMC_OK) return s;
  std::vector<double> b(nb);
  std::copy(ph->xbounds, ph->xbounds + ph->nx + 1, b.begin());
  std::copy(ph->ybounds, ph->ybounds + ph->ny + 1, b.begin() + ph->nx + 1);
  std::copy(ph->zbounds, ph->zbounds + ph->nz + 1, b.begin() + ph->nx + 1 + ph->ny + 1);
  CUDA_TRY(cudaMemcpy(j->bl_first.p, first.data(), first.size() * sizeof(long long), cudaMemcpyHostToDevice));
  CUDA_TRY(cudaMemcpy(j->density.p, ph->density, nvox * sizeof(double), cudaMemcpyHostToDevice));
  CUDA_TRY(cudaMemcpy(j->bounds.p, b.data(), nb * sizeof(double), cudaMemcpyHostToDevice));
  CUDA_TRY(cudaMemset(j->tally.p, 0, static_cast<size_t>(j->nbl) * j->nreg * sizeof(double)));
  CUDA_TRY(cudaMemset(j->ensrc.p, 0, sizeof(double)));
  *out = j.release();
  return OMC_OK;
}

extern "C" omc_status omc_engine_job_dij(omc_engine *e, omc_job *j, double rel_threshold, int fp32_values,
                                         omc_dij **out) {
  if (!e || !j || !out) return fail(OMC_ERR_ARG, "null argument");
  *out = nullptr;
  if (j->nbl < 1) return fail(OMC_ERR_ARG, "not a beamlet job");
  if (!(rel_threshold >= 0.0)) return fail(OMC_ERR_ARG, "relative dose threshold must be >= 0");
  if (j->done < j->nhist) return fail(OMC_ERR_STATE, "job has %lld of %lld histories left", j->nhist - j->done, j->nhist);
  omc_status s;
  if ((s = ensure_device(e)) != OMC_OK) return s;
  auto *d = static_cast<omc_dij *>(std::calloc(1, sizeof(omc_dij)));
  if (!d) return fail(OMC_ERR_NOMEM, "host allocation failed");
  d->nrows = static_cast<int>(j->nreg - 1);
  d->ncols = j->nbl;
  d->col_ptr = static_cast<long long *>(std::calloc(static_cast<size_t>(j->nbl) + 1, sizeof(long long)));
  if (!d->col_ptr) {
    omc_dij_free(d);
    return fail(OMC_ERR_NOMEM, "host allocation failed");
  }
  const double *xb = static_cast<const double *>(j->bounds.p);
  const double *yb = xb + j->nx + 1, *zb = yb + j->ny + 1;
  long long host_cap = 0;
  // Tallies in groups of at most 65535 beamlets (grid y of the kernels).
  for (int g0 = 0; g0 < j->nbl; g0 += 65535) {
    const int ng = std::min(65535, j->nbl - g0);
    s = dij_group_to_csc(e, static_cast<double *>(j->tally.p) + static_cast<size_t>(g0) * j->nreg, ng, j->nreg,
                         j->nx, j->ny, xb, yb, zb, static_cast<const double *>(j->density.p), j->nh.data() + g0,
                         j->nbatch, rel_threshold, fp32_values != 0, d, g0, host_cap);
    if (s != OMC_OK) {
      omc_dij_free(d);
      return s;
    }
  }
  *out = d;
  return OMC_OK;
}

extern "C" long long omc_job_done(const omc_job *j) { return j ? j->done : 0; }
extern "C" long long omc_job_histories(const omc_job *j) { return j ? j->nhist : 0; }

extern "C" omc_status omc_engine_job_round(omc_engine *e, omc_job *const *jobs, const long long *quota, int njobs,
                                           const omc_run_config *cfg, omc_run_stats *stats) {
  if (!e || !jobs || !quota || !cfg || njobs < 1) return fail(OMC_ERR_ARG, "bad argument");
  if (!e->f64.tables_ok) return fail(OMC_ERR_STATE, "omc_engine_set_tables must come first");
  if (njobs > (1 << 19)) return fail(OMC_ERR_ARG, "too many jobs in one round");
  if (cfg->history_stats) return fail(OMC_ERR_ARG, "history-by-history scoring is for single-job runs");
  const int prec = jobs[0]->precision;
  for (int i = 0; i < njobs; i++) {
    if (!jobs[i] || jobs[i]->precision != prec) return fail(OMC_ERR_ARG, "jobs of one round share one precision");
    if (quota[i] < 0 || jobs[i]->done + quota[i] > jobs[i]->nhist)
      return fail(OMC_ERR_ARG, "job %d: quota %lld beyond its remaining histories", i, quota[i]);
  }
  omc_status s;
  if ((s = ensure_device(e)) != OMC_OK) return s;
  omc_run_stats gs{};
  s = prec == OMC_FP32 ? job_round(e, e->f32, jobs, quota, njobs, cfg, &gs)
                       : job_round(e, e->f64, jobs, quota, njobs, cfg, &gs);
  if (stats) *stats = gs;
  return s;
}

extern "C" omc_status omc_engine_job_result(omc_engine *e, omc_job *j, double *accum_endep, double *accum_endep2,
                                            double *ensrc) {
  if (!e || !j) return fail(OMC_ERR_ARG, "null argument");
  omc_status s;
  if ((s = ensure_device(e)) != OMC_OK) return s;
  double *acc = static_cast<double *>(j->result.p), *acc2 = acc + j->nreg;
  batch_accumulate_kernel<<<std::max(1, static_cast<int>(std::min<long long>(4 * e->nsm, (j->nreg + 255) / 256))), 256, 0,
                          e->stream>>>(static_cast<const double *>(j->tally.p), j->nbatch, j->nreg, acc, acc2);
  if (accum_endep)
    CUDA_TRY(cudaMemcpyAsync(accum_endep, acc, j->nreg * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
  if (accum_endep2)
    CUDA_TRY(cudaMemcpyAsync(accum_endep2, acc2, j->nreg * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
  if (ensrc) CUDA_TRY(cudaMemcpyAsync(ensrc, j->ensrc.p, sizeof(double), cudaMemcpyDeviceToHost, e->stream));
  CUDA_TRY(cudaStreamSynchronize(e->stream));
  CUDA_TRY(cudaGetLastError());
  return OMC_OK;
}

extern "C" void omc_engine_job_remove(omc_engine *e, omc_job *j) {
  if (!j) return;
  if (e) cudaSetDevice(e->device);
  j->s32.geom.clear();
  j->s32.source.clear();
  j->s64.geom.clear();
  j->s64.source.clear();
  j->tally.release();
  j->ensrc.release();
  j->result.release();
  delete j;
}

extern "C" omc_status omc_engine_trace(omc_engine *e, int iterations) {
  if (!e || iterations < 0) return fail(OMC_ERR_ARG, "bad argument");
  omc_status s;
  if ((s = ensure_device(e)) != OMC_OK) return s;
  if (iterations == 0) {
    e->trace.release();
    e->trace_cap = 0;
    return OMC_OK;
  }
  if ((s = e->trace.ensure(static_cast<size_t>(iterations) * 4 * sizeof(unsigned long long))) != OMC_OK) return s;
  e->trace_cap = iterations;
  return OMC_OK;
}

extern "C" omc_status omc_engine_trace_read(omc_engine *e, long long *out, int cap, int *n) {
  if (!e || !out || !n) return fail(OMC_ERR_ARG, "null argument");
  omc_status s;
  if ((s = ensure_device(e)) != OMC_OK) return s;
  int k = std::min(std::min(cap, e->trace_cap), e->trace_iters + 1);
  *n = k < 0 ? 0 : k;
  if (*n > 0) CUDA_TRY(cudaMemcpy(out, e->trace.p, static_cast<size_t>(*n) * 4 * sizeof(long long),
                                  cudaMemcpyDeviceToHost));
  return OMC_OK;
}

extern "C" omc_status omc_device_memory(int device, size_t *free_bytes, size_t *total_bytes) {
  if (!free_bytes || !total_bytes) return fail(OMC_ERR_ARG, "null argument");
  CUDA_TRY(cudaSetDevice(device));
  CUDA_TRY(cudaMemGetInfo(free_bytes, total_bytes));
  return OMC_OK;
}

namespace {

// Scattered FP64 atomicAdd, the access pattern of ausgab in the wavefront
// schedule: the 32 lanes of a warp hold unrelated particles, so each adds
// to its own voxel.  Indices come from a per-thread xorshift32 sequence,
// mapped onto [0, nreg) by a 32x64-bit multiply-high.
__global__ void atomic_rate_kernel(double *t, unsigned long long nreg, int per_thread, unsigned seed) {
  unsigned long long tid = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x;
  unsigned h = (static_cast<unsigned>(tid) * 0x9E3779B9u ^ seed) | 1u;
  for (int k = 0; k < per_thread; k++) {
    h ^= h << 13;
    h ^= h >> 17;
    h ^= h << 5;
    atomicAdd(t + ((static_cast<unsigned long long>(h) * nreg) >> 32), 1.0);
  }
}

}  // namespace

extern "C" omc_status omc_measure_atomic_rate(int device, long long nreg, double *per_s) {
  if (!per_s || nreg < 1 || nreg > (1ll << 32)) return fail(OMC_ERR_ARG, "need 1 <= nreg <= 2^32");
  *per_s = 0;
  CUDA_TRY(cudaSetDevice(device));
  int sms = 0;
  CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  DevBuf t;
  omc_status st = t.ensure(static_cast<size_t>(nreg) * sizeof(double));
  if (st != OMC_OK) return st;
  const int threads = 256, per = 1024, blocks = sms * 8;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 0;
  cudaError_t err = cudaMemset(t.p, 0, static_cast<size_t>(nreg) * sizeof(double));
  for (int rep = 0; rep < 4 && err == cudaSuccess; rep++) {  // first launch warms up
    cudaEventRecord(e0);
    atomic_rate_kernel<<<blocks, threads>>>(static_cast<double *>(t.p), static_cast<unsigned long long>(nreg), per,
                                            0x2545F491u + rep);
    cudaEventRecord(e1);
    err = cudaEventSynchronize(e1);
    float ms = 0;
    if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && (best == 0 || ms < best)) best = ms;
  }
  if (err == cudaSuccess) err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  t.release();
  if (err != cudaSuccess) return fail(OMC_ERR_CUDA, "atomic rate: %s", cudaGetErrorString(err));
  *per_s = static_cast<double>(blocks) * threads * per / (best * 1e-3);
  return OMC_OK;
}

extern "C" void omc_stream_seeds(int ixx, int jxx, long long k, int *ixx_k, int *jxx_k) {
  stream_seeds(ixx, jxx, k, ixx_k, jxx_k);
}

extern "C" omc_status omc_gpu_ranmar(int device, int ixx, int jxx, int nstreams, long long n, int32_t *out) {
  if (!out || nstreams < 1 || n < 0) return fail(OMC_ERR_ARG, "bad argument");
  CUDA_TRY(cudaSetDevice(device));
  DevBuf u, ijc, o;
  omc_status s;
  if ((s = u.ensure(static_cast<size_t>(RNG_WORDS) * nstreams * sizeof(int))) != OMC_OK) return s;
  if ((s = ijc.ensure(static_cast<size_t>(3) * nstreams * sizeof(int))) != OMC_OK) return s;
  if ((s = o.ensure(static_cast<size_t>(nstreams) * (n ? n : 1) * sizeof(int))) != OMC_OK) return s;
  seed_kernel<<<(nstreams + 255) / 256, 256>>>(ixx, jxx, nstreams, static_cast<int *>(u.p), static_cast<int *>(ijc.p));
  ranmar_draw_kernel<<<(nstreams + 127) / 128, 128>>>(nstreams, n, static_cast<int *>(u.p), static_cast<int *>(ijc.p),
                                                     static_cast<int *>(o.p));
  cudaError_t err = cudaDeviceSynchronize();
  if (err == cudaSuccess)
    err = cudaMemcpy(out, o.p, static_cast<size_t>(nstreams) * n * sizeof(int), cudaMemcpyDeviceToHost);
  u.release();
  ijc.release();
  o.release();
  if (err != cudaSuccess) return fail(OMC_ERR_CUDA, "ranmar: %s", cudaGetErrorString(err));
  return OMC_OK;
}

// ---------------------------------------------------------------------------
// Transport without device allocation (omc_engine_run_noalloc).  The
// per-lane transport kernel runs on scratch taken from one file-scope
// device array instead of engine buffers, and deposits into the caller's
// device tally.  Layout of the array (byte offsets, sized for FP64):
//   RANMAR words   [97][OMC_NOALLOC_MAX_LANES] int
//   RANMAR i/j/c   [3][OMC_NOALLOC_MAX_LANES] int
//   stack planes   [8][OMC_NOALLOC_MAX_DEPTH][OMC_NOALLOC_MAX_LANES] double
//   stack keys     [OMC_NOALLOC_MAX_DEPTH][OMC_NOALLOC_MAX_LANES] int
//   counters       256 bytes
// ---------------------------------------------------------------------------
#include <chrono>
#include <mutex>

static __device__ __align__(256) unsigned char g_noalloc_scratch[OMC_NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int kNoallocMaxDevices = 64;
constexpr size_t kNoallocRngBytes = static_cast<size_t>(OMC_NOALLOC_MAX_LANES) * 97 * 4;
constexpr size_t kNoallocIjcBytes = static_cast<size_t>(OMC_NOALLOC_MAX_LANES) * 3 * 4;
constexpr size_t kNoallocStackBytes = static_cast<size_t>(OMC_NOALLOC_MAX_LANES) * OMC_NOALLOC_MAX_DEPTH * 8 * 8;
constexpr size_t kNoallocKeyBytes = static_cast<size_t>(OMC_NOALLOC_MAX_LANES) * OMC_NOALLOC_MAX_DEPTH * 4;
static_assert(kNoallocRngBytes + kNoallocIjcBytes + kNoallocStackBytes + kNoallocKeyBytes + 256 ==
                  OMC_NOALLOC_SCRATCH_BYTES,
              "scratch layout and OMC_NOALLOC_SCRATCH_BYTES disagree");
static_assert(sizeof(Counters) <= 256, "counters do not fit their scratch slot");

std::mutex g_noalloc_mu;
unsigned char *g_noalloc_ptr[kNoallocMaxDevices] = {};
int g_noalloc_lanes[kNoallocMaxDevices] = {};  // lane count the streams in the array were seeded for

// Device address of the scratch array on `device`, looked up once per
// device with that device current.  The host-side symbol is only a
// stand-in and must never be passed to a kernel.
omc_status noalloc_scratch(int device, unsigned char **out) {
  if (device < 0 || device >= kNoallocMaxDevices) return fail(OMC_ERR_ARG, "device %d unsupported", device);
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[device]) {
    void *p = nullptr;
    cudaError_t err = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (err != cudaSuccess || !p)
      return fail(OMC_ERR_CUDA, "cudaGetSymbolAddress(scratch) on device %d: %s", device, cudaGetErrorString(err));
    g_noalloc_ptr[device] = static_cast<unsigned char *>(p);
  }
  *out = g_noalloc_ptr[device];
  return OMC_OK;
}

template <typename R>
omc_status run_noalloc(omc_engine *e, PrecisionState<R> &S, const omc_run_config *cfg, int nlanes, int depth,
                       double *d_endep, cudaStream_t stream, omc_run_stats *stats) {
  unsigned char *base = nullptr;
  omc_status s = noalloc_scratch(e->device, &base);
  if (s != OMC_OK) return s;
  int *rng_u = reinterpret_cast<int *>(base);
  int *rng_ijc = reinterpret_cast<int *>(base + kNoallocRngBytes);
  R *stk = reinterpret_cast<R *>(base + kNoallocRngBytes + kNoallocIjcBytes);
  int *keys = reinterpret_cast<int *>(base + kNoallocRngBytes + kNoallocIjcBytes + kNoallocStackBytes);
  Counters *dc = reinterpret_cast<Counters *>(base + kNoallocRngBytes + kNoallocIjcBytes + kNoallocStackBytes +
                                              kNoallocKeyBytes);
  auto t0 = std::chrono::steady_clock::now();
  // Everything runs on the caller's stream, behind the work the caller
  // queued there (typically the clearing of d_endep).
  {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!(cfg->continue_streams && g_noalloc_lanes[e->device] == nlanes)) {
      g_noalloc_lanes[e->device] = 0;
      seed_kernel<<<(nlanes + 255) / 256, 256, 0, stream>>>(cfg->ixx, cfg->jxx, nlanes, rng_u, rng_ijc);
      CUDA_TRY(cudaGetLastError());
      g_noalloc_lanes[e->device] = nlanes;
    }
  }
  CUDA_TRY(cudaMemsetAsync(dc, 0, sizeof(Counters), stream));  // counters must start at zero
  Params<R> P{};
  P.T = S.T;
  P.G = S.G;
  P.S = S.S;
  P.nsplit = cfg->nsplit < 1 ? 1 : cfg->nsplit;
  P.nlanes = nlanes;
  P.depth = depth;
  P.nhist = cfg->nperbatch;
  P.next = &dc->next;
  P.rng_u = rng_u;
  P.rng_ijc = rng_ijc;
  P.stk = stk;
  P.stk_key = keys;
  P.endep = d_endep;
  P.ensrc = &dc->ensrc;
  P.events = &dc->events;
  P.n_geom = &dc->n_geom;
  P.n_dep = &dc->n_dep;
  P.max_np = &dc->max_np;
  P.err = &dc->err;
  transport_kernel<R><<<(nlanes + kBlock - 1) / kBlock, kBlock, kRngSmem, stream>>>(P);
  Counters hc{};
  cudaError_t err = cudaGetLastError();
  if (err == cudaSuccess) err = cudaMemcpyAsync(&hc, dc, sizeof hc, cudaMemcpyDeviceToHost, stream);
  if (err == cudaSuccess) err = cudaStreamSynchronize(stream);
  if (err != cudaSuccess) return fail(OMC_ERR_CUDA, "no-alloc transport: %s", cudaGetErrorString(err));
  double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if (stats) {
    stats->ensrc = hc.ensrc;
    stats->transport_ms = ms;
    stats->kernel_ms = ms;
    stats->histories = cfg->nperbatch;
    stats->steps = static_cast<long long>(hc.events);
    stats->voxel_steps = static_cast<long long>(hc.n_geom);
    stats->deposits = static_cast<long long>(hc.n_dep);
    stats->max_stack = hc.max_np + 1;
    stats->error_flags = static_cast<int>(hc.err & ~ERR_TABLE);
    stats->warnings = static_cast<int>(hc.err & ERR_TABLE);
  }
  if (hc.err & ERR_STACK) return fail(OMC_ERR_STACK, "particle stack overflow (depth %d); histories were dropped", depth);
  if (hc.err & (ERR_LOOP | ERR_EVENTS)) return fail(OMC_ERR_LIMIT, "a device loop hit its iteration limit");
  return OMC_OK;
}

}  // namespace

extern "C" omc_status omc_engine_run_noalloc(omc_engine *e, const omc_run_config *cfg, double *d_endep,
                                             void *stream, omc_run_stats *stats) {
  if (!e || !cfg || !d_endep) return fail(OMC_ERR_ARG, "null argument");
  if (!e->f64.tables_ok || !e->f64.geom_ok || !e->f64.source_ok)
    return fail(OMC_ERR_STATE, "tables, geometry and source must be set before a run");
  if (cfg->nbatch != 1) return fail(OMC_ERR_ARG, "omc_engine_run_noalloc transports one batch per call (nbatch = 1)");
  if (cfg->nperbatch < 0) return fail(OMC_ERR_ARG, "nperbatch must be >= 0");
  if (cfg->precision != OMC_FP64 && cfg->precision != OMC_FP32) return fail(OMC_ERR_ARG, "unknown precision");
  int nlanes = cfg->serial ? 1 : (cfg->nlanes > 0 ? cfg->nlanes : OMC_NOALLOC_MAX_LANES);
  if (nlanes > OMC_NOALLOC_MAX_LANES)
    return fail(OMC_ERR_ARG, "nlanes %d exceeds the no-allocation maximum of %d lanes", nlanes, OMC_NOALLOC_MAX_LANES);
  // Default depth: omc_engine_run's, so that a configuration that fits
  // its stacks there fits them here.
  const int nsplit = cfg->nsplit < 1 ? 1 : cfg->nsplit;
  int depth = cfg->stack_depth > 0 ? cfg->stack_depth : kDefaultDepth + 4 * nsplit;
  if (depth > OMC_NOALLOC_MAX_DEPTH) {
    if (cfg->stack_depth > 0)
      return fail(OMC_ERR_ARG, "stack depth %d exceeds the no-allocation maximum of %d", depth, OMC_NOALLOC_MAX_DEPTH);
    return fail(OMC_ERR_ARG,
                "nsplit %d needs a stack depth of %d, above the no-allocation maximum of %d (pass stack_depth)",
                nsplit, depth, OMC_NOALLOC_MAX_DEPTH);
  }
  if (cudaSetDevice(e->device) != cudaSuccess) return fail(OMC_ERR_CUDA, "cudaSetDevice(%d) failed", e->device);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (cfg->precision == OMC_FP64) return run_noalloc(e, e->f64, cfg, nlanes, depth, d_endep, st, stats);
  return run_noalloc(e, e->f32, cfg, nlanes, depth, d_endep, st, stats);
}
