// Photon/electron transport physics of one lane (one CUDA thread).
//
// Each routine restates the reference routine named in its comment
// (edoerner/ompMC src/ompmc.c, ucodes/omc_dosxyz/omc_dosxyz.c) with the same
// random-number consumption, so a lane processes its histories exactly as a
// thread of the reference does; R is the transport precision (double or
// float), tallies are always FP64.
//
// Two schedules share this code (WF template parameter):
//  - per-lane histories (WF = false): the top particle lives in registers
//    (p, at slot np); slots 0..np-1 live in HBM in the lane's interleaved
//    stack; a lane finishes a history before it takes the next, so a lane
//    with its stream is exactly a thread of the reference;
//  - wavefront (WF = true): p is one particle taken from a photon or
//    electron queue in HBM; every particle an event leaves behind is
//    appended to the queue of its kind (warp-aggregated), and the next
//    phase of the persistent kernel picks it up.
#pragma once

#include "device.cuh"

namespace omcgpu {

#define RC(x) static_cast<R>(x)

template <typename R>
__device__ __forceinline__ R pwlf(const R *c1, const R *c0, int idx, R lv) {
  return lv * __ldg(c1 + idx) + __ldg(c0 + idx);
}

__device__ __forceinline__ V4<float> ld4(const V4<float> *p) {
  float4 v = __ldg(reinterpret_cast<const float4 *>(p));
  return V4<float>{v.x, v.y, v.z, v.w};
}
__device__ __forceinline__ V4<double> ld4(const V4<double> *p) {
  const double2 *q = reinterpret_cast<const double2 *>(p);
  double2 a = __ldg(q), b = __ldg(q + 1);
  return V4<double>{a.x, a.y, b.x, b.y};
}

// One vector load per voxel record.
__device__ __forceinline__ VoxelRec<float> load_voxel(const VoxelRec<float> *p) {
  float2 v = __ldg(reinterpret_cast<const float2 *>(p));
  return VoxelRec<float>{v.x, __float_as_int(v.y)};
}
__device__ __forceinline__ VoxelRec<double> load_voxel(const VoxelRec<double> *p) {
  double2 v = __ldg(reinterpret_cast<const double2 *>(p));
  return VoxelRec<double>{v.x, static_cast<int>(__double_as_longlong(v.y))};
}

// Separately rounded products and sums (never fused into an FMA), where a
// one-ulp difference from the reference's arithmetic matters.
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
// Correctly rounded quotient and square root, also in a fast-math build.
__device__ __forceinline__ float div_rn(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double div_rn(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float sqrt_rn(float a) { return __fsqrt_rn(a); }
__device__ __forceinline__ double sqrt_rn(double a) { return __dsqrt_rn(a); }

// Output queues of the current wavefront phase.
template <typename R>
struct EmitTargets {
  R *ph_f;            // photon queue planes [8][cap]
  int *ph_k;          // photon queue keys   [cap]
  unsigned *ph_n;     // photon queue counter
  R *el_f;
  int *el_k;
  unsigned *el_n;
  int *ph_s, *el_s;   // tally slots [cap] (beamlet jobs only)
  R *ei_f;            // electrons waiting for their discrete interaction
  int *ei_k;
  unsigned *ei_n;
  int *ei_s;
  R *pi_f;            // photons waiting for their interaction
  int *pi_k;
  unsigned *pi_n;
  int *pi_s;
  unsigned *eb_n;     // electrons within a skin depth of a boundary: the
                      // electron queue's slots counted down from the top
  R *ph_t;            // photon flights: mean free paths left (-1: a new flight)
};

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

template <typename R, bool WF, bool MULTI = false, bool HBH = false>
struct Lane {
  const Params<R> &P;
  Ranmar rng;
  int lane;
  int slot;  // tally slot of the current history / particle (beamlet jobs;
             // multi-job launches: the job slot)
  int batch; // multi-job launches: batch of the job the particle scores in
  const JobSlot<R> *js;  // multi-job launches: P.jobs + slot
  int np;    // top slot, -1 = empty (per-lane schedule)
  Particle<R> p;
  bool alive;           // wavefront: p still needs to be queued
  bool defer_interactions = false;  // wavefront: queue photon and discrete electron interactions
  bool pending_interaction = false; // wavefront: p ended its step at an interaction
  R skin = 0;           // wavefront: skin depth of p's last step (0: none, or vacuum)
  R cont_mfp = -1;      // wavefront: mean free paths left of the photon emitted (-1: a new flight)
  R taken_mfp = -1;     // wavefront: mean free paths left of the photon taken (-1: a new flight)
  int flight_cap = kNoFlightCap;  // wavefront: voxel crossings of a photon flight per event
  EmitTargets<R> out;   // wavefront: where this phase appends
  unsigned queue_cap;
  unsigned queue_hwm;   // highest slot appended
  double ensrc;
  unsigned err;
  int max_np;
  unsigned long long n_geom;  // howfar calls (voxel-stepping decisions)
  unsigned long long n_dep;   // ausgab calls (energy deposits)
  // history-by-history scoring (HBH): head block of the current particle's
  // history (-1: not tracked), particles emitted by the current take, the
  // ring entries written before this iteration began, a history this lane
  // completed and its warp is to merge (-1: none), and the warp's merge
  // table in shared memory
  int hblk = -1;
  int emitted = 0;
  unsigned long long hbh_pop_limit = 0;
  int hbh_done = -1;
  int *hbh_tir = nullptr;
  double *hbh_tx = nullptr;
  unsigned long long hbh_merged = 0, hbh_split = 0;

  __device__ Lane(const Params<R> &prm, int ln, unsigned short *slo, unsigned char *shi, int sstride)
      : P(prm), lane(ln) {
    rng.lo = slo;
    rng.hi = shi;
    rng.stride = sstride;
    np = -1;
    slot = 0;
    batch = 0;
    js = nullptr;
    ensrc = 0.0;
    err = 0;
    max_np = 0;
    n_geom = 0;
    n_dep = 0;
    alive = false;
    queue_cap = 0;
    queue_hwm = 0;
  }

  __device__ __forceinline__ R rnd() { return static_cast<R>(rng.next_int()) * RC(1.0 / 16777216.0); }

  // Geometry and source of the current particle: the launch's, or its
  // job's in a multi-job launch.
  __device__ __forceinline__ const Geometry<R> &geo() const {
    if constexpr (MULTI) return js->G;
    else return P.G;
  }
  __device__ __forceinline__ const Source<R> &src() const {
    if constexpr (MULTI) return js->S;
    else return P.S;
  }
  __device__ __forceinline__ int tag_value() const {
    if constexpr (MULTI) return slot * kBatchTag + batch;
    else return slot;
  }
  __device__ __forceinline__ void set_tag(int t) {
    if constexpr (MULTI) {
      slot = t / kBatchTag;
      batch = t - slot * kBatchTag;
      js = P.jobs + slot;
    } else {
      slot = t;
    }
  }

  // ---- stack --------------------------------------------------------------
  __device__ __forceinline__ size_t sidx(int slot) const {
    return static_cast<size_t>(slot) * P.nlanes + lane;
  }
  __device__ __forceinline__ void store(int slot, const Particle<R> &q) {
    size_t i = sidx(slot), plane = static_cast<size_t>(P.depth) * P.nlanes;
    R *s = P.stk;
    s[i] = q.e;
    s[i + plane] = q.x;
    s[i + 2 * plane] = q.y;
    s[i + 3 * plane] = q.z;
    s[i + 4 * plane] = q.u;
    s[i + 5 * plane] = q.v;
    s[i + 6 * plane] = q.w;
    s[i + 7 * plane] = q.wt;
    P.stk_key[i] = q.ir * 4 + (q.iq + 1);
  }
  __device__ __forceinline__ void load(int slot, Particle<R> &q) const {
    size_t i = sidx(slot), plane = static_cast<size_t>(P.depth) * P.nlanes;
    const R *s = P.stk;
    q.e = s[i];
    q.x = s[i + plane];
    q.y = s[i + 2 * plane];
    q.z = s[i + 3 * plane];
    q.u = s[i + 4 * plane];
    q.v = s[i + 5 * plane];
    q.w = s[i + 6 * plane];
    q.wt = s[i + 7 * plane];
    int key = P.stk_key[i];
    q.ir = key >> 2;
    q.iq = (key & 3) - 1;
  }
  // Per-lane schedule: the top (p) goes to memory and q becomes the new top
  // (false, history dropped, error flagged, if the stack is full).
  // Wavefront: q is appended to its queue and p stays current.
  __device__ __forceinline__ bool push(const Particle<R> &q) {
    if constexpr (WF) {
      emit(q);
      return true;
    } else {
      if (np + 1 >= P.depth) {
        err |= ERR_STACK;
        np = -1;
        return false;
      }
      store(np, p);
      np += 1;
      p = q;
      if (np > max_np) max_np = np;
      return true;
    }
  }
  // Per-lane schedule: remove the top; wavefront: p is consumed.
  __device__ __forceinline__ void pop() {
    if constexpr (WF) {
      alive = false;
    } else {
      np -= 1;
      if (np >= 0) load(np, p);
    }
  }

  // Wavefront append: lanes that emit together share one atomic per queue
  // (ballot + popc), so a warp writes consecutive, coalesced slots.  mfp
  // (the photon flight queue only): where the mean free paths the flight
  // has left go (cont_mfp; -1 for a new flight).
  __device__ __forceinline__ void emit_to(R *f, int *k, unsigned *n, const Particle<R> &q, int *tag,
                                          R *mfp = nullptr) {
    unsigned m = __activemask();
    int leader = __ffs(m) - 1;
    unsigned base = 0;
    if ((threadIdx.x & 31) == leader) base = atomicAdd(n, static_cast<unsigned>(__popc(m)));
    base = __shfl_sync(m, base, leader);
    const unsigned slot = base + __popc(m & lanemask_lt());
    if (slot >= queue_cap) {
      err |= ERR_QUEUE;
      return;
    }
    if (slot > queue_hwm) queue_hwm = slot;
    store_slot(f, k, slot, q, tag);
    if (mfp) __stcg(mfp + slot, cont_mfp);
  }
  __device__ __forceinline__ void store_slot(R *f, int *k, unsigned slot, const Particle<R> &q, int *tag) {
    size_t c = queue_cap;
    __stcg(f + slot, q.e);
    __stcg(f + c + slot, q.x);
    __stcg(f + 2 * c + slot, q.y);
    __stcg(f + 3 * c + slot, q.z);
    __stcg(f + 4 * c + slot, q.u);
    __stcg(f + 5 * c + slot, q.v);
    __stcg(f + 6 * c + slot, q.w);
    __stcg(f + 7 * c + slot, q.wt);
    __stcg(k + slot, q.ir * 4 + (q.iq + 1));
    if constexpr (HBH) {
      __stcg(tag + slot, hblk);
      emitted++;
    } else if (tag) {
      __stcg(tag + slot, tag_value());
    }
  }
  __device__ __forceinline__ void emit(const Particle<R> &q) {
    if (q.iq == 0) emit_photon(q);
    else emit_to(out.el_f, out.el_k, out.el_n, q, out.el_s);
  }
  // A photon to the flight queue, with the mean free paths its flight has
  // left (cont_mfp; -1 for a new flight).
  __device__ __forceinline__ void emit_photon(const Particle<R> &q) {
    emit_to(out.ph_f, out.ph_k, out.ph_n, q, out.ph_s, out.ph_t);
  }
  // An electron after its step (or the particle left on top of its take).
  // Electrons go to one of two queues by the kind of step they will take
  // next, so that a warp's chunk runs one of the two branches of the step
  // (ompmc.c:4963-5048).  Within the skin depth of a boundary (hownear <=
  // skindepth) the step is a single-scattering step: tustep is capped at
  // max(tperp, skindepth), so the test tustep > skindepth of the
  // condensed-history branch fails.  The skin depth is the last step's,
  // taken at the slightly higher energy before the step; on the 6 MV slab
  // the guess matches the branch taken in 99.7% of the steps.  Only the
  // order in which particles are processed changes.  The two share one
  // buffer: the others fill it from slot 0 up, the boundary electrons from
  // the top down, so together they have the one queue's worst-case room.
  __device__ __forceinline__ void emit_step(const Particle<R> &q) {
    if (q.iq == 0) {
      emit_photon(q);
      return;
    }
    const bool b = skin > RC(0) && hownear(q) <= skin;
    // One append site for both queues: the lanes bound for each queue
    // share one atomic.
    const unsigned act = __activemask();
    const unsigned g = __ballot_sync(act, b);
    const unsigned m = b ? g : (act & ~g);
    const int leader = __ffs(m) - 1;
    unsigned base = 0;
    if ((threadIdx.x & 31) == leader) base = atomicAdd(b ? out.eb_n : out.el_n, static_cast<unsigned>(__popc(m)));
    base = __shfl_sync(act, base, leader);
    const unsigned idx = base + __popc(m & lanemask_lt());
    if (idx >= queue_cap) {
      err |= ERR_QUEUE;
      return;
    }
    if (idx > queue_hwm) queue_hwm = idx;
    store_slot(out.el_f, out.el_k, b ? queue_cap - 1 - idx : idx, q, out.el_s);
  }
  // The current electron, which ended its step at a discrete interaction.
  __device__ __forceinline__ void emit_pending() { emit_to(out.ei_f, out.ei_k, out.ei_n, p, out.ei_s); }
  // A photon at its interaction point.  Its key holds iq + 1 = 1 for a
  // split whose scattered photon is dropped and 3 for the surviving one.
  __device__ __forceinline__ void emit_photon_interaction(const Particle<R> &q, bool survivor) {
    Particle<R> t = q;
    t.iq = survivor ? 2 : 0;
    emit_to(out.pi_f, out.pi_k, out.pi_n, t, out.pi_s);
  }
  __device__ __forceinline__ void take(const R *f, const int *k, unsigned slot, const int *tag) {
    if constexpr (HBH) {
      // The tag is the history's head block; the block holds the tally slot.
      hblk = __ldcg(tag + slot);
      emitted = 0;
      if (hblk >= 0) this->slot = __ldcg(&P.hbh.blocks[hblk].slot);
    } else if (tag) {
      set_tag(__ldcg(tag + slot));
    }
    size_t c = queue_cap;
    p.e = __ldcg(f + slot);
    p.x = __ldcg(f + c + slot);
    p.y = __ldcg(f + 2 * c + slot);
    p.z = __ldcg(f + 3 * c + slot);
    p.u = __ldcg(f + 4 * c + slot);
    p.v = __ldcg(f + 5 * c + slot);
    p.w = __ldcg(f + 6 * c + slot);
    p.wt = __ldcg(f + 7 * c + slot);
    int key = __ldcg(k + slot);
    p.ir = key >> 2;
    p.iq = (key & 3) - 1;
    alive = true;
  }

  // ---- scoring: ausgab (omc_dosxyz.c:683-694) ------------------------------
  __device__ __forceinline__ void ausgab(int ir, R wt, R edep) {
    n_dep++;
    if constexpr (MULTI)
      atomicAdd(js->tally + static_cast<size_t>(batch) * js->nreg + ir, static_cast<double>(wt * edep));
    else
      atomicAdd(P.endep + static_cast<size_t>(slot) * P.tally_stride + ir, static_cast<double>(wt * edep));
    if constexpr (HBH) hbh_append(ir, wt * edep);
  }

  // ---- history-by-history scoring (HBH) --------------------------------------
  __device__ int hbh_pop() {
    const unsigned long long i = atomicAdd(P.hbh.ctr + 1, 1ull);
    if (i >= hbh_pop_limit) {
      atomicAdd(P.hbh.ctr + 1, ~0ull);  // undo: no entry written before this iteration is left
      err |= ERR_HISTORY;
      return -1;
    }
    return __ldcg(P.hbh.ring + (i & P.hbh.ring_mask));
  }
  __device__ void hbh_push(int b) {
    const unsigned long long i = atomicAdd(P.hbh.ctr, 1ull);
    __stcg(P.hbh.ring + (i & P.hbh.ring_mask), b);
  }
  // A new history: its head block, with no particle counted yet.  The
  // lanes that start histories together take their blocks with one atomic.
  __device__ void hbh_start() {
    emitted = 0;
    const unsigned am = __activemask();
    const int leader = __ffs(am) - 1;
    const unsigned cnt = __popc(am);
    unsigned long long b = 0;
    if ((threadIdx.x & 31) == leader) {
      b = atomicAdd(P.hbh.ctr + 1, static_cast<unsigned long long>(cnt));
      if (b + cnt > hbh_pop_limit) {  // undo the ids that are not there this iteration
        const unsigned long long over = b + cnt - (b > hbh_pop_limit ? b : hbh_pop_limit);
        atomicAdd(P.hbh.ctr + 1, 0ull - over);
      }
    }
    b = __shfl_sync(am, b, leader);
    const unsigned long long i = b + __popc(am & lanemask_lt());
    if (i >= hbh_pop_limit) {
      err |= ERR_HISTORY;
      hblk = -1;
      return;
    }
    hblk = __ldcg(P.hbh.ring + (i & P.hbh.ring_mask));
    HbhBlock<R> *h = P.hbh.blocks + hblk;
    __stcg(&h->count, 0);
    __stcg(&h->next, -1);
    __stcg(&h->live, 0);
    __stcg(&h->slot, slot);
  }
  // Append (region, energy) to the history's chain; a full block gets a
  // continuation block (the first lane to install one wins, the others
  // return theirs).
  __device__ void hbh_append(int ir, R x) {
    int b = hblk;
    for (int guard = 0; b >= 0 && guard < 1024; guard++) {
      HbhBlock<R> *blk = P.hbh.blocks + b;
      const int i = atomicAdd(&blk->count, 1);
      if (i < HbhBlock<R>::kEntries) {
        __stcg(&blk->ir[i], ir);
        __stcg(&blk->x[i], x);
        return;
      }
      int nb = *static_cast<volatile int *>(&blk->next);
      if (nb < 0) {
        const int cand = hbh_pop();
        if (cand < 0) return;  // pool empty: this deposit is missing from the history sums (flagged)
        HbhBlock<R> *c = P.hbh.blocks + cand;
        __stcg(&c->count, 0);
        __stcg(&c->next, -1);
        __threadfence();
        const int old = atomicCAS(&blk->next, -1, cand);
        if (old == -1) {
          nb = cand;
        } else {
          hbh_push(cand);
          nb = old;
        }
      }
      b = nb;
    }
    err |= ERR_HISTORY;
  }
  // End of a take (consumed = 1) or of an injection (consumed = 0): the
  // history's particle count changes by emitted - consumed; at zero the
  // history is complete, and this lane hands it to its warp's merge.
  __device__ void hbh_finish(int consumed) {
    if (hblk < 0) return;
    const int delta = emitted - consumed;
    emitted = 0;
    if (delta == 0) return;
    __threadfence();  // this lane's appends before the count
    const int left = atomicAdd(&P.hbh.blocks[hblk].live, delta) + delta;
    if (left == 0) {
      __threadfence();  // every other lane's appends before the merge
      hbh_done = hblk;
    }
    hblk = -1;
  }
  // The warp merges the histories its lanes completed, one after another
  // and all 32 lanes on each: the lanes load a block's entries together and
  // sum them per region in the warp's shared-memory table, then score each
  // region's total x as x (sum) and x^2 (sum2) and return the blocks.  A
  // history over the table's regions is scored in parts (counted in split).
  // Called by all 32 lanes of the warp at the same point.
  __device__ void hbh_warp_merge() {
    const unsigned full = 0xffffffffu;
    const int lane_id = threadIdx.x & 31;
    unsigned pending = __ballot_sync(full, hbh_done >= 0);
    while (pending) {
      const int src = __ffs(pending) - 1;
      pending &= pending - 1;
      const int head = __shfl_sync(full, hbh_done, src);
      for (int k = lane_id; k < kHbhRegions; k += 32) {
        hbh_tir[k] = -1;
        hbh_tx[k] = 0.0;
      }
      __syncwarp();
      bool split = false;
      int b = head;
      int mine = -1;  // block `guard` of the chain when guard == this lane
      for (int guard = 0; b >= 0 && guard < (1 << 20); guard++) {
        const HbhBlock<R> *blk = P.hbh.blocks + b;
        const int n = min(__ldcg(&blk->count), HbhBlock<R>::kEntries);
        const int nb = __ldcg(&blk->next);
        for (int i = lane_id; i < n; i += 32) {
          const int ir = __ldcg(&blk->ir[i]);
          const double x = static_cast<double>(__ldcg(&blk->x[i]));
          unsigned h = (static_cast<unsigned>(ir) * 2654435761u) >> 25;  // 7 bits: kHbhRegions = 128
          int probe = 0;
          for (; probe < kHbhRegions; probe++) {
            const int old = atomicCAS(hbh_tir + h, -1, ir);
            if (old == -1 || old == ir) {
              atomicAdd(hbh_tx + h, x);
              break;
            }
            h = (h + 1) & (kHbhRegions - 1);
          }
          if (probe == kHbhRegions) {  // table full: this deposit scores as a part of its own
            atomicAdd(P.hbh.sum + ir, x);
            atomicAdd(P.hbh.sum2 + ir, x * x);
            split = true;
          }
        }
        if (guard < 32) {
          if (lane_id == guard) mine = b;
        } else if (lane_id == 0) {
          hbh_push(b);  // chains over 32 blocks: the rest one by one
        }
        b = nb;
      }
      // Return the chain's first 32 blocks with one atomic.
      const unsigned have = __ballot_sync(full, mine >= 0);
      if (have) {
        unsigned long long base = 0;
        if (lane_id == 0) base = atomicAdd(P.hbh.ctr, static_cast<unsigned long long>(__popc(have)));
        base = __shfl_sync(full, base, 0);
        if (mine >= 0) __stcg(P.hbh.ring + ((base + __popc(have & lanemask_lt())) & P.hbh.ring_mask), mine);
      }
      __syncwarp();
      for (int k = lane_id; k < kHbhRegions; k += 32) {
        const int ir = hbh_tir[k];
        if (ir < 0) continue;
        const double x = hbh_tx[k];
        atomicAdd(P.hbh.sum + ir, x);
        atomicAdd(P.hbh.sum2 + ir, x * x);
      }
      __syncwarp();
      split = __any_sync(full, split);
      if (lane_id == src) {
        hbh_done = -1;
        hbh_merged++;
        if (split) hbh_split++;
      }
    }
  }

  // ---- geometry: region decode, howfar, hownear (omc_dosxyz.c:187-334) ----
  __device__ __forceinline__ VoxelRec<R> voxel(int ir) const { return load_voxel(geo().vox + ir); }
  __device__ __forceinline__ int med_of(int ir) const { return voxel(ir).med; }
  __device__ __forceinline__ R rhof_of(int ir) const { return voxel(ir).rhof; }
  __device__ __forceinline__ R ecut_of(int ir) const { return __ldg(geo().ecut_m + med_of(ir) + 1); }
  __device__ __forceinline__ R pcut_of(int ir) const { return __ldg(geo().pcut_m + med_of(ir) + 1); }

  // Voxel indices of region irl >= 1: irl = 1 + ix + iy*nx + iz*nx*ny.
  __device__ __forceinline__ void decode(int irl, int &ix, int &iy, int &iz) const {
    const Geometry<R> &g = geo();
    const unsigned n = static_cast<unsigned>(irl - 1);
    const unsigned z = divide(n, g.div_nxy);
    const unsigned rem = n - z * static_cast<unsigned>(g.nxy);
    const unsigned y = divide(rem, g.div_nx);
    ix = static_cast<int>(rem - y * static_cast<unsigned>(g.nx));
    iy = static_cast<int>(y);
    iz = static_cast<int>(z);
  }

  __device__ void howfar(const Particle<R> &q, int &idisc, int &irnew, R &ustep) {
    const Geometry<R> &g = geo();
    n_geom++;
    int irl = q.ir;
    if (irl == 0) {
      idisc = 1;
      return;
    }
    int irx, iry, irz;
    decode(irl, irx, iry, irz);
    R dist;
    if (q.w > RC(0)) {
      dist = (__ldg(g.zb + irz + 1) - q.z) / q.w;
      if (dist < ustep) {
        ustep = dist;
        irnew = (irz != g.nz - 1) ? irl + g.nxy : 0;
      }
    } else if (q.w < RC(0)) {
      dist = -(q.z - __ldg(g.zb + irz)) / q.w;
      if (dist < ustep) {
        ustep = dist;
        irnew = (irz != 0) ? irl - g.nxy : 0;
      }
    }
    if (q.u > RC(0)) {
      dist = (__ldg(g.xb + irx + 1) - q.x) / q.u;
      if (dist < ustep) {
        ustep = dist;
        irnew = (irx != g.nx - 1) ? irl + 1 : 0;
      }
    } else if (q.u < RC(0)) {
      dist = -(q.x - __ldg(g.xb + irx)) / q.u;
      if (dist < ustep) {
        ustep = dist;
        irnew = (irx != 0) ? irl - 1 : 0;
      }
    }
    if (q.v > RC(0)) {
      dist = (__ldg(g.yb + iry + 1) - q.y) / q.v;
      if (dist < ustep) {
        ustep = dist;
        irnew = (iry != g.ny - 1) ? irl + g.nx : 0;
      }
    } else if (q.v < RC(0)) {
      dist = -(q.y - __ldg(g.yb + iry)) / q.v;
      if (dist < ustep) {
        ustep = dist;
        irnew = (iry != 0) ? irl - g.nx : 0;
      }
    }
  }

  __device__ R hownear(const Particle<R> &q) const {
    const Geometry<R> &g = geo();
    int irl = q.ir;
    if (irl == 0) return RC(0);
    int irx, iry, irz;
    decode(irl, irx, iry, irz);
    R t = RC(1.0E10);
    t = fmin(t, __ldg(g.xb + irx + 1) - q.x);
    t = fmin(t, q.x - __ldg(g.xb + irx));
    t = fmin(t, __ldg(g.yb + iry + 1) - q.y);
    t = fmin(t, q.y - __ldg(g.yb + iry));
    t = fmin(t, __ldg(g.zb + irz + 1) - q.z);
    t = fmin(t, q.z - __ldg(g.zb + irz));
    return t;
  }

  // ---- packed interpolation records ---------------------------------------
  __device__ __forceinline__ size_t eidx(int qel, int m, int l) const {
    return (static_cast<size_t>(qel) * P.T.nmed + m) * MXEKE + l;
  }
  __device__ __forceinline__ V4<R> esd(int qel, int m, int l) const { return ld4(P.T.el_sd + eidx(qel, m, l)); }
  __device__ __forceinline__ V4<R> ete(int qel, int m, int l) const { return ld4(P.T.el_te + eidx(qel, m, l)); }
  __device__ __forceinline__ V4<R> erg(int qel, int m, int l) const { return ld4(P.T.el_rg + eidx(qel, m, l)); }
  __device__ __forceinline__ V4<R> eq(int qel, int m, int l) const { return ld4(P.T.el_q + eidx(qel, m, l)); }

  // ---- interpolation indices, clamped to the table --------------------------
  __device__ __forceinline__ int photon_bin(int imed, R gle) {
    int l = static_cast<int>(gle * __ldg(P.T.ge1 + imed) + __ldg(P.T.ge0 + imed)) - 1;
    if (l < 0 || l >= MXGE) {
      err |= ERR_TABLE;
      l = l < 0 ? 0 : MXGE - 1;
    }
    return l;
  }
  __device__ __forceinline__ int electron_bin(int imed, R elke) {
    int l = static_cast<int>(elke * __ldg(P.T.eke1 + imed) + __ldg(P.T.eke0 + imed)) - 1;
    int top = __ldg(P.T.meke + imed) - 1;
    if (l < 0 || l > top) {
      err |= ERR_TABLE;
      l = l < 0 ? 0 : top;
    }
    return l;
  }

  // ---- rotations (ompmc.c:101-201) ------------------------------------------
  struct Uphi {
    R A, B, C, cosphi, sinphi;
  };

  __device__ void azimuth(R &cphi, R &sphi) {
    R xphi, xphi2, yphi, yphi2, rhophi2;
    int guard = 0;
    do {
      xphi = rnd();
      xphi = RC(2) * xphi - RC(1);
      xphi2 = xphi * xphi;
      yphi = rnd();
      yphi2 = yphi * yphi;
      rhophi2 = xphi2 + yphi2;
      if (++guard > kRejectCap) {
        err |= ERR_LOOP;
        break;
      }
    } while (rhophi2 > RC(1));
    rhophi2 = RC(1) / rhophi2;
    cphi = (xphi2 - yphi2) * rhophi2;
    sphi = RC(2) * xphi * yphi * rhophi2;
  }

  __device__ __forceinline__ static void rotate(Particle<R> &q, const Uphi &up, R costhe, R sinthe) {
    R sinps2 = up.A * up.A + up.B * up.B;
    if (sinps2 < RC(1.0E-20)) {
      q.u = sinthe * up.cosphi;
      q.v = sinthe * up.sinphi;
      q.w = up.C * costhe;
    } else {
      R sinpsi = sqrt(sinps2);
      R us = sinthe * up.cosphi;
      R vs = sinthe * up.sinphi;
      R sindel = up.B / sinpsi;
      R cosdel = up.A / sinpsi;
      q.u = up.C * cosdel * us - sindel * vs + up.A * costhe;
      q.v = up.C * sindel * us + cosdel * vs + up.B * costhe;
      q.w = -sinpsi * us + up.C * costhe;
    }
  }

  // uphi21: new direction of q itself, azimuth sampled here.
  __device__ void uphi21(Particle<R> &q, Uphi &up, R costhe, R sinthe) {
    azimuth(up.cosphi, up.sinphi);
    up.A = q.u;
    up.B = q.v;
    up.C = q.w;
    rotate(q, up, costhe, sinthe);
  }
  // uphi32: a second particle at the position of `from`, rotated from the
  // direction saved in up (transferProperties + rotation, ompmc.c:166-201).
  __device__ static void uphi32(Particle<R> &q, const Particle<R> &from, const Uphi &up, R costhe, R sinthe) {
    q.x = from.x;
    q.y = from.y;
    q.z = from.z;
    q.ir = from.ir;
    q.wt = from.wt;
    rotate(q, up, costhe, sinthe);
  }

#include "photon.inc"
#include "electron.inc"

  // ---- source -------------------------------------------------------------
  // Energy and charge of a new history (initHistory's first part, the same
  // in omc_dosxyz.c:970-996 and omc_matrad.c:1092-1123).
  __device__ __forceinline__ void source_energy(Particle<R> &q) {
    const Source<R> &s = src();
    q.iq = s.charge;
    R ein;
    if (s.spectrum) {
      R rnno1 = rnd();
      R rnno2 = rnd();
      int k = static_cast<int>(fmin(s.deltak * rnno1, s.deltak - RC(1)));
      ein = __ldg(s.cdfinv1 + k) + rnno2 * __ldg(s.cdfinv2 + k);
    } else {
      ein = s.energy;
    }
    q.e = (q.iq != 0) ? ein + RC(0.5109989461) : ein;
    if constexpr (MULTI) atomicAdd(js->ensrc, static_cast<double>(ein));
    else ensrc += static_cast<double>(ein);
  }

  // History h of the launch: its tally slot (beamlet jobs), then the
  // source particle.
  __device__ void init_history(long long h) {
    if (P.nslots > 0) {
      int lo = 0, hi = P.nslots - 1;
      while (lo < hi) {  // last slot whose first history is <= h
        int mid = (lo + hi + 1) >> 1;
        if (__ldg(P.slot_first + mid) <= h) lo = mid;
        else hi = mid - 1;
      }
      slot = lo;
    }
    if constexpr (MULTI) {
      js = P.jobs + slot;
      const long long hj = js->h0 + (h - __ldg(P.slot_first + slot));
      if (js->nbl > 0) {
        int lo = 0, hi = js->nbl - 1;
        while (lo < hi) {  // last beamlet whose first history is <= hj
          int mid = (lo + hi + 1) >> 1;
          if (__ldg(js->bl_first + mid) <= hj) lo = mid;
          else hi = mid - 1;
        }
        batch = lo;
        init_beamlet_history(lo);
      } else {
        batch = static_cast<int>(hj / js->nperbatch);
        init_point_history();
      }
    } else {
      if (P.S.beamlets) init_beamlet_history(__ldg(P.slot_beamlet + slot));
      else init_point_history();
    }
  }

  // initHistory(ibeamlet) (omc_matrad.c:1084-1254): a uniform point of the
  // bixel, moved back along the line to the beam's source point onto the
  // phantom surface, heading into the phantom.  The reference clamps z
  // against ybounds[0] (:1225); that is kept.  A point that lands a
  // rounding error below zbounds[0] is moved by that clamp, so the
  // arithmetic here is rounded operation by operation like the
  // reference's: no fused multiply-adds, and correctly rounded division
  // and square root.
  __device__ void init_beamlet_history(int ib) {
    const Source<R> &s = src();
    const Geometry<R> &g = geo();
    Particle<R> q;
    source_energy(q);
    R rnno1 = rnd();
    R rnno2 = rnd();
    const R *b = s.bixel + static_cast<size_t>(ib) * 9;
    R xiso = add_rn(add_rn(mul_rn(rnno1, __ldg(b + 3)), mul_rn(rnno2, __ldg(b + 6))), __ldg(b + 0));
    R yiso = add_rn(add_rn(mul_rn(rnno1, __ldg(b + 4)), mul_rn(rnno2, __ldg(b + 7))), __ldg(b + 1));
    R ziso = add_rn(add_rn(mul_rn(rnno1, __ldg(b + 5)), mul_rn(rnno2, __ldg(b + 8))), __ldg(b + 2));
    const R *src = s.beam_src + 3 * __ldg(s.ibeam + ib);
    R dx = xiso - __ldg(src + 0), dy = yiso - __ldg(src + 1), dz = ziso - __ldg(src + 2);
    R vnorm = sqrt_rn(add_rn(add_rn(mul_rn(dx, dx), mul_rn(dy, dy)), mul_rn(dz, dz)));
    R u = div_rn(-dx, vnorm), v = div_rn(-dy, vnorm), w = div_rn(-dz, vnorm);
    R ustep = RC(1.0E5), dist;
    const R x0 = __ldg(g.xb), x1 = __ldg(g.xb + g.nx);
    const R y0 = __ldg(g.yb), y1 = __ldg(g.yb + g.ny);
    const R z0 = __ldg(g.zb), z1 = __ldg(g.zb + g.nz);
    if (u > RC(0)) {
      dist = div_rn(x1 - xiso, u);
      if (dist < ustep) ustep = dist;
    }
    if (u < RC(0)) {
      dist = div_rn(-(xiso - x0), u);
      if (dist < ustep) ustep = dist;
    }
    if (v > RC(0)) {
      dist = div_rn(y1 - yiso, v);
      if (dist < ustep) ustep = dist;
    }
    if (v < RC(0)) {
      dist = div_rn(-(yiso - y0), v);
      if (dist < ustep) ustep = dist;
    }
    if (w > RC(0)) {
      dist = div_rn(z1 - ziso, w);
      if (dist < ustep) ustep = dist;
    }
    if (w < RC(0)) {
      dist = div_rn(-(ziso - z0), w);
      if (dist < ustep) ustep = dist;
    }
    R x = add_rn(xiso, mul_rn(ustep, u)), y = add_rn(yiso, mul_rn(ustep, v)), z = add_rn(ziso, mul_rn(ustep, w));
    q.u = -u;
    q.v = -v;
    q.w = -w;
    const R tiny = RC(2.0 * 2.2250738585072014e-308);  // 2*DBL_MIN
    if (x < x0) x = x0 + tiny;
    if (x > x1) x = x1 - tiny;
    if (y < y0) y = y0 + tiny;
    if (y > y1) y = y1 - tiny;
    if (z < z0) z = y0 + tiny;
    if (z > z1) z = z1 - tiny;
    q.x = x;
    q.y = y;
    q.z = z;
    int ix = 0, iy = 0, iz = 0;
    while (ix < g.nx - 1 && __ldg(g.xb + ix + 1) < x) ix++;
    while (iy < g.ny - 1 && __ldg(g.yb + iy + 1) < y) iy++;
    while (iz < g.nz - 1 && __ldg(g.zb + iz + 1) < z) iz++;
    q.ir = 1 + ix + iy * g.nx + iz * g.nxy;
    q.wt = RC(1);
    p = q;
    np = 0;
  }

  // initHistory (omc_dosxyz.c:964-1068): collimated point source.
  __device__ void init_point_history() {
    const Source<R> &s = src();
    const Geometry<R> &g = geo();
    Particle<R> q;
    source_energy(q);
    R rxyz;
    if (s.xsize == RC(0) || s.ysize == RC(0)) {
      q.x = s.xinl;
      q.y = s.yinl;
      rxyz = sqrt(s.ssd * s.ssd + q.x * q.x + q.y * q.y);
      q.w = s.ssd / rxyz;
    } else {
      R fw, rnno3;
      int guard = 0;
      do {
        rnno3 = rnd();
        q.x = rnno3 * s.xsize + s.xinl;
        rnno3 = rnd();
        q.y = rnno3 * s.ysize + s.yinl;
        rnno3 = rnd();
        rxyz = sqrt(s.ssd * s.ssd + q.x * q.x + q.y * q.y);
        q.w = s.ssd / rxyz;
        fw = q.w * q.w * q.w;
        if (++guard > kRejectCap) {
          err |= ERR_LOOP;
          break;
        }
      } while (rnno3 >= fw);
    }
    q.z = __ldg(g.zb + 0);
    q.u = q.x / rxyz;
    q.v = q.y / rxyz;
    int ix, iy;
    if (s.xsize == RC(0)) {
      ix = s.ixinl;
    } else {
      ix = s.ixinl - 1;
      while ((__ldg(g.xb + ix + 1) < q.x) && ix < g.nx - 1) ix++;
    }
    if (s.ysize == RC(0)) {
      iy = s.iyinl;
    } else {
      iy = s.iyinl - 1;
      while ((__ldg(g.yb + iy + 1) < q.y) && iy < g.ny - 1) iy++;
    }
    q.ir = 1 + ix + iy * g.nx;
    q.wt = RC(1);
    p = q;
    np = 0;
  }
};

#undef RC

}  // namespace omcgpu
